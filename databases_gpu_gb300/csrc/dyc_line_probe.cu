// dyc_line_probe.cu -- measures the random DRAM access ceiling that bounds
// a hash-table probe on this GPU (not part of libdycuckoo.so; built and run by
// `python bench.py --line-probe`).
//
// Reads random 128-byte lines of a 2 GiB buffer (far larger than L2) in the
// access shape the find kernel uses -- four lanes per line, one 256-bit load
// each, one line per four lanes per warp instruction -- plus one random
// 32-byte sector per lane for comparison, and prints one JSON line with the
// lines (or sectors) per second and the DRAM bytes they imply.
#include <cstdint>
#include <cstdio>

#include <cuda_runtime.h>

namespace {

#define CK(x)                                                                          \
    do {                                                                               \
        cudaError_t e_ = (x);                                                          \
        if (e_ != cudaSuccess) {                                                       \
            std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));              \
            return 1;                                                                  \
        }                                                                              \
    } while (0)

__device__ __forceinline__ uint32_t mix(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// one line per 4 lanes; n lanes in total (a multiple of 256), one tile each
__global__ void __launch_bounds__(256) lines(const char *__restrict__ buf, uint32_t nl,
                                             uint32_t *__restrict__ out, uint32_t salt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31, g = lane >> 2, r = lane & 3;
    const uint32_t mine = mix(i ^ salt) % nl;  // < nl
    uint32_t acc = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint32_t l = __shfl_sync(0xffffffffu, mine, q * 8 + g);
        const char *p = buf + (uint64_t)l * 128 + r * 32;
        uint32_t v[8];
        asm volatile("ld.global.nc.L1::no_allocate.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                     : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                       "=r"(v[6]), "=r"(v[7])
                     : "l"(p));
        acc += v[0] ^ v[7];
    }
    out[i] = acc;
}

// one random 32-byte sector per lane
__global__ void __launch_bounds__(256) sectors(const char *__restrict__ buf, uint32_t ns,
                                               uint32_t *__restrict__ out, uint32_t salt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const char *p = buf + (uint64_t)(mix(i ^ salt) % ns) * 32;
    uint32_t v[8];
    asm volatile("ld.global.nc.L1::no_allocate.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                   "=r"(v[6]), "=r"(v[7])
                 : "l"(p));
    out[i] = v[0] ^ v[7];
}

}  // namespace

int main() {
    const uint64_t bytes = 2ull << 30;
    const uint32_t nl = (uint32_t)(bytes / 128), ns = (uint32_t)(bytes / 32);
    const uint32_t n = 1u << 24;  // lanes per launch
    char *buf = nullptr;
    uint32_t *out = nullptr;
    CK(cudaMalloc(&buf, bytes));
    CK(cudaMemset(buf, 1, bytes));
    CK(cudaMalloc(&out, (size_t)n * 4));
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    const int reps = 20;
    lines<<<n / 256, 256>>>(buf, nl, out, 1u);
    CK(cudaEventRecord(a));
    for (int r = 0; r < reps; ++r) lines<<<n / 256, 256>>>(buf, nl, out, 7u + 977u * r);
    CK(cudaEventRecord(b));
    CK(cudaEventSynchronize(b));
    float ms_l = 0.f;
    CK(cudaEventElapsedTime(&ms_l, a, b));
    sectors<<<n / 256, 256>>>(buf, ns, out, 1u);
    CK(cudaEventRecord(a));
    for (int r = 0; r < reps; ++r) sectors<<<n / 256, 256>>>(buf, ns, out, 7u + 977u * r);
    CK(cudaEventRecord(b));
    CK(cudaEventSynchronize(b));
    float ms_s = 0.f;
    CK(cudaEventElapsedTime(&ms_s, a, b));
    CK(cudaGetLastError());
    const double lines_per_s = (double)reps * n / (ms_l / 1e3);  // one line per lane per launch
    const double sectors_per_s = (double)reps * n / (ms_s / 1e3);
    std::printf("{\"random_lines_per_s\": %.4g, \"line_bytes_per_s\": %.4g, "
                "\"random_sectors_per_s\": %.4g, \"buffer_bytes\": %llu}\n",
                lines_per_s, lines_per_s * 128.0, sectors_per_s, (unsigned long long)bytes);
    return 0;
}
