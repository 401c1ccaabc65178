/* TEST INFRASTRUCTURE ONLY: C launchers over the reference's own DyCuckoo
 * GPU kernels (pauline-ly/databases_gpu GPU/dyhash/cuckoo.cu), compiled for
 * sm_103a by oracle/build_ref.py from the reference source it stages under
 * oracle/_ref/src (git-ignored, never committed), with the warp-intrinsic
 * shim oracle/ref_shim/gpu/ref_warp_sync.h forced in.
 *
 * The tests use this library as a second oracle (differential parity of the
 * library's results against the reference's kernels on the same inputs) and
 * bench.py times its search beside the library's find. The product never
 * links it.
 *
 * The reference kernels read their table from one __constant__ descriptor
 * (`table`, cuckoo.cu:16), so one reference table is live per process, as in
 * the reference itself. Kernels are launched with the reference's own grid
 * (BLOCK_NUM_k blocks of THREAD_NUM_k threads, dy_hash.h:19-20) and its
 * 16-lane groups; these launchers only add a stream argument and drop the
 * timing printouts of the gpu_lp_* wrappers (cuckoo.cu:858-916).
 *
 * Return values are cudaError_t codes (0 = success); -1 marks a request the
 * reference kernels cannot serve safely (see refgpu_resize_down).
 */
#include "cuckoo.cu"

#include <cstring>

namespace {
cuckoo g_host;  // host copy of the descriptor uploaded to `table`
bool g_ready = false;
}  // namespace

extern "C" {

/* The reference's launch shape and bucket geometry. */
int refgpu_geometry(unsigned *blocks, unsigned *threads, unsigned *slots_per_bucket,
                    unsigned *subtables) {
    *blocks = BLOCK_NUM_k;
    *threads = THREAD_NUM_k;
    *slots_per_bucket = BUCKET_SIZE;
    *subtables = TABLE_NUM;
    return 0;
}

/* Point the kernels at TABLE_NUM subtables: subtable t is lsize[t] slots
 * (8 bytes each, key << 32 | value, 0 = empty; lsize[t] a multiple of
 * BUCKET_SIZE) at the device address subtables[t], zeroed by the caller, as
 * hashAPI::hashAPI lays them out (api.cpp:46-74). Same upload as
 * gpu_lp_set_table (cuckoo.cu:918-923). */
int refgpu_set_table(void *const *subtables, const unsigned *lsize) {
    std::memset(&g_host, 0, sizeof(g_host));
    for (int t = 0; t < TABLE_NUM; ++t) {
        if (!subtables[t] || lsize[t] < (unsigned)BUCKET_SIZE || lsize[t] % BUCKET_SIZE)
            return -1;
        g_host.table[t] = (bucket_t *)subtables[t];
        g_host.Lsize[t] = lsize[t];
    }
    g_ready = true;
    return (int)cudaMemcpyToSymbol(table, &g_host, sizeof(cuckoo));
}

/* Current subtable addresses and sizes (they change with the resizes). */
int refgpu_layout(void **subtables, unsigned *lsize) {
    if (!g_ready) return -1;
    for (int t = 0; t < TABLE_NUM; ++t) {
        subtables[t] = g_host.table[t];
        lsize[t] = g_host.Lsize[t];
    }
    return 0;
}

/* cuckoo_insert (cuckoo.cu:324-355) over n keys and values. The kernel sets
 * *d_rehash to 1 when an entry is left over at the end of a MAX_ITER-step
 * eviction chain (that entry is dropped, cuckoo.cu:422-431) and writes every
 * key's exchange count to d_iter_count[0..n). Values must be below 2^31:
 * the kernel reads them as int and makeEntry sign-extends (cuckoo.h:14). */
int refgpu_insert(const unsigned *keys, const unsigned *vals, unsigned n, int *d_rehash,
                  int *d_iter_count, void *stream) {
    if (!g_ready) return -1;
    if (n == 0) return 0;
    cuckoo_insert<<<BLOCK_NUM_k, THREAD_NUM_k, 0, (cudaStream_t)stream>>>(
        (TYPE *)keys, (TYPE *)vals, n, d_rehash, d_iter_count);
    return (int)cudaGetLastError();
}

/* cuckoo_search (cuckoo.cu:460-520): vals[i] is written only on a hit, so
 * the caller zeroes vals first (hashAPI::hash_search does, api.cpp:275). */
int refgpu_search(const unsigned *keys, unsigned *vals, unsigned n, void *stream) {
    if (!g_ready) return -1;
    if (n == 0) return 0;
    cuckoo_search<<<BLOCK_NUM_k, THREAD_NUM_k, 0, (cudaStream_t)stream>>>(
        (TYPE *)keys, (TYPE *)vals, n);
    return (int)cudaGetLastError();
}

/* cuckoo_delete (cuckoo.cu:524-587); the kernel reports nothing. */
int refgpu_delete(const unsigned *keys, unsigned n, void *stream) {
    if (!g_ready) return -1;
    if (n == 0) return 0;
    cuckoo_delete<<<BLOCK_NUM_k, THREAD_NUM_k, 0, (cudaStream_t)stream>>>(
        (TYPE *)keys, nullptr, n);
    return (int)cudaGetLastError();
}

/* GPU_cuckoo_resize_up (cuckoo.cu:731-758) of subtable t into new_table,
 * which holds 2 x Lsize[t] zeroed slots (hashAPI::resize_up allocates and
 * clears it the same way, api.cpp:130-136). Legacy default stream; returns
 * after the kernel. */
int refgpu_resize_up(int t, void *new_table) {
    if (!g_ready || t < 0 || t >= TABLE_NUM || !new_table) return -1;
    GPU_cuckoo_resize_up(t, g_host.Lsize[t], (bucket_t *)new_table, &g_host);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return (int)e;
}

/* GPU_cuckoo_resize_down (cuckoo.cu:762-788) of subtable t into new_table,
 * which holds Lsize[t] / 2 zeroed slots. The kernel merges bucket j with
 * bucket j + nb/2 and assumes an even bucket count nb: with an odd count its
 * last group reads one bucket past the old subtable (the reference only
 * prints a warning, cuckoo.cu:768-769), so an odd count is refused here. */
int refgpu_resize_down(int t, void *new_table) {
    if (!g_ready || t < 0 || t >= TABLE_NUM || !new_table) return -1;
    unsigned nb = g_host.Lsize[t] / BUCKET_SIZE;
    if (nb < 2 || (nb & 1u)) return -1;
    GPU_cuckoo_resize_down(t, g_host.Lsize[t], (bucket_t *)new_table, &g_host);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return (int)e;
}

}  // extern "C"
