// dyc_apply.cuh -- kernels of a mixed batch (finds, inserts and erases in
// one call) with batch-order semantics: ops on the same key take effect in
// index order, a find sees the latest earlier insert/erase of its key in the
// batch (else the table as it was before the batch), and the table ends up
// as if the ops had run one by one.
//
// Steps (stream-ordered kernels; the host reads two counters in between):
//   group   : each op claims its key's cell in an open-addressing scratch
//             table and counts the cell (atomics in L2)
//   compact : each used cell gets a distinct-key id, a segment of the op
//             index array and the key itself
//   scatter : op indices land in their key's segment
//   (the table's own find kernel reads the pre-batch state of every
//    distinct key)
//   replay  : one thread per distinct key sorts its segment by op index
//             (segments are tiny: one op for a key seen once) and replays the
//             ops, writing every op's result and the key's final state;
//             keys whose state changed are listed as erases or upserts
//   (the table's erase and insert kernels apply those lists)
// Only the lists touch the table, each key at most once, so the usual
// insert/erase phases keep their guarantees.
#pragma once

#include "dyc_kernels.cuh"

namespace dyc {

// ApplyScratch (dyc_internal.h) holds the buffers of these kernels.

enum : uint8_t { kOpFind = 0, kOpInsert = 1, kOpErase = 2 };

// Keys with at most this many ops in a batch are replayed by one thread after
// an insertion sort of their op indices; longer segments (a key repeated
// many times) go through a stable radix sort and a warp-cooperative replay.
constexpr uint32_t kShortSeg = 64;

template <int KB>
__global__ void __launch_bounds__(256) k_apply_group(const __grid_constant__ ApplyScratch A,
                                                     const void *__restrict__ keys, uint64_t n) {
    using K = typename SlotT<KB>::K;
    K *ck = (K *)A.cell_key;
    const uint64_t mask = A.cap_cells - 1;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const K k = load_key<KB>(keys, i);
        if (k == 0) {
            A.op_cell[i] = 0xffffffffu;  // key 0: a miss / rejected op, no cell
            continue;
        }
        uint64_t h = mix32(fold(k) ^ (uint32_t)((uint64_t)k >> 32)) & mask;
        uint32_t cell = 0xffffffffu;
        for (uint64_t probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
            K old;
            if (KB == 4) old = (K)atomicCAS((unsigned *)&ck[h], 0u, (unsigned)k);
            else old = (K)atomicCAS((unsigned long long *)&ck[h], 0ull, (unsigned long long)k);
            if (old == 0 || old == k) {
                cell = (uint32_t)h;
                break;
            }
        }
        A.op_cell[i] = cell;
        if (cell != 0xffffffffu) atomicAdd(&A.cell_cnt[cell], 1u);
    }
}

// Block-wide allocation from a shared counter: thread gets base + the sum of
// x over the threads before it in the block; one atomic per block (the same
// address taken once per warp serialised these kernels). Every thread of the
// block must call it at the same point.
__device__ __forceinline__ uint32_t block_alloc(unsigned long long *ctr, uint32_t x) {
    __shared__ uint32_t wsum[32];
    __shared__ unsigned long long bbase;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    if (w == 0) {
        const uint32_t v = lane < nw ? wsum[lane] : 0u;
        uint32_t vi = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, vi, o);
            if (lane >= o) vi += y;
        }
        if (lane < nw) wsum[lane] = vi - v;
        if (lane == 31) bbase = vi ? atomicAdd(ctr, (unsigned long long)vi) : 0ull;
    }
    __syncthreads();
    const uint32_t r = (uint32_t)bbase + wsum[w] + incl - x;
    __syncthreads();  // wsum / bbase are reused by the next call
    return r;
}

// The loop steps whole blocks (cap_cells is a multiple of 256), so every
// thread reaches each block_alloc.
template <int KB>
__global__ void __launch_bounds__(256) k_apply_compact(const __grid_constant__ ApplyScratch A) {
    using K = typename SlotT<KB>::K;
    const K *ck = (const K *)A.cell_key;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < A.cap_cells; c += stride) {
        const uint32_t cnt = A.cell_cnt[c];
        const uint32_t d = block_alloc(&A.ctr[0], cnt ? 1u : 0u);
        const uint32_t off = block_alloc(&A.ctr[1], cnt);
        if (!cnt) continue;
        A.cell_did[c] = d;
        ((K *)A.dkey)[d] = ck[c];
        A.dcnt[d] = cnt;
        A.doff[d] = off;
        A.dfill[d] = 0u;
    }
}

template <int KB>
__global__ void __launch_bounds__(256) k_apply_scatter(const __grid_constant__ ApplyScratch A,
                                                       uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t cell = A.op_cell[i];
        if (cell == 0xffffffffu) continue;
        const uint32_t d = A.cell_did[cell];
        const uint32_t pos = A.doff[d] + atomicAdd(&A.dfill[d], 1u);
        A.seg[pos] = (uint32_t)i;
    }
}

// Replay. Results: vals_out[i] (value found / previous value / removed
// value, 0 when absent) and bit i of bits_out (found / key was present /
// removed). Ops on key 0 miss and change nothing.
template <int KB>
__global__ void __launch_bounds__(256) k_apply_replay(const __grid_constant__ ApplyScratch A,
                                                      const uint8_t *__restrict__ ops,
                                                      const void *__restrict__ keys,
                                                      const void *__restrict__ vals, uint32_t vb,
                                                      void *__restrict__ vals_out,
                                                      uint32_t *__restrict__ bits_out, uint64_t n,
                                                      uint64_t nd) {
    using K = typename SlotT<KB>::K;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    // key-0 ops (no cell): miss, output 0
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        if (A.op_cell[i] == 0xffffffffu && vals_out) store_val(vals_out, vb, i, 0ull);
    // whole blocks step through the distinct keys so every thread reaches
    // the block_alloc calls
    for (uint64_t d0 = (uint64_t)blockIdx.x * blockDim.x; d0 < nd; d0 += stride) {
        const uint64_t d = d0 + threadIdx.x;
        bool up = false, er = false, lg = false;
        K k = 0;
        uint64_t value = 0ull;
        if (d < nd) {
            const uint32_t cnt = A.dcnt[d], off = A.doff[d];
            if (cnt > kShortSeg) {
                lg = true;  // replayed by a warp after a stable sort
            } else {
                uint32_t *s = A.seg + off;
                // insertion sort of the segment by op index (segments are short)
                for (uint32_t a = 1; a < cnt; ++a) {
                    const uint32_t x = s[a];
                    uint32_t b = a;
                    while (b > 0 && s[b - 1] > x) {
                        s[b] = s[b - 1];
                        --b;
                    }
                    s[b] = x;
                }
                k = ((const K *)A.dkey)[d];
                const bool pre_present = (A.pre_hit[d >> 5] >> (d & 31)) & 1u;
                const uint64_t pre_value = load_val(A.pre_val, vb, d);
                bool present = pre_present;
                value = pre_value;
                for (uint32_t a = 0; a < cnt; ++a) {
                    const uint32_t i = s[a];
                    const uint8_t op = ops[i];
                    // every op reports the state just before it
                    const bool bit = present;
                    const uint64_t out = present ? value : 0ull;
                    if (op == kOpInsert) {
                        present = true;
                        value = load_val(vals, vb, i);
                    } else if (op == kOpErase) {
                        present = false;
                        value = 0ull;
                    }
                    if (vals_out) store_val(vals_out, vb, i, out);
                    if (bit && bits_out) atomicOr(&bits_out[i >> 5], 1u << (i & 31));
                }
                up = present && (!pre_present || value != pre_value);
                er = !present && pre_present;
            }
        }
        const uint32_t u = block_alloc(&A.ctr[2], up ? 1u : 0u);
        const uint32_t e = block_alloc(&A.ctr[3], er ? 1u : 0u);
        const uint32_t l = block_alloc(&A.ctr[4], lg ? 1u : 0u);
        if (up) {
            ((K *)A.up_key)[u] = k;
            if (vb == 4) ((uint32_t *)A.up_val)[u] = (uint32_t)value;
            else ((unsigned long long *)A.up_val)[u] = value;
        } else if (er) {
            ((K *)A.er_key)[e] = k;
        } else if (lg) {
            A.large[l] = (uint32_t)d;
        }
    }
}


// ---------------------------------------------------------------------------
// Long segments. A stable LSD radix sort of (distinct id, op index) pairs by
// distinct id -- the input is in op-index order, so stability keeps every
// segment in op-index order -- and one warp per long segment replays it 32
// ops at a time: the latest mutation before each op inside the chunk comes
// from a ballot, the state before the chunk is carried along.
// ---------------------------------------------------------------------------

template <int KB>
__global__ void __launch_bounds__(256) k_apply_sort_init(const __grid_constant__ ApplyScratch A,
                                                         uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t cell = A.op_cell[i];
        A.sort_key[i] = cell == 0xffffffffu ? 0xffffffffu : A.cell_did[cell];
        A.sort_val[i] = (uint32_t)i;
    }
}

template <int KB>
__global__ void __launch_bounds__(256) k_radix_hist(const uint32_t *__restrict__ key, uint64_t n,
                                                    int shift, uint32_t *__restrict__ hist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0u;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * kSortTile;
    for (int j = 0; j < kSortTile / 256; ++j) {
        const uint64_t i = base + (uint64_t)j * 256 + threadIdx.x;
        if (i < n) atomicAdd(&h[(key[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(uint64_t)threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// exclusive scan of m counts in place, one block of 1024 threads
template <int KB>
__global__ void __launch_bounds__(1024) k_scan_exclusive(uint32_t *__restrict__ v, uint64_t m) {
    __shared__ uint32_t part[1024];
    const uint64_t per = (m + 1023) / 1024;
    const uint64_t lo = per * threadIdx.x, hi = lo + per < m ? lo + per : m;
    uint32_t sum = 0u;
    for (uint64_t i = lo; i < hi; ++i) sum += v[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const uint32_t x = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += x;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - sum;  // exclusive prefix of this thread's range
    for (uint64_t i = lo; i < hi; ++i) {
        const uint32_t c = v[i];
        v[i] = run;
        run += c;
    }
}

// stable scatter: rounds of 256 elements in order; ranks among equal digits
// come from match_any within a warp and per-warp digit counts across warps
template <int KB>
__global__ void __launch_bounds__(256) k_radix_scatter(const uint32_t *__restrict__ key,
                                                       const uint32_t *__restrict__ val, uint64_t n,
                                                       int shift, const uint32_t *__restrict__ hist,
                                                       uint32_t *__restrict__ okey,
                                                       uint32_t *__restrict__ oval) {
    __shared__ uint32_t run[256];
    __shared__ uint32_t wcnt[8][256];
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    run[tid] = hist[(uint64_t)tid * gridDim.x + blockIdx.x];
    const uint64_t base = (uint64_t)blockIdx.x * kSortTile;
    for (int j = 0; j < kSortTile / 256; ++j) {
        for (int q = 0; q < 8; ++q) wcnt[q][tid] = 0u;
        __syncthreads();
        const uint64_t i = base + (uint64_t)j * 256 + tid;
        const bool valid = i < n;
        const uint32_t k = valid ? key[i] : 0u;
        const uint32_t dg = valid ? (k >> shift) & 255u : 256u + (uint32_t)lane;  // invalid: unique
        const unsigned peers = __match_any_sync(kFull, dg);
        const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0) wcnt[w][dg] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t before = 0u;
            for (int q = 0; q < w; ++q) before += wcnt[q][dg];
            const uint32_t pos = run[dg] + before + rank;
            okey[pos] = k;
            oval[pos] = val[i];
        }
        __syncthreads();
        uint32_t tot = 0u;
        for (int q = 0; q < 8; ++q) tot += wcnt[q][tid];
        run[tid] += tot;
        __syncthreads();
    }
}

template <int KB>
__global__ void __launch_bounds__(256) k_apply_seg_start(const __grid_constant__ ApplyScratch A,
                                                         const uint32_t *__restrict__ skey,
                                                         uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride) {
        const uint32_t d = skey[p];
        if (d != 0xffffffffu && (p == 0 || skey[p - 1] != d)) A.seg_start[d] = (uint32_t)p;
    }
}

template <int KB>
__global__ void __launch_bounds__(256) k_apply_replay_long(const __grid_constant__ ApplyScratch A,
                                                           const uint32_t *__restrict__ sval,
                                                           const uint8_t *__restrict__ ops,
                                                           const void *__restrict__ vals,
                                                           uint32_t vb, void *__restrict__ vals_out,
                                                           uint32_t *__restrict__ bits_out,
                                                           uint64_t nlarge) {
    using K = typename SlotT<KB>::K;
    const int lane = threadIdx.x & 31;
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t x = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; x < nlarge; x += warps) {
        const uint32_t d = A.large[x];
        const uint32_t start = A.seg_start[d], cnt = A.dcnt[d];
        const bool pre_present = (A.pre_hit[d >> 5] >> (d & 31)) & 1u;
        const uint64_t pre_value = load_val(A.pre_val, vb, d);
        bool present = pre_present;
        uint64_t value = pre_value;
        for (uint32_t c0 = 0; c0 < cnt; c0 += 32) {
            const bool v = c0 + lane < cnt;
            const uint32_t i = v ? sval[start + c0 + lane] : 0u;
            const uint8_t op = v ? ops[i] : kOpFind;
            const bool mut = v && (op == kOpInsert || op == kOpErase);  // other codes read
            const uint64_t myval = (v && op == kOpInsert) ? load_val(vals, vb, i) : 0ull;
            const unsigned mm = __ballot_sync(kFull, mut);
            const unsigned ins = __ballot_sync(kFull, v && op == kOpInsert);
            // latest mutation strictly before this lane within the chunk
            const unsigned before = mm & ((1u << lane) - 1u);
            const int src = before ? 31 - __clz(before) : -1;
            const uint64_t srcval = shfl64(myval, src < 0 ? lane : src);
            bool st_present = present;
            uint64_t st_value = value;
            if (src >= 0) {
                st_present = (ins >> src) & 1u;
                st_value = st_present ? srcval : 0ull;
            }
            if (v) {
                if (vals_out) store_val(vals_out, vb, i, st_present ? st_value : 0ull);
                if (st_present && bits_out) atomicOr(&bits_out[i >> 5], 1u << (i & 31));
            }
            // state after the chunk
            if (mm) {
                const int last = 31 - __clz(mm);
                present = (ins >> last) & 1u;
                const uint64_t lv = shfl64(myval, last);
                value = present ? lv : 0ull;
            }
        }
        if (lane == 0) {
            const K k = ((const K *)A.dkey)[d];
            if (present && (!pre_present || value != pre_value)) {
                const uint32_t u = (uint32_t)atomicAdd(&A.ctr[2], 1ull);
                ((K *)A.up_key)[u] = k;
                if (vb == 4) ((uint32_t *)A.up_val)[u] = (uint32_t)value;
                else ((unsigned long long *)A.up_val)[u] = value;
            } else if (!present && pre_present) {
                const uint32_t e = (uint32_t)atomicAdd(&A.ctr[3], 1ull);
                ((K *)A.er_key)[e] = k;
            }
        }
    }
}

}  // namespace dyc
