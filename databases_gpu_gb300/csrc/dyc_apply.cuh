// dyc_apply.cuh -- kernels of a mixed batch (finds, inserts and erases in
// one call) with batch-order semantics: ops on the same key take effect in
// index order, a find sees the latest earlier insert/erase of its key in the
// batch (else the table as it was before the batch), and the table ends up
// as if the ops had run one by one.
//
// Steps (stream-ordered kernels):
//   group   : each op claims its key's cell in an open-addressing scratch
//             table and counts the cell (atomics in L2); for a batch over
//             many tables every table has its own region of cells
//   compact : each used cell gets a distinct-key id, a segment of the op
//             index array and the key itself
//   scatter : op indices land in their key's segment (in no order)
//   (the table's own find kernel reads the pre-batch state of every
//    distinct key)
//   replay  : one thread per distinct key sorts a short segment (at most
//             kShortSeg ops) by op index and replays it, writing every op's
//             result and the key's final state; keys whose state changed are
//             listed as erases or upserts. Mid segments (up to kMidSeg ops)
//             are sorted in shared memory by one block and replayed by a
//             warp; giant ones go through a stable radix sort of the batch.
//   (the table's erase and insert kernels apply the lists)
// Only the lists touch the table, each key at most once, so the usual
// insert/erase phases keep their guarantees. Counts the kernels need are read
// from ApplyScratch::ctr on the device, so the sequence has no host reads.
#pragma once

#include "dyc_kernels.cuh"

namespace dyc {

enum : uint8_t { kOpFind = 0, kOpInsert = 1, kOpErase = 2 };

constexpr uint32_t kShortSeg = 64;   // segments replayed by one thread
constexpr uint32_t kMidSeg = 4096;   // segments sorted in shared memory by one block
constexpr uint32_t kNoCell = 0xffffffffu;

__device__ __forceinline__ uint64_t cell_hash(uint64_t k) {
    return mix32(fold(k) ^ (uint32_t)(k >> 32));
}

template <int KB>
__device__ __forceinline__ uint32_t claim_cell(typename SlotT<KB>::K *ck, uint64_t base,
                                               uint64_t mask, typename SlotT<KB>::K k) {
    using K = typename SlotT<KB>::K;
    uint64_t h = cell_hash((uint64_t)k) & mask;
    for (uint64_t probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
        K old;
        if (KB == 4) old = (K)atomicCAS((unsigned *)&ck[base + h], 0u, (unsigned)k);
        else old = (K)atomicCAS((unsigned long long *)&ck[base + h], 0ull, (unsigned long long)k);
        if (old == 0 || old == k) return (uint32_t)(base + h);
    }
    return kNoCell;  // unreachable: a region has at least twice as many cells as ops
}

template <int KB>
__global__ void __launch_bounds__(256) k_apply_group(const __grid_constant__ ApplyScratch A,
                                                     const void *__restrict__ keys, uint64_t n) {
    using K = typename SlotT<KB>::K;
    K *ck = (K *)A.cell_key;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const K k = load_key<KB>(keys, i);
        const uint32_t cell = k == 0 ? kNoCell : claim_cell<KB>(ck, 0, A.cap_cells - 1, k);
        A.op_cell[i] = cell;  // key 0: a miss / rejected op, no cell
        if (cell != kNoCell) atomicAdd(&A.cell_cnt[cell], 1u);
    }
}

// Many tables: ops of table t are [off[t], off[t+1]); its cells are
// [tcell_off[t], tcell_off[t+1]), a power of two at least twice its ops.
__device__ __forceinline__ uint32_t table_of(const uint32_t *__restrict__ off, uint32_t ntables,
                                             uint32_t i) {
    uint32_t lo = 0, hi = ntables;  // largest t with off[t] <= i
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <int KB>
__global__ void __launch_bounds__(256) k_set_group(const __grid_constant__ ApplyScratch A,
                                                   const uint32_t *__restrict__ off,
                                                   const void *__restrict__ keys, uint64_t n) {
    using K = typename SlotT<KB>::K;
    K *ck = (K *)A.cell_key;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const K k = load_key<KB>(keys, i);
        uint32_t cell = kNoCell;
        if (k != 0) {
            const uint32_t t = table_of(off, A.ntables, (uint32_t)i);
            const uint32_t c0 = A.tcell_off[t], c1 = A.tcell_off[t + 1];
            cell = claim_cell<KB>(ck, c0, (uint64_t)(c1 - c0) - 1, k);
            A.cell_tid[cell] = t;
        }
        A.op_cell[i] = cell;
        if (cell != kNoCell) atomicAdd(&A.cell_cnt[cell], 1u);
    }
}

// Cell regions: next_pow2(2 * ops of table t) cells each (none for a table
// without ops); exclusive scan into tcell_off, total in tcell_off[ntables].
// One block of 1024 threads. (A template only so that each key width's
// translation unit has its own copy.)
template <int KB>
__global__ void __launch_bounds__(1024) k_set_cells(const __grid_constant__ ApplyScratch A,
                                                    const uint32_t *__restrict__ off) {
    __shared__ uint32_t part[1024];
    const uint32_t m = A.ntables;
    const uint32_t per = (m + 1023) / 1024;
    const uint32_t lo = per * threadIdx.x, hi = lo + per < m ? lo + per : m;
    auto cells = [&](uint32_t t) {
        const uint32_t c = off[t + 1] - off[t];
        if (!c) return 0u;
        uint32_t p = 2;
        while (p < 2 * c) p <<= 1;
        return p;
    };
    uint32_t sum = 0u;
    for (uint32_t t = lo; t < hi; ++t) sum += cells(t);
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const uint32_t x = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0u;
        __syncthreads();
        part[threadIdx.x] += x;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - sum;
    for (uint32_t t = lo; t < hi; ++t) {
        A.tcell_off[t] = run;
        run += cells(t);
    }
    if (threadIdx.x == 1023) A.tcell_off[m] = part[1023];
}

// Zero the cells in use (tcell_off[ntables] of them) and the per-table counts.
template <int KB>
__global__ void __launch_bounds__(256) k_set_clear(const __grid_constant__ ApplyScratch A) {
    using K = typename SlotT<KB>::K;
    const uint64_t nc = A.tcell_off[A.ntables];
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += stride) {
        ((K *)A.cell_key)[c] = 0;
        A.cell_cnt[c] = 0u;
    }
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < A.ntables; t += stride)
        A.tnew[t] = 0u;
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

// Add 1 to cnt[t] for every lane with pred, one atomic per distinct t in the
// warp. All 32 lanes must call.
__device__ __forceinline__ void warp_count_by(uint32_t *cnt, uint32_t t, bool pred) {
    const unsigned peers = __match_any_sync(kFull, pred ? t : 0xffffffffu);
    const int lane = threadIdx.x & 31;
    if (pred && (__ffs(peers) - 1) == lane) atomicAdd(&cnt[t], (uint32_t)__popc(peers));
}

// Compaction of the cells in use: cap_cells for one table, tcell_off[ntables]
// for many. Whole blocks step through the cells so every thread reaches each
// block_alloc.
template <int KB>
__global__ void __launch_bounds__(256) k_apply_compact(const __grid_constant__ ApplyScratch A) {
    using K = typename SlotT<KB>::K;
    const K *ck = (const K *)A.cell_key;
    const uint64_t nc = A.tcell_off ? (uint64_t)A.tcell_off[A.ntables] : A.cap_cells;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t c0 = (uint64_t)blockIdx.x * blockDim.x; c0 < nc; c0 += stride) {
        const uint64_t c = c0 + threadIdx.x;
        const uint32_t cnt = c < nc ? A.cell_cnt[c] : 0u;
        const uint32_t d = block_alloc(&A.ctr[kCtrDistinct], cnt ? 1u : 0u);
        const uint32_t off = block_alloc(&A.ctr[kCtrPlaced], cnt);
        if (!cnt) continue;
        A.cell_did[c] = d;
        ((K *)A.dkey)[d] = ck[c];
        A.dcnt[d] = cnt;
        A.doff[d] = off;
        A.dfill[d] = 0u;
        if (A.dtid) A.dtid[d] = A.cell_tid[c];
    }
}

template <int KB>
__global__ void __launch_bounds__(256) k_apply_scatter(const __grid_constant__ ApplyScratch A,
                                                       uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t cell = A.op_cell[i];
        if (cell == kNoCell) continue;
        const uint32_t d = A.cell_did[cell];
        const uint32_t pos = A.doff[d] + atomicAdd(&A.dfill[d], 1u);
        A.seg[pos] = (uint32_t)i;
    }
}

// State after one op (an insert stores inval, an erase removes, any other
// code reads).
__device__ __forceinline__ void replay_op(uint8_t op, uint64_t inval, bool &present,
                                          uint64_t &value) {
    if (op == kOpInsert) {
        present = true;
        value = inval;
    } else if (op == kOpErase) {
        present = false;
        value = 0ull;
    }
}

// Final state of distinct key d, recorded by one thread (mid / giant paths).
template <int KB>
__device__ __forceinline__ void record_final_one(const ApplyScratch &A, uint32_t d, bool present,
                                                 uint64_t value, bool pre_present,
                                                 uint64_t pre_value, uint32_t vb) {
    using K = typename SlotT<KB>::K;
    const K k = ((const K *)A.dkey)[d];
    if (present && (!pre_present || value != pre_value)) {
        const uint32_t u = (uint32_t)atomicAdd(&A.ctr[kCtrUp], 1ull);
        ((K *)A.up_key)[u] = k;
        if (vb == 4) ((uint32_t *)A.up_val)[u] = (uint32_t)value;
        else ((unsigned long long *)A.up_val)[u] = value;
        if (A.dtid) {
            A.up_tid[u] = A.dtid[d];
            if (!pre_present) atomicAdd(&A.tnew[A.dtid[d]], 1u);
        }
    } else if (!present && pre_present) {
        const uint32_t e = (uint32_t)atomicAdd(&A.ctr[kCtrEr], 1ull);
        ((K *)A.er_key)[e] = k;
        if (A.dtid) A.er_tid[e] = A.dtid[d];
    }
}

// Replay of the segment idx[0..cnt) (op indices in increasing order) by one
// warp, 32 ops at a time: each op's state comes from the latest mutation
// before it in the chunk (a ballot), else from the state carried in.
__device__ __forceinline__ void warp_replay(const uint32_t *idx, uint32_t cnt, bool &present,
                                            uint64_t &value, const uint8_t *__restrict__ ops,
                                            const void *__restrict__ vals, uint32_t vb,
                                            void *__restrict__ vals_out,
                                            uint32_t *__restrict__ bits_out) {
    const int lane = threadIdx.x & 31;
    for (uint32_t c0 = 0; c0 < cnt; c0 += 32) {
        const bool v = c0 + lane < cnt;
        const uint32_t i = v ? idx[c0 + lane] : 0u;
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
}

// Replay. Results: vals_out[i] (value found / previous value / removed
// value, 0 when absent) and bit i of bits_out (the key was present just
// before op i). Ops on key 0 miss and change nothing.
template <int KB>
__global__ void __launch_bounds__(256) k_apply_replay(const __grid_constant__ ApplyScratch A,
                                                      const uint8_t *__restrict__ ops,
                                                      const void *__restrict__ vals, uint32_t vb,
                                                      void *__restrict__ vals_out,
                                                      uint32_t *__restrict__ bits_out, uint64_t n) {
    using K = typename SlotT<KB>::K;
    const uint64_t nd = A.ctr[kCtrDistinct];
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    // key-0 ops (no cell): miss, output 0
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        if (A.op_cell[i] == kNoCell && vals_out) store_val(vals_out, vb, i, 0ull);
    // whole blocks step through the distinct keys so every thread reaches
    // the block_alloc calls
    for (uint64_t d0 = (uint64_t)blockIdx.x * blockDim.x; d0 < nd; d0 += stride) {
        const uint64_t d = d0 + threadIdx.x;
        bool up = false, er = false, md = false, gi = false, fresh = false;
        K k = 0;
        uint64_t value = 0ull;
        uint32_t tid = 0u;
        if (d < nd) {
            const uint32_t cnt = A.dcnt[d], off = A.doff[d];
            if (cnt > kMidSeg) {
                gi = true;
            } else if (cnt > kShortSeg) {
                md = true;
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
                    if (vals_out) store_val(vals_out, vb, i, present ? value : 0ull);
                    if (present && bits_out) atomicOr(&bits_out[i >> 5], 1u << (i & 31));
                    replay_op(op, op == kOpInsert ? load_val(vals, vb, i) : 0ull, present, value);
                }
                up = present && (!pre_present || value != pre_value);
                er = !present && pre_present;
                fresh = up && !pre_present;
                if (A.dtid) tid = A.dtid[d];
            }
        }
        const uint32_t u = block_alloc(&A.ctr[kCtrUp], up ? 1u : 0u);
        const uint32_t e = block_alloc(&A.ctr[kCtrEr], er ? 1u : 0u);
        const uint32_t m = block_alloc(&A.ctr[kCtrMid], md ? 1u : 0u);
        const uint32_t g = block_alloc(&A.ctr[kCtrGiant], gi ? 1u : 0u);
        if (A.tnew) warp_count_by(A.tnew, tid, fresh);
        if (up) {
            ((K *)A.up_key)[u] = k;
            if (vb == 4) ((uint32_t *)A.up_val)[u] = (uint32_t)value;
            else ((unsigned long long *)A.up_val)[u] = value;
            if (A.up_tid) A.up_tid[u] = tid;
        } else if (er) {
            ((K *)A.er_key)[e] = k;
            if (A.er_tid) A.er_tid[e] = tid;
        } else if (md) {
            A.mid[m] = (uint32_t)d;
        } else if (gi) {
            A.giant[g] = (uint32_t)d;
        }
    }
}

// Mid segments: one block per segment sorts its op indices in shared memory
// (bitonic network over the next power of two), then warp 0 replays them.
template <int KB>
__global__ void __launch_bounds__(256) k_apply_replay_mid(const __grid_constant__ ApplyScratch A,
                                                          const uint8_t *__restrict__ ops,
                                                          const void *__restrict__ vals,
                                                          uint32_t vb, void *__restrict__ vals_out,
                                                          uint32_t *__restrict__ bits_out) {
    __shared__ uint32_t s[kMidSeg];
    const uint64_t nmid = A.ctr[kCtrMid];
    for (uint64_t x = blockIdx.x; x < nmid; x += gridDim.x) {
        const uint32_t d = A.mid[x];
        const uint32_t cnt = A.dcnt[d], off = A.doff[d];  // kShortSeg < cnt <= kMidSeg
        uint32_t P = 2u * kShortSeg;
        while (P < cnt) P <<= 1;
        for (uint32_t j = threadIdx.x; j < P; j += blockDim.x)
            s[j] = j < cnt ? A.seg[off + j] : 0xffffffffu;
        __syncthreads();
        for (uint32_t k = 2; k <= P; k <<= 1) {
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                for (uint32_t t = threadIdx.x; t < P; t += blockDim.x) {
                    const uint32_t u = t ^ j;
                    if (u > t) {
                        const uint32_t a = s[t], b = s[u];
                        if ((a > b) == ((t & k) == 0)) {
                            s[t] = b;
                            s[u] = a;
                        }
                    }
                }
                __syncthreads();
            }
        }
        if (threadIdx.x < 32) {
            const bool pre_present = (A.pre_hit[d >> 5] >> (d & 31)) & 1u;
            const uint64_t pre_value = load_val(A.pre_val, vb, d);
            bool present = pre_present;
            uint64_t value = pre_value;
            warp_replay(s, cnt, present, value, ops, vals, vb, vals_out, bits_out);
            if (threadIdx.x == 0)
                record_final_one<KB>(A, d, present, value, pre_present, pre_value, vb);
        }
        __syncthreads();  // s is reused by the next segment
    }
}

// ---------------------------------------------------------------------------
// Giant segments (more than kMidSeg ops on one key). A stable LSD radix sort
// of (distinct id, op index) pairs by distinct id -- the input is in
// op-index order, so stability keeps every segment in op-index order; ops of
// other keys sort last -- and one warp per giant segment replays it.
// ---------------------------------------------------------------------------
template <int KB>
__global__ void __launch_bounds__(256) k_apply_sort_init(const __grid_constant__ ApplyScratch A,
                                                         uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t cell = A.op_cell[i];
        uint32_t key = 0xffffffffu;
        if (cell != kNoCell) {
            const uint32_t d = A.cell_did[cell];
            if (A.dcnt[d] > kMidSeg) key = d;
        }
        A.sort_key[i] = key;
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
__global__ void __launch_bounds__(256) k_apply_replay_giant(const __grid_constant__ ApplyScratch A,
                                                            const uint32_t *__restrict__ sval,
                                                            const uint8_t *__restrict__ ops,
                                                            const void *__restrict__ vals,
                                                            uint32_t vb,
                                                            void *__restrict__ vals_out,
                                                            uint32_t *__restrict__ bits_out) {
    const uint64_t ngiant = A.ctr[kCtrGiant];
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t x = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; x < ngiant;
         x += warps) {
        const uint32_t d = A.giant[x];
        const bool pre_present = (A.pre_hit[d >> 5] >> (d & 31)) & 1u;
        const uint64_t pre_value = load_val(A.pre_val, vb, d);
        bool present = pre_present;
        uint64_t value = pre_value;
        warp_replay(sval + A.seg_start[d], A.dcnt[d], present, value, ops, vals, vb, vals_out,
                    bits_out);
        if ((threadIdx.x & 31) == 0)
            record_final_one<KB>(A, d, present, value, pre_present, pre_value, vb);
    }
}

}  // namespace dyc
