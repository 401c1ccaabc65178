// dyc_apply.cuh -- kernels of a mixed batch (finds, inserts and erases in
// one call) with batch-order semantics: ops on the same key take effect in
// index order, a find sees the latest earlier insert/erase of its key in the
// batch (else the table as it was before the batch), and the table ends up
// as if the ops had run one by one.
//
// Steps (stream-ordered kernels):
//   group   : each op claims its key's cell in an open-addressing scratch
//             table, a {key, count} word updated by one atomic for a new key,
//             and gets its rank (the count before it); for a batch over many
//             tables every table has its own region of twice its ops in cells
//   compact : each used cell gets a distinct-key id (written over its count),
//             a segment of the op index array and the key itself
//   (the find of dyc_set.cuh reads the pre-batch state of every distinct key)
//   scatter : one pass in op order: a key with a single op in the batch is
//             resolved there (result, hit bit, list entry); the other ops land
//             in their key's segment at their rank
//   replay  : one thread per distinct key replays a segment of 2 to kShortSeg
//             ops after sorting it in registers; longer segments are sorted
//             and replayed by a warp (up to kWarpSeg ops) or by one block (any
//             length: shared-memory sort, merged in global memory beyond
//             kMidSeg). Every op's result is written; keys whose state changed
//             are listed as erases or upserts.
//   (the erase + upsert and eviction-walk kernels of dyc_set.cuh apply the
//    lists)
// Only the lists touch the table, each key at most once, so the usual
// insert/erase phases keep their guarantees. Counts the kernels need are read
// from ApplyScratch::ctr on the device, so the sequence has no host reads.
// Every such count, distinct-key id and segment range is checked against the
// scratch capacity before it indexes anything (values out of range are
// clamped or their item skipped and counted in ctr[kCtrBad]); a set batch's
// op count is the smaller of its device offsets' total and the count the
// host declared (ctr[kCtrHostN]), a disagreement counted in
// ctr[kCtrBadOffsets].
#pragma once

#include "dyc_kernels.cuh"

namespace dyc {

enum : uint8_t { kOpFind = 0, kOpInsert = 1, kOpErase = 2 };

constexpr uint32_t kShortSeg = 8;    // segments replayed by one thread
constexpr uint32_t kWarpSeg = 256;   // segments sorted and replayed by one warp
constexpr uint32_t kMidSeg = 4096;   // longest segment sorted in shared memory alone
// Warp segments a warp replays in a row; lane j keeps segment j's final
// state, so the upsert / erase lists take one warp-aggregated atomic per
// task. Few segments per task keep more warps busy when segments are few.
constexpr uint32_t kWarpTask = 8;
constexpr uint32_t kNoCell = 0xffffffffu;

// Cells: 4-byte keys {key (low word), count (high word)} in one 64-bit word;
// 8-byte keys {key, count, pad} in 16 bytes. After compaction the count
// field holds the distinct-key id.
template <int KB> __host__ __device__ constexpr int cell_bytes() { return KB == 4 ? 8 : 16; }

__device__ __forceinline__ uint32_t cell_hash(uint64_t k) {
    return mix32(fold(k) ^ (uint32_t)(k >> 32));
}

template <int KB>
__device__ __forceinline__ typename SlotT<KB>::K cell_key(const void *cells, uint64_t c) {
    if constexpr (KB == 4) return (uint32_t)((const unsigned long long *)cells)[c];
    else return *(const unsigned long long *)((const char *)cells + c * 16);
}
template <int KB> __device__ __forceinline__ uint32_t *cell_word(void *cells, uint64_t c) {
    if constexpr (KB == 4) return (uint32_t *)cells + 2 * c + 1;
    else return (uint32_t *)((char *)cells + c * 16 + 8);
}

__device__ __forceinline__ void note_bad(const ApplyScratch &A, int slot = kCtrBad) {
    atomicAdd(&A.ctr[slot], 1ull);
}

// Op count of a set batch: offsets[ntables], bounded by the count the host
// declared for this batch and by the scratch.
__device__ __forceinline__ uint64_t set_op_count(const ApplyScratch &A,
                                                 const uint32_t *__restrict__ off) {
    uint64_t n = off[A.ntables];
    const uint64_t h = A.ctr[kCtrHostN];
    if (n > h) n = h;
    return n < A.cap_ops ? n : A.cap_ops;
}

// A device counter of listed items, clamped to the scratch's op capacity.
__device__ __forceinline__ uint64_t ctr_count(const ApplyScratch &A, int slot) {
    const uint64_t n = A.ctr[slot];
    return n < A.cap_ops ? n : A.cap_ops;
}

// Segment [off, off + cnt) of a distinct key lies inside the op scratch.
__device__ __forceinline__ bool seg_ok(const ApplyScratch &A, uint32_t off, uint32_t cnt) {
    return (uint64_t)off + cnt <= A.cap_ops;
}

// Claim (or join) key k's cell in region [base, base + size): fastrange
// start, linear probing. One CAS (64-bit for 4-byte keys, 128-bit for
// 8-byte keys) claims a new key with count 1; a repeat adds 1 to the count.
// `rank` gets the count before this op (0 for the op that claimed the cell):
// a distinct place for the op inside its key's segment, so the scatter pass
// needs no atomics. (L2 atomic throughput bounds the grouping kernels;
// keeping several first probes of a thread in flight measured slower.)
// LOAD_FIRST suits batches whose keys repeat many times (a table set's small
// tables): the ops of a hot key read its cell and add, instead of each
// failing a CAS on it first. 4096-table round: 4.22-4.31 -> 4.17-4.20 ms.
// On one large table's batch, where keys rarely repeat, the extra read per
// probe cost more than it saved (2^26 mixed ops: 11.4 -> 10.3 G ops/s; the
// batch dedup of inserts and erases lost 13-15 % the same way).
template <int KB, bool LOAD_FIRST>
__device__ __forceinline__ uint32_t claim_cell(void *cells, uint64_t base, uint64_t size,
                                               typename SlotT<KB>::K k, uint32_t &rank) {
    uint64_t idx = ((uint64_t)cell_hash((uint64_t)k) * size) >> 32;
    for (uint64_t probe = 0; probe < size; ++probe) {
        const uint64_t c = base + idx;
        // LOAD_FIRST: the cell is read from the L2 first and an atomic is
        // used only on a free cell (CAS) or on the key's own (add). A cell's
        // key never changes within a batch, so a read that finds another key
        // is final. Otherwise every probe is a CAS.
        if constexpr (KB == 4) {
            unsigned long long *p = (unsigned long long *)cells + c;
            unsigned long long old = LOAD_FIRST ? __ldcg(p) : 0ull;
            if (old == 0ull) {
                old = atomicCAS(p, 0ull, (unsigned long long)k | (1ull << 32));
                if (old == 0ull) {
                    rank = 0u;
                    return (uint32_t)c;
                }
            }
            if ((uint32_t)old == k) {
                rank = (uint32_t)(atomicAdd(p, 1ull << 32) >> 32);
                return (uint32_t)c;
            }
        } else {
            u128 *p = (u128 *)((char *)cells + c * 16);
            unsigned long long key = LOAD_FIRST ? __ldcg(&p->lo) : 0ull;
            if (key == 0ull) {
                const u128 old =
                    SlotT<8>::cas(p, u128{0ull, 0ull}, u128{(unsigned long long)k, 1ull});
                if (old.lo == 0ull) {
                    rank = 0u;
                    return (uint32_t)c;
                }
                key = old.lo;
            }
            if (key == k) {
                rank = atomicAdd((unsigned *)&p->hi, 1u);
                return (uint32_t)c;
            }
        }
        idx = idx + 1 == size ? 0 : idx + 1;
    }
    return kNoCell;  // unreachable: a region has twice as many cells as ops
}

// One table: cells [0, 2n).
template <int KB>
__global__ void __launch_bounds__(256) k_apply_group(const __grid_constant__ ApplyScratch A,
                                                     const void *__restrict__ keys, uint64_t n) {
    using K = typename SlotT<KB>::K;
    const uint64_t size = 2 * n;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    bool repeat = false;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const K k = load_key<KB>(keys, i);
        uint32_t rank = 0u;
        // key 0: no cell
        A.op_cell[i] = k == 0 ? kNoCell : claim_cell<KB, false>(A.cells, 0, size, k, rank);
        A.op_rank[i] = rank;
        repeat |= rank != 0u;
    }
    if (repeat && A.gate != nullptr) *(volatile unsigned long long *)A.gate = 1ull;
}

// Largest t < ntables with off[t] <= i (for cell offsets: the table owning
// cell i, since a table without cells shares its offset with the next one).
__device__ __forceinline__ uint32_t table_of(const uint32_t *__restrict__ off, uint32_t ntables,
                                             uint32_t i) {
    uint32_t lo = 0, hi = ntables;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Table of op i through the coarse index tidx (the table of every
// kTidxStep-th op, filled by k_set_prep): a lower bound, then a forward scan
// over the offsets `bound` (off for ops; tcell_off for cells, with i the
// cell index and the index entry of op i / 2). Replaces a binary search of
// log2(ntables) dependent loads per lookup.
__device__ __forceinline__ uint32_t table_at(const uint32_t *__restrict__ tidx,
                                             const uint32_t *__restrict__ bound, uint32_t i,
                                             uint32_t op) {
    uint32_t t = __ldg(tidx + (op / kTidxStep));
    while (__ldg(bound + t + 1) <= i) ++t;
    return t;
}

// Many tables: ops of table t are [off[t], off[t+1]); its cells are
// [tcell_off[t], tcell_off[t+1]), twice its ops.
template <int KB>
__global__ void __launch_bounds__(256) k_set_group(const __grid_constant__ ApplyScratch A,
                                                   const uint32_t *__restrict__ off,
                                                   const void *__restrict__ keys) {
    using K = typename SlotT<KB>::K;
    const uint64_t n = set_op_count(A, off);  // the op count, read on the device
    // offsets that disagree with the host's, or are out of order, are reported
    // (every access below stays inside the scratch either way)
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid == 0 && ((uint64_t)off[A.ntables] != A.ctr[kCtrHostN] || off[0] != 0u))
        note_bad(A, kCtrBadOffsets);
    for (uint64_t t = gid; t < A.ntables; t += (uint64_t)gridDim.x * blockDim.x)
        if (off[t] > off[t + 1]) note_bad(A, kCtrBadOffsets);
    // warp-uniform loop: a warp's 32 consecutive ops mostly belong to one
    // table, found by one search when the first and last lane's tables agree
    for (uint64_t base = warp_base(); base < n; base += warp_stride()) {
        const uint64_t i = base + (threadIdx.x & 31);
        const uint64_t last = base + 31 < n ? base + 31 : n - 1;
        const uint32_t t0 = table_at(A.tidx, off, (uint32_t)base, (uint32_t)base);
        const bool one = t0 == A.ntables - 1 || __ldg(off + t0 + 1) > (uint32_t)last;
        if (i >= n) continue;
        const K k = load_key<KB>(keys, i);
        uint32_t cell = kNoCell, rank = 0u;
        if (k != 0) {
            const uint32_t t = one ? t0 : table_at(A.tidx, off, (uint32_t)i, (uint32_t)i);
            const uint32_t c0 = A.tcell_off[t], c1 = A.tcell_off[t + 1];
            if (c1 > c0) cell = claim_cell<KB, true>(A.cells, c0, c1 - c0, k, rank);
            else note_bad(A, kCtrBadOffsets);  // offsets out of order: no region for the op
        }
        A.op_cell[i] = cell;
        A.op_rank[i] = rank;
    }
}

// Start of a set batch of off[ntables] ops, in one launch: zero the batch
// counters (all but kCtrHostN, copied in before this kernel), the probe
// phase's counters (gctr, gctr_words words) and the result bits; cell
// regions of twice each table's ops, so table t's region starts at
// tcell_off[t] = 2 * off[t] (offsets clamped to the op count, so every
// region lies in the 2n cells zeroed here); zero the cells in use and the
// per-table new-key counts.
template <int KB>
__global__ void __launch_bounds__(256) k_set_prep(const __grid_constant__ ApplyScratch A,
                                                  const uint32_t *__restrict__ off,
                                                  uint32_t *__restrict__ bits,
                                                  unsigned long long *__restrict__ gctr,
                                                  uint32_t gctr_words) {
    const uint64_t n = set_op_count(A, off);
    const uint64_t id = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    if (id < (uint64_t)kCtrSlots && id != (uint64_t)kCtrHostN) A.ctr[id] = 0ull;
    if (gctr != nullptr && id < gctr_words) gctr[id] = 0ull;
    for (uint64_t t = id; t <= A.ntables; t += stride) {
        A.tcell_off[t] = 2u * (uint32_t)(off[t] < n ? off[t] : n);
        if (t < A.ntables) A.tup[t] = A.ter[t] = 0u;
    }
    for (uint64_t b = id; b * kTidxStep < n; b += stride)
        A.tidx[b] = table_of(off, A.ntables, (uint32_t)(b * kTidxStep));
    const uint64_t words = 2 * n * (cell_bytes<KB>() / 8);
    for (uint64_t c = id; c < words; c += stride) ((unsigned long long *)A.cells)[c] = 0ull;
    if (bits != nullptr)
        for (uint64_t w = id; w < (n + 31) / 32; w += stride) bits[w] = 0u;
}

// Block-wide exclusive allocation of F counters at once: x packs F fields of
// B bits (no field's block total may exceed B bits); one scan, one atomic per
// nonzero field total, out[f] = that counter's base + the field's sum over
// the threads before this one. Every thread of the block must call it at the
// same point.
template <int F, int B>
__device__ __forceinline__ void block_alloc(unsigned long long *ctr, const int (&slot)[F],
                                            unsigned long long x, uint32_t (&out)[F]) {
    __shared__ unsigned long long wsum[32];
    __shared__ unsigned long long bbase[F];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const unsigned long long mask = B == 64 ? ~0ull : ((1ull << B) - 1ull);
    unsigned long long incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    if (w == 0) {
        const unsigned long long v = lane < nw ? wsum[lane] : 0ull;
        unsigned long long vi = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(kFull, vi, o);
            if (lane >= o) vi += y;
        }
        if (lane < nw) wsum[lane] = vi - v;
        if (lane == 31) {
#pragma unroll
            for (int f = 0; f < F; ++f) {
                const unsigned long long tot = (vi >> (f * B)) & mask;
                bbase[f] = tot ? atomicAdd(&ctr[slot[f]], tot) : 0ull;
            }
        }
    }
    __syncthreads();
    const unsigned long long ex = wsum[w] + incl - x;
#pragma unroll
    for (int f = 0; f < F; ++f) out[f] = (uint32_t)(bbase[f] + ((ex >> (f * B)) & mask));
    __syncthreads();  // wsum / bbase are reused by the next call
}

// Add 1 to cnt[t] for every lane with pred, one atomic per distinct t in the
// warp. All 32 lanes must call.
__device__ __forceinline__ void warp_count_by(uint32_t *cnt, uint32_t t, bool pred) {
    const unsigned peers = __match_any_sync(kFull, pred ? t : 0xffffffffu);
    const int lane = threadIdx.x & 31;
    if (pred && (__ffs(peers) - 1) == lane) atomicAdd(&cnt[t], (uint32_t)__popc(peers));
}

// Compaction of the cells in use: nc for one table, tcell_off[ntables] for
// many (nc = 0). A block takes a tile of 256 * kCompactRun cells; in step k
// its threads read cells k * 256 + threadIdx.x of the tile (coalesced), so
// ids and segment offsets come out in cell order from per-(step, warp)
// ballots and one shared-memory scan per tile.
constexpr int kCompactRun = 4;

template <int KB>
__global__ void __launch_bounds__(256) k_apply_compact(const __grid_constant__ ApplyScratch A,
                                                       uint64_t nc) {
    __shared__ unsigned long long part[kCompactRun * kWarpsPerBlock];  // ops << 32 | keys
    __shared__ unsigned long long base_keys, base_ops;
    __shared__ int tile_ok;  // the tile's key and op ranges lie inside the scratch
    if (A.gate != nullptr && *A.gate == 0ull) return;  // no key repeats: one-pass path
    if (A.tcell_off) nc = A.tcell_off[A.ntables];
    if (nc > A.cap_cells) nc = A.cap_cells;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint64_t tile = (uint64_t)blockDim.x * kCompactRun;
    const uint64_t stride = (uint64_t)gridDim.x * tile;
    for (uint64_t c0 = (uint64_t)blockIdx.x * tile; c0 < nc; c0 += stride) {
        uint32_t cnt[kCompactRun], ex_ops[kCompactRun], ex_keys[kCompactRun];
#pragma unroll
        for (int k = 0; k < kCompactRun; ++k) {
            const uint64_t c = c0 + (uint64_t)k * blockDim.x + threadIdx.x;
            cnt[k] = c < nc ? *cell_word<KB>(A.cells, c) : 0u;
            if (A.single_pass && cnt[k] == 1u) cnt[k] = 0u;  // left to the one-pass kernel
            const unsigned used = __ballot_sync(kFull, cnt[k] != 0u);
            ex_keys[k] = __popc(used & ((1u << lane) - 1u));
            uint32_t incl = cnt[k];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(kFull, incl, o);
                if (lane >= o) incl += y;
            }
            ex_ops[k] = incl - cnt[k];
            if (lane == 31)
                part[k * kWarpsPerBlock + w] = ((unsigned long long)incl << 32) | __popc(used);
        }
        __syncthreads();
        if (w == 0) {  // exclusive scan of the 32 (step, warp) totals, one per lane
            static_assert(kCompactRun * kWarpsPerBlock == 32, "one total per lane");
            const unsigned long long a0 = part[lane];
            unsigned long long incl = a0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long y = __shfl_up_sync(kFull, incl, o);
                if (lane >= o) incl += y;
            }
            part[lane] = incl - a0;
            if (lane == 31) {
                const unsigned long long nk = incl & 0xffffffffull, no = incl >> 32;
                base_keys = nk ? atomicAdd(&A.ctr[kCtrDistinct], nk) : 0ull;
                base_ops = no ? atomicAdd(&A.ctr[kCtrPlaced], no) : 0ull;
                tile_ok = base_keys + nk <= A.cap_ops && base_ops + no <= A.cap_ops;
            }
        }
        __syncthreads();
        if (tile_ok) {  // every id and segment of the tile is inside its range
#pragma unroll
            for (int k = 0; k < kCompactRun; ++k) {
                if (!cnt[k]) continue;
                const unsigned long long pk = part[k * kWarpsPerBlock + w];
                const uint32_t d = (uint32_t)base_keys + (uint32_t)pk + ex_keys[k];
                const uint32_t off = (uint32_t)base_ops + (uint32_t)(pk >> 32) + ex_ops[k];
                const uint64_t c = c0 + (uint64_t)k * blockDim.x + threadIdx.x;
                *cell_word<KB>(A.cells, c) = kIdBit | d;  // the count becomes the distinct id
                ((typename SlotT<KB>::K *)A.dkey)[d] = cell_key<KB>(A.cells, c);
                A.dcnt[d] = cnt[k];
                A.dseg[d] = (unsigned long long)off << 32;
                if (A.dtid)
                    A.dtid[d] = table_at(A.tidx, A.tcell_off, (uint32_t)c, (uint32_t)(c >> 1));
            }
        } else {
            // more keys or ops than the scratch holds (counts this batch's
            // grouping cannot have produced; the call reports them): the
            // tile's cells get no id, and its ids inside the range a count
            // of 0, so the later passes skip them and every id below the
            // distinct count is written
            if (threadIdx.x == 0) note_bad(A);
            for (int k = 0; k < kCompactRun; ++k) {
                if (!cnt[k]) continue;
                const uint64_t d64 =
                    base_keys + (uint32_t)part[k * kWarpsPerBlock + w] + ex_keys[k];
                *cell_word<KB>(A.cells, c0 + (uint64_t)k * blockDim.x + threadIdx.x) = kNoId;
                if (d64 < A.cap_ops) A.dcnt[d64] = 0u;
            }
        }
        __syncthreads();  // part / bases / tile_ok are reused by the next tile
    }
}

__device__ __forceinline__ uint32_t seg_off(const ApplyScratch &A, uint32_t d) {
    return (uint32_t)(A.dseg[d] >> 32);
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

// Final state of distinct key d, recorded by one thread (warp and block
// paths).
template <int KB>
__device__ __forceinline__ void record_final_one(const ApplyScratch &A, uint32_t d, bool present,
                                                 uint64_t value, bool pre_present,
                                                 uint64_t pre_value, uint32_t vb) {
    using K = typename SlotT<KB>::K;
    const K k = ((const K *)A.dkey)[d];
    if (present && (!pre_present || value != pre_value)) {
        const unsigned long long u = atomicAdd(&A.ctr[kCtrUp], 1ull);
        if (u >= A.cap_ops) {
            note_bad(A);
            return;
        }
        ((K *)A.up_key)[u] = k;
        if (vb == 4) ((uint32_t *)A.up_val)[u] = (uint32_t)value;
        else ((unsigned long long *)A.up_val)[u] = value;
        if (A.dtid) {
            A.up_tid[u] = A.dtid[d];
            atomicAdd(&A.tup[A.dtid[d]], 1u);
        }
    } else if (!present && pre_present) {
        const unsigned long long e = atomicAdd(&A.ctr[kCtrEr], 1ull);
        if (e >= A.cap_ops) {
            note_bad(A);
            return;
        }
        ((K *)A.er_key)[e] = k;
        if (A.dtid) {
            A.er_tid[e] = A.dtid[d];
            atomicAdd(&A.ter[A.dtid[d]], 1u);
        }
    }
}

// The pass over the ops in op order, after the find of the distinct keys.
// A key with a single op in the batch is resolved here: its result is the
// key's state before the batch, written in op order (values coalesced, the
// hit bits one word per warp by ballot), and its final state goes to the
// upsert / erase lists. Ops of keys with several ops go into their key's
// segment, at the rank the grouping handed them, for the replay kernels.
// Key-0 ops (no cell) report a miss. Whole blocks step through the ops so
// every thread reaches block_alloc. n_ptr (many tables: offsets[ntables])
// gives the op count on the device instead of n, so that a captured launch
// serves batches of any size.
template <int KB>
__global__ void __launch_bounds__(256) k_apply_scatter(const __grid_constant__ ApplyScratch A,
                                                       uint64_t n, const uint32_t *n_ptr,
                                                       const uint8_t *__restrict__ ops,
                                                       const void *__restrict__ vals, uint32_t vb,
                                                       void *__restrict__ vals_out,
                                                       uint32_t *__restrict__ bits_out) {
    using K = typename SlotT<KB>::K;
    if (A.gate != nullptr && *A.gate == 0ull) return;  // no key repeats: one-pass path
    const uint32_t *off = n_ptr ? n_ptr - A.ntables : nullptr;  // n_ptr = offsets + ntables
    if (n_ptr) n = set_op_count(A, off);
    const int slots[2] = {kCtrUp, kCtrEr};
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
        const uint64_t i = i0 + threadIdx.x;
        bool up = false, er = false, hit = false;
        bool one_up = false;  // an insert the one-pass kernel resolves (a table's upsert count)
        bool left = false;    // op i is left to the one-pass kernel
        K k = 0;
        uint64_t value = 0ull;
        uint32_t tid = 0u;
        if (i < n) {
            const uint32_t cell = A.op_cell[i];
            uint32_t d = (cell == kNoCell || cell >= A.cap_cells)
                             ? kNoId : *cell_word<KB>(A.cells, cell);
            if (d != kNoId) d = (d & kIdBit) ? (d & ~kIdBit) : kNoId - 1u;  // no bit: one op
            if (A.single_pass && (cell == kNoCell || d == kNoId - 1u)) {
                left = true;
                // key 0 or a key with one op: resolved by the one-pass kernel;
                // a set's upsize policy counts the insert of a key with one op
                // as an upsert of its table
                if (A.tup && cell != kNoCell && ops[i] == kOpInsert) {
                    one_up = true;
                    tid = table_at(A.tidx, off, (uint32_t)i, (uint32_t)i);
                }
            } else if (d >= A.cap_ops) {  // key 0 (no cell), or a cell compaction could not list
                if (cell != kNoCell) note_bad(A);
                if (vals_out) store_val(vals_out, vb, i, 0ull);
            } else {
                const uint32_t cnt = A.dcnt[d];
                if (cnt == 1u) {
                    const bool pre = (A.pre_hit[d >> 5] >> (d & 31)) & 1u;
                    const uint64_t pre_value = load_val(A.pre_val, vb, d);
                    if (vals_out) store_val(vals_out, vb, i, pre ? pre_value : 0ull);
                    hit = pre;
                    const uint8_t op = ops[i];
                    bool present = pre;
                    value = pre_value;
                    replay_op(op, op == kOpInsert ? load_val(vals, vb, i) : 0ull, present, value);
                    up = present && (!pre || value != pre_value);
                    er = !present && pre;
                    if (up || er) {
                        k = ((const K *)A.dkey)[d];
                        if (A.dtid) tid = A.dtid[d];
                    }
                } else {
                    // a rank is below its key's count by construction; the
                    // test keeps a write inside the key's own segment even
                    // if the grouping's state were not (as under a profiler
                    // replay of the grouping)
                    const uint32_t r = A.op_rank[i];
                    if (r < cnt && seg_ok(A, seg_off(A, d), r + 1))
                        A.seg[seg_off(A, d) + r] = (uint32_t)i;
                    else
                        note_bad(A);
                }
            }
        }
        // i0 is a multiple of 256: a warp's 32 ops are one word of bits
        const unsigned hits = __ballot_sync(kFull, hit);
        if (bits_out && (threadIdx.x & 31) == 0 && i < n) bits_out[i >> 5] = hits;
        const unsigned lefts = __ballot_sync(kFull, left);
        if (A.single_pass && (threadIdx.x & 31) == 0 && i < n) A.single[i >> 5] = lefts;
        uint32_t got[2];
        block_alloc<2, 32>(A.ctr, slots, (unsigned long long)up | ((unsigned long long)er << 32),
                           got);
        if (A.tup) {
            warp_count_by(A.tup, tid, up || one_up);
            warp_count_by(A.ter, tid, er);
        }
        if ((up && got[0] >= A.cap_ops) || (er && got[1] >= A.cap_ops)) {
            note_bad(A);
        } else if (up) {
            ((K *)A.up_key)[got[0]] = k;
            if (vb == 4) ((uint32_t *)A.up_val)[got[0]] = (uint32_t)value;
            else ((unsigned long long *)A.up_val)[got[0]] = value;
            if (A.up_tid) A.up_tid[got[0]] = tid;
        } else if (er) {
            ((K *)A.er_key)[got[1]] = k;
            if (A.er_tid) A.er_tid[got[1]] = tid;
        }
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
                                                      uint32_t *__restrict__ bits_out, uint64_t n,
                                                      const uint32_t *n_ptr) {
    using K = typename SlotT<KB>::K;
    (void)n;  // key-0 ops and single-op keys were resolved by the scatter pass
    (void)n_ptr;
    const uint64_t nd = ctr_count(A, kCtrDistinct);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const int slots[4] = {kCtrUp, kCtrEr, kCtrWarp, kCtrMid};
    // whole blocks step through the distinct keys so every thread reaches
    // the block_alloc call
    for (uint64_t d0 = (uint64_t)blockIdx.x * blockDim.x; d0 < nd; d0 += stride) {
        const uint64_t d = d0 + threadIdx.x;
        bool up = false, er = false, wp = false, md = false;
        K k = 0;
        uint64_t value = 0ull;
        uint32_t tid = 0u;
        if (d < nd) {
            const uint32_t cnt = A.dcnt[d];
            if (cnt > kWarpSeg) {
                md = true;
            } else if (cnt > kShortSeg) {
                wp = true;
            } else if (cnt > 1u) {  // segment inside the op scratch: compaction checked it
                uint32_t s[kShortSeg];
                const uint32_t off = seg_off(A, (uint32_t)d);
#pragma unroll
                for (uint32_t a = 0; a < kShortSeg; ++a) s[a] = a < cnt ? A.seg[off + a] : 0xffffffffu;
                // odd-even transposition network in registers (padding sorts last)
#pragma unroll
                for (uint32_t r = 0; r < kShortSeg; ++r) {
#pragma unroll
                    for (uint32_t a = r & 1u; a + 1 < kShortSeg; a += 2) {
                        const uint32_t lo = min(s[a], s[a + 1]), hi = max(s[a], s[a + 1]);
                        s[a] = lo;
                        s[a + 1] = hi;
                    }
                }
                k = ((const K *)A.dkey)[d];
                const bool pre_present = (A.pre_hit[d >> 5] >> (d & 31)) & 1u;
                const uint64_t pre_value = load_val(A.pre_val, vb, d);
                bool present = pre_present;
                value = pre_value;
#pragma unroll
                for (uint32_t a = 0; a < kShortSeg; ++a) {
                    if (a >= cnt) break;
                    const uint32_t i = s[a];
                    const uint8_t op = ops[i];
                    // every op reports the state just before it
                    if (vals_out) store_val(vals_out, vb, i, present ? value : 0ull);
                    if (present && bits_out) atomicOr(&bits_out[i >> 5], 1u << (i & 31));
                    replay_op(op, op == kOpInsert ? load_val(vals, vb, i) : 0ull, present, value);
                }
                up = present && (!pre_present || value != pre_value);
                er = !present && pre_present;
                if (A.dtid) tid = A.dtid[d];
            }
        }
        uint32_t got[4];
        block_alloc<4, 16>(A.ctr, slots,
                           (unsigned long long)up | ((unsigned long long)er << 16) |
                               ((unsigned long long)wp << 32) | ((unsigned long long)md << 48),
                           got);
        if (A.tup) {
            warp_count_by(A.tup, tid, up);
            warp_count_by(A.ter, tid, er);
        }
        const uint32_t at = up ? got[0] : er ? got[1] : wp ? got[2] : got[3];
        if ((up || er || wp || md) && at >= A.cap_ops) {
            note_bad(A);
        } else if (up) {
            ((K *)A.up_key)[got[0]] = k;
            if (vb == 4) ((uint32_t *)A.up_val)[got[0]] = (uint32_t)value;
            else ((unsigned long long *)A.up_val)[got[0]] = value;
            if (A.up_tid) A.up_tid[got[0]] = tid;
        } else if (er) {
            ((K *)A.er_key)[got[1]] = k;
            if (A.er_tid) A.er_tid[got[1]] = tid;
        } else if (wp) {
            A.wseg[got[2]] = (uint32_t)d;
        } else if (md) {
            A.mid[got[3]] = (uint32_t)d;
        }
    }
}

// Ascending bitonic sort of s[0..P) (P a power of two) by the threads
// [t0, t0 + nt) of the caller's group; sync() separates the stages.
template <class Sync>
__device__ __forceinline__ void bitonic_sort(uint32_t *s, uint32_t P, uint32_t t0, uint32_t nt,
                                             Sync sync) {
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t t = t0; t < P; t += nt) {
                const uint32_t u = t ^ j;
                if (u > t) {
                    const uint32_t a = s[t], b = s[u];
                    if ((a > b) == ((t & k) == 0)) {
                        s[t] = b;
                        s[u] = a;
                    }
                }
            }
            sync();
        }
    }
}

// Warp segments (kShortSeg < ops <= kWarpSeg): one warp per segment sorts
// it in its own shared memory and replays it. A warp takes kWarpTask
// segments in a row and keeps segment j's final state in lane j, so the
// erase / upsert lists get one warp-aggregated allocation per task (one
// global counter bumped per segment serialised this kernel; tasks of 32
// segments left most warps idle when a round had few warp segments).
template <int KB>
__global__ void __launch_bounds__(256) k_apply_replay_warp(const __grid_constant__ ApplyScratch A,
                                                           const uint8_t *__restrict__ ops,
                                                           const void *__restrict__ vals,
                                                           uint32_t vb, void *__restrict__ vals_out,
                                                           uint32_t *__restrict__ bits_out) {
    using K = typename SlotT<KB>::K;
    __shared__ uint32_t s_all[kWarpsPerBlock][kWarpSeg];
    uint32_t *s = s_all[threadIdx.x >> 5];
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t nw = ctr_count(A, kCtrWarp);
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    for (uint64_t x0 = gw * kWarpTask; x0 < nw; x0 += warps * kWarpTask) {
        uint32_t rd = 0;
        bool rvalid = false, rpresent = false, rpre = false;
        uint64_t rvalue = 0ull, rpre_value = 0ull;
        for (uint32_t j = 0; j < kWarpTask && x0 + j < nw; ++j) {
            const uint32_t d = A.wseg[x0 + j];  // d, cnt and off are warp-uniform
            if (d >= A.cap_ops) {
                if (lane == 0) note_bad(A);
                continue;
            }
            const uint32_t cnt = A.dcnt[d], off = seg_off(A, d);  // kShortSeg < cnt <= kWarpSeg
            if (cnt <= kShortSeg || cnt > kWarpSeg || !seg_ok(A, off, cnt)) {
                if (lane == 0) note_bad(A);
                continue;
            }
            uint32_t P = 32;
            while (P < cnt) P <<= 1;
            for (uint32_t q = lane; q < P; q += 32) s[q] = q < cnt ? A.seg[off + q] : 0xffffffffu;
            __syncwarp();
            bitonic_sort(s, P, lane, 32, [] { __syncwarp(); });
            const bool pre_present = (A.pre_hit[d >> 5] >> (d & 31)) & 1u;
            const uint64_t pre_value = load_val(A.pre_val, vb, d);
            bool present = pre_present;
            uint64_t value = pre_value;
            warp_replay(s, cnt, present, value, ops, vals, vb, vals_out, bits_out);
            if (lane == j) {
                rd = d;
                rvalid = true;
                rpresent = present;
                rvalue = value;
                rpre = pre_present;
                rpre_value = pre_value;
            }
            __syncwarp();  // s is reused by the next segment
        }
        const bool up = rvalid && rpresent && (!rpre || rvalue != rpre_value);
        const bool er = rvalid && !rpresent && rpre;
        const uint32_t tid = (rvalid && A.dtid) ? A.dtid[rd] : 0u;
        const unsigned long long u = agg_inc(&A.ctr[kCtrUp], up);
        const unsigned long long e = agg_inc(&A.ctr[kCtrEr], er);
        if (A.tup) {
            warp_count_by(A.tup, tid, up);
            warp_count_by(A.ter, tid, er);
        }
        if ((up && u >= A.cap_ops) || (er && e >= A.cap_ops)) {
            note_bad(A);
        } else if (up) {
            ((K *)A.up_key)[u] = ((const K *)A.dkey)[rd];
            if (vb == 4) ((uint32_t *)A.up_val)[u] = (uint32_t)rvalue;
            else ((unsigned long long *)A.up_val)[u] = rvalue;
            if (A.up_tid) A.up_tid[u] = tid;
        } else if (er) {
            ((K *)A.er_key)[e] = ((const K *)A.dkey)[rd];
            if (A.er_tid) A.er_tid[e] = tid;
        }
    }
}

// Block segments (more than kWarpSeg ops on one key): one block per segment.
// Up to kMidSeg ops are sorted in shared memory; a longer segment is sorted
// in kMidSeg chunks in shared memory and then merged in global memory, run
// widths doubling, each element placed by its rank in the other run (op
// indices are distinct, so ranks are exact), ping-ponging with the scratch
// copy at the same offsets. Warp 0 replays the sorted segment.
template <int KB>
__global__ void __launch_bounds__(256) k_apply_replay_mid(const __grid_constant__ ApplyScratch A,
                                                          const uint8_t *__restrict__ ops,
                                                          const void *__restrict__ vals,
                                                          uint32_t vb, void *__restrict__ vals_out,
                                                          uint32_t *__restrict__ bits_out) {
    __shared__ uint32_t s[kMidSeg];
    const uint64_t nmid = ctr_count(A, kCtrMid);
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    for (uint64_t x = blockIdx.x; x < nmid; x += gridDim.x) {
        const uint32_t d = A.mid[x];  // d, cnt and off are the same for the whole block
        if (d >= A.cap_ops) {
            if (tid == 0) note_bad(A);
            continue;
        }
        const uint32_t cnt = A.dcnt[d], off = seg_off(A, d);  // cnt > kWarpSeg
        if (cnt <= kWarpSeg || !seg_ok(A, off, cnt)) {
            if (tid == 0) note_bad(A);
            continue;
        }
        const uint32_t *sorted = s;
        if (cnt <= kMidSeg) {
            uint32_t P = 2u * kWarpSeg;
            while (P < cnt) P <<= 1;
            for (uint32_t j = tid; j < P; j += nt) s[j] = j < cnt ? A.seg[off + j] : 0xffffffffu;
            __syncthreads();
            bitonic_sort(s, P, tid, nt, [] { __syncthreads(); });
        } else {
            uint32_t *src = A.seg + off, *dst = A.sort_tmp + off;
            for (uint32_t c0 = 0; c0 < cnt; c0 += kMidSeg) {  // sorted chunks, in place
                const uint32_t m = cnt - c0 < kMidSeg ? cnt - c0 : kMidSeg;
                for (uint32_t j = tid; j < kMidSeg; j += nt) s[j] = j < m ? src[c0 + j] : 0xffffffffu;
                __syncthreads();
                bitonic_sort(s, kMidSeg, tid, nt, [] { __syncthreads(); });
                for (uint32_t j = tid; j < m; j += nt) src[c0 + j] = s[j];
                __syncthreads();
            }
            for (uint32_t w = kMidSeg; w < cnt; w *= 2) {  // merge runs of w into runs of 2w
                for (uint32_t i = tid; i < cnt; i += nt) {
                    const uint32_t r0 = i / (2 * w) * (2 * w);
                    const uint32_t mid = r0 + w < cnt ? r0 + w : cnt;
                    const uint32_t end = r0 + 2 * w < cnt ? r0 + 2 * w : cnt;
                    const uint32_t v = src[i];
                    // rank of v in the other run (elements smaller than v)
                    uint32_t lo = i < mid ? mid : r0, hi = i < mid ? end : mid;
                    const uint32_t base = lo;
                    while (lo < hi) {
                        const uint32_t m = (lo + hi) >> 1;
                        if (src[m] < v) lo = m + 1;
                        else hi = m;
                    }
                    const uint32_t own = i < mid ? i - r0 : i - mid;
                    dst[r0 + own + (lo - base)] = v;
                }
                __syncthreads();
                uint32_t *t = src;
                src = dst;
                dst = t;
            }
            sorted = src;
        }
        if (tid < 32) {
            const bool pre_present = (A.pre_hit[d >> 5] >> (d & 31)) & 1u;
            const uint64_t pre_value = load_val(A.pre_val, vb, d);
            bool present = pre_present;
            uint64_t value = pre_value;
            warp_replay(sorted, cnt, present, value, ops, vals, vb, vals_out, bits_out);
            if (tid == 0) record_final_one<KB>(A, d, present, value, pre_present, pre_value, vb);
        }
        __syncthreads();  // s and the scratch run are reused by the next segment
    }
}

// ----------------------------------------------------------------------------
// Mixed batch whose keys are all distinct (dyc_apply with DYC_FLAG_UNIQUE):
// with one op per key no op depends on another, so each is resolved and
// applied in a single pass, without the grouping, compaction and replay the
// general path needs for repeated keys. An op probes its key's first bucket,
// and the second one where the key or (for an insert) an empty slot may be
// there; it reports the key's state before it, as the general path does.
// Then an insert updates the key's own slot or claims an empty one (ops left
// without a slot go to list_a for the eviction walks that follow the pass),
// and an erase clears the key's slot. Ops on different keys run side by
// side: nothing in the pass moves an entry, so a find never misses a key
// that is present, and a key's own slot is written only by its own op.
// ----------------------------------------------------------------------------
template <int KB, int SB, bool HINT>
__global__ void __launch_bounds__(256) k_apply_unique(
    const __grid_constant__ Desc D, const __grid_constant__ Scratch S,
    const uint8_t *__restrict__ ops, const void *__restrict__ keys,
    const void *__restrict__ vals, uint32_t vb, void *__restrict__ vals_out,
    uint32_t *__restrict__ bits_out, uint64_t n, Counters *ctr, const uint32_t *single,
    const unsigned long long *gate) {
    using T = SlotT<KB>;
    using Sl = typename T::S;
    using Gm = Geo<KB, SB>;
    // no key repeated in the chunk (the grouping's flag): every op is ours
    // (the scatter did not run, so the bitmap is not written)
    if (single != nullptr && gate != nullptr && *gate == 0ull) single = nullptr;
    const bool all_ops = single == nullptr;
    __shared__ __align__(128) unsigned char s_stage[SB >= 64 ? kWarpsPerBlock : 1][32 * SB];
    unsigned char *stage = s_stage[SB >= 64 ? (threadIdx.x >> 5) : 0];
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t step = warp_stride();
    const unsigned long long tpol = HINT ? l2_policies(true).table : 0ull;
    uint32_t n_ins = 0, n_upd = 0, n_del = 0;
    for (uint64_t base = warp_base(); base < n; base += step) {
        const uint64_t i = base + lane;
        typename T::K k = 0;
        uint8_t op = kOpFind;
        Sl e = T::empty();
        bool mine = i < n;  // this kernel resolves op i
        if (mine && !all_ops) mine = (single[i >> 5] >> (i & 31)) & 1u;  // one op, or key 0
        if (mine) {
            k = load_key<KB>(keys, i);
            op = ops[i];
        }
        const bool act = k != 0;  // ops on key 0 miss and change nothing
        const bool ins = act && op == kOpInsert, del = act && op == kOpErase;
        if (ins) e = T::make(k, load_val(vals, vb, i));
        const uint32_t hk = fold(k);
        const Pair p = pair_of(hk, D.d);
        char *p1 = bucket_ptr<KB, SB>(D, p.first, bucket_index(D, p.first, hk));
        char *p2 = bucket_ptr<KB, SB>(D, p.second, bucket_index(D, p.second, hk));
        const KvOut r1 = place_probe<KB, SB, HINT>(p1, k, act, p.first, D.d, stage, tpol);
        const bool found1 = act && r1.match >= 0;
        // the second bucket holds the key only if the first one's fingerprint
        // bit allows it (always without metadata); an insert also looks there
        // for an empty slot when the first bucket is full
        const bool check2 =
            act && !found1 && ((!Gm::kMeta || r1.overflow) || (ins && r1.empty == 0u));
        KvOut r2{-1, 0ull, false, 0u};
        if (__any_sync(kFull, check2))
            r2 = place_probe<KB, SB, HINT>(p2, k, check2, p.second, D.d, stage, tpol);
        const bool found2 = check2 && r2.match >= 0;
        const bool present = found1 || found2;
        const uint64_t before = found1 ? r1.value : (found2 ? r2.value : 0ull);
        bool pend = false;
        if (ins) {
            if (found1) {
                T::store(slot_ptr<KB, SB>(p1, r1.match), e);
                ++n_upd;
            } else if (found2) {
                T::store(slot_ptr<KB, SB>(p2, r2.match), e);
                ++n_upd;
            } else {
                bool ok = claim_empty<KB, SB>(p1, r1.empty, e);
                if (!ok && check2 && r2.empty) {
                    mark_overflow<KB, SB>(p1, hk);
                    ok = claim_empty<KB, SB>(p2, r2.empty, e);
                }
                if (ok) ++n_ins;
                else pend = true;
            }
        } else if (del && present) {
            T::store(found1 ? slot_ptr<KB, SB>(p1, r1.match) : slot_ptr<KB, SB>(p2, r2.match),
                     T::empty());
            ++n_del;
        }
        if (vals_out != nullptr && mine) store_val(vals_out, vb, i, before);
        const unsigned m = __ballot_sync(kFull, present);
        if (bits_out != nullptr && lane == 0) {
            if (all_ops) bits_out[base >> 5] = m;
            else if (m) atomicOr(&bits_out[base >> 5], m);  // the replays own the other bits
        }
        __syncwarp();
        const unsigned long long at = agg_inc(&ctr->pending, pend);
        if (pend) {
            if (at < S.list_cap) ((Sl *)S.list_a)[at] = e;
            else atomicAdd(&ctr->spill, 1ull);
        }
    }
    // one atomic per counter per block
    __shared__ unsigned long long s_sum[3];
    if (threadIdx.x < 3) s_sum[threadIdx.x] = 0ull;
    __syncthreads();
    const uint32_t w_ins = __reduce_add_sync(kFull, n_ins), w_upd = __reduce_add_sync(kFull, n_upd);
    const uint32_t w_del = __reduce_add_sync(kFull, n_del);
    if (lane == 0) {
        if (w_ins) atomicAdd(&s_sum[0], (unsigned long long)w_ins);
        if (w_upd) atomicAdd(&s_sum[1], (unsigned long long)w_upd);
        if (w_del) atomicAdd(&s_sum[2], (unsigned long long)w_del);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_sum[0]) atomicAdd(&ctr->inserted, s_sum[0]);
        if (s_sum[1]) atomicAdd(&ctr->updated, s_sum[1]);
        if (s_sum[2]) atomicAdd(&ctr->erased, s_sum[2]);
        const long long net = (long long)s_sum[0] - (long long)s_sum[2];
        if (net) atomicAdd(&ctr->size, (unsigned long long)net);  // size += inserted - erased
    }
}

// *count += the INSERT ops among ops[0..n) (one atomic per block).
template <int KB>
__global__ void __launch_bounds__(256) k_count_inserts(const uint8_t *__restrict__ ops, uint64_t n,
                                                       unsigned long long *count) {
    uint32_t c = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        c += ops[i] == kOpInsert ? 1u : 0u;
    __shared__ unsigned long long s_c;
    if (threadIdx.x == 0) s_c = 0ull;
    __syncthreads();
    c = __reduce_add_sync(kFull, c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(&s_c, (unsigned long long)c);
    __syncthreads();
    if (threadIdx.x == 0 && s_c) atomicAdd(count, s_c);
}

}  // namespace dyc
