// dyc_wide.cuh -- kernels of the wide-value table (dyc_wide_*): values of
// any size (a multiple of 4 bytes) kept in a value heap, the cuckoo table
// mapping each key to a 32-bit handle (its row in the heap).
//
// The reference's variant for values wider than its 4-byte slot half
// (GPU/warp: separate key[]/value[] arrays per bucket, cuckoo.h:15-18) takes
// an atomicCAS lock per bucket (cuckoo.cu:95-101) so that a key and its
// value move together. Here a batch is deduplicated first, so every key has
// one writer per call, and an entry that moves (eviction walk, resize) is the
// 8- or 16-byte (key, handle) slot, exchanged atomically as in the plain
// table; the value itself never moves. No locks, nothing spins.
#pragma once

#include "dyc_kernels.cuh"

namespace dyc {

// Handle allocator state (device): free handles are a stack; handles at and
// above `bump` were never used.
struct WideAlloc {
    uint32_t free_top;  // entries on the free stack
    uint32_t bump;      // first never-used handle
    uint32_t cap;       // heap rows
    uint32_t taken;     // handles handed out by the current stage kernel
    uint32_t pushed;    // handles pushed by the current free kernel
    uint32_t pad[3];
};

__device__ __forceinline__ void copy_words(uint32_t *__restrict__ dst,
                                           const uint32_t *__restrict__ src, uint32_t words) {
    if ((((uintptr_t)dst | (uintptr_t)src) & 15u) == 0 && (words & 3u) == 0) {
        for (uint32_t w = 0; w < words; w += 4)
            *(uint4 *)(dst + w) = *(const uint4 *)(src + w);
    } else {
        for (uint32_t w = 0; w < words; ++w) dst[w] = src[w];
    }
}

// Insert staging: present keys (hit in `pre_bits`, handle in `pre_h`) get
// their heap row overwritten; new keys get a handle (free stack first, then
// the never-used range), their value is written, and (key, handle) is listed
// for placement. Ops on key 0 and ops superseded by a later one in the batch
// do nothing. The allocator state is only read here (k_wide_commit applies
// what was handed out).
template <int KB>
__global__ void __launch_bounds__(256) k_wide_stage(const __grid_constant__ Scratch S, int use_dedup,
                                                    const void *__restrict__ keys,
                                                    const uint32_t *__restrict__ vals,
                                                    uint32_t words, uint64_t n,
                                                    const uint32_t *__restrict__ pre_h,
                                                    const uint32_t *__restrict__ pre_bits,
                                                    uint32_t *__restrict__ heap,
                                                    const uint32_t *__restrict__ stack,
                                                    WideAlloc *A, void *new_keys,
                                                    uint32_t *new_h,
                                                    unsigned long long *new_count,
                                                    unsigned long long *upd_count) {
    using K = typename SlotT<KB>::K;
    const uint32_t free_top = A->free_top, bump = A->bump;
    const uint64_t step = warp_stride();
    for (uint64_t base = warp_base(); base < n; base += step) {
        const uint64_t i = base + (threadIdx.x & 31);
        bool fresh = false, upd = false;
        K k = 0;
        if (i < n) {
            k = load_key<KB>(keys, i);
            if (k != 0 && (!use_dedup || Dedup<KB>::winner(S, k, (uint32_t)i))) {
                if ((pre_bits[i >> 5] >> (i & 31)) & 1u) {
                    copy_words(heap + (uint64_t)pre_h[i] * words, vals + i * words, words);
                    upd = true;
                } else {
                    fresh = true;
                }
            }
        }
        agg_inc(upd_count, upd);
        const unsigned long long at = agg_inc(new_count, fresh);
        if (fresh) {
            const uint32_t x = atomicAdd(&A->taken, 1u);
            const uint32_t h = x < free_top ? stack[free_top - 1 - x] : bump + (x - free_top);
            copy_words(heap + (uint64_t)h * words, vals + i * words, words);
            ((K *)new_keys)[at] = k;
            new_h[at] = h;
        }
    }
}

// After a stage kernel: the free stack and the never-used range shrink by
// what it handed out.
__global__ void k_wide_commit(WideAlloc *A) {
    const uint32_t t = A->taken;
    const uint32_t from_stack = t < A->free_top ? t : A->free_top;
    A->free_top -= from_stack;
    A->bump += t - from_stack;
    A->taken = 0;
}

// Find: the value of every hit (zeros on a miss; bits == nullptr: all hit).
__global__ void __launch_bounds__(256) k_wide_gather(const uint32_t *__restrict__ h,
                                                     const uint32_t *__restrict__ bits,
                                                     uint64_t n, const uint32_t *__restrict__ heap,
                                                     uint32_t words, uint32_t *__restrict__ out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint32_t *o = out + i * words;
        if (!bits || ((bits[i >> 5] >> (i & 31)) & 1u)) {
            copy_words(o, heap + (uint64_t)h[i] * words, words);
        } else {
            for (uint32_t w = 0; w < words; ++w) o[w] = 0u;
        }
    }
}

// Erase: every removed key's handle goes back on the free stack, and its
// value to out (when given; zeros for ops that removed nothing).
__global__ void __launch_bounds__(256) k_wide_free(const uint32_t *__restrict__ h,
                                                   const uint32_t *__restrict__ erased,
                                                   uint64_t n, const uint32_t *__restrict__ heap,
                                                   uint32_t words, uint32_t *__restrict__ out,
                                                   uint32_t *__restrict__ stack, WideAlloc *A) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const bool e = (erased[i >> 5] >> (i & 31)) & 1u;
        if (out) {
            uint32_t *o = out + i * words;
            if (e) copy_words(o, heap + (uint64_t)h[i] * words, words);
            else
                for (uint32_t w = 0; w < words; ++w) o[w] = 0u;
        }
        if (e) stack[A->free_top + atomicAdd(&A->pushed, 1u)] = h[i];
    }
}

__global__ void k_wide_commit_free(WideAlloc *A) {
    A->free_top += A->pushed;
    A->pushed = 0;
}

}  // namespace dyc
