// dyc_kernels.cuh -- the sm_103a kernels of the DyCuckoo table, templated on
// key width KB (4 or 8 bytes) and bucket size SB (32, 64 or 128 bytes).
//
// Design (GB300):
//   * A random DRAM access on this part moves a whole 128-byte line and the
//     part sustains about 5e10 of them per second whatever their size, so a
//     128-byte bucket (one line) costs the same as a 32-byte one and holds 4x
//     the entries. A bucket is read by a group of SB/32 lanes, one 256-bit
//     load each; a warp instruction therefore fetches whole lines (a single
//     thread issuing four loads to one line runs four times slower).
//   * Every lane owns one op; probe() serves the ops of a warp round by
//     round and hands each owner the facts about its bucket (matching slot,
//     empty slots, metadata word). Reads need cooperation; the atomics that
//     follow are per-owner.
//   * Loops are warp-uniform (all 32 lanes run the same iterations), so
//     shuffles and ballots always use the full mask.
//   * Insert runs in phases separated by kernel boundaries: (1) resolve
//     repeated keys of the batch, (2) update present keys / claim empty
//     slots -- nothing moves while keys are being searched, (3) eviction
//     walks for the ops whose two buckets were full. Phase 3 only places keys
//     known to be absent, so an entry in flight can never be mistaken for a
//     missing key.
//   * Every loop is bounded: probe loops by the table size, walks by the
//     eviction bound. Nothing spins on another thread.
//   * Random-access kernels run one block per 2048 items (tile_grid in
//     dyc_ops.cuh): many short blocks keep more line fetches in flight than
//     one resident wave looping; their counters are added once per block.
#pragma once

#include "dyc_device.cuh"

namespace dyc {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ uint64_t warp_base() {
    return (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) << 5;
}
__device__ __forceinline__ uint64_t warp_stride() {
    return ((uint64_t)gridDim.x * blockDim.x) & ~31ull;
}

template <int KB, int SB>
__device__ __forceinline__ typename SlotT<KB>::S *slot_ptr(char *bucket, int j) {
    return reinterpret_cast<typename SlotT<KB>::S *>(bucket + j * SlotT<KB>::kBytes);
}

__device__ __forceinline__ unsigned long long shfl64(unsigned long long v, int src) {
    return __shfl_sync(kFull, v, src);
}
__device__ __forceinline__ unsigned long long shfl_slot(unsigned long long v, int src) {
    return shfl64(v, src);
}
__device__ __forceinline__ u128 shfl_slot(u128 v, int src) {
    return {shfl64(v.lo, src), shfl64(v.hi, src)};
}

// Claim the first empty slot of `mask` in the bucket at p for e (CAS).
template <int KB, int SB>
__device__ __forceinline__ bool claim_empty(char *p, unsigned mask, const typename SlotT<KB>::S &e) {
    using T = SlotT<KB>;
#pragma unroll 1
    while (mask) {
        const int j = __ffs(mask) - 1;
        mask &= mask - 1;
        const typename T::S old = T::cas(slot_ptr<KB, SB>(p, j), T::empty(), e);
        if (T::same(old, T::empty())) return true;
    }
    return false;
}

// The first-probe bucket of an entry's key.
template <int KB, int SB>
__device__ __forceinline__ char *first_bucket(const Desc &D, typename SlotT<KB>::K k, Pair &pr,
                                              uint32_t &hk) {
    hk = fold(k);
    pr = pair_of(hk, D.d);
    return bucket_ptr<KB, SB>(D, pr.first, bucket_index(D, pr.first, hk));
}

// Set the entry's fingerprint in its first-probe bucket before storing it
// anywhere else (hk = fold(key)).
template <int KB, int SB>
__device__ __forceinline__ void mark_overflow(char *first, uint32_t hk) {
    if (Geo<KB, SB>::kMeta) atomicOr(meta_ptr<KB, SB>(first), fp_bit(hk));
}

// ----------------------------------------------------------------------------
// Cooperative bucket probe. Each lane owns one op: bucket pointer p, key
// `key`, flag `act`, and the subtable `t` the bucket belongs to. The ops of
// a warp are served in kG rounds; in round q the group of kG lanes g reads
// the bucket of op q*(32/kG)+g, one 32-byte chunk per lane. The group
// combines its per-lane facts with an xor butterfly (log2 kG shuffles) and
// the owner collects them:
//   match / mslot : lowest slot holding `key` (-1 if none) and its content
//   empty         : mask of empty entry slots            (WANT_EMPTY)
//   pref          : mask of slots whose resident's first-probe subtable is
//                   not t, i.e. residents in their second bucket (WANT_PREF)
//   meta          : the bucket's metadata word (0 without one)
// MODE 1 reads through the read-only path (nobody writes the table during
// the kernel), MODE 2 through L2 (other lanes update it with atomics).
// All 32 lanes must call it.
// ----------------------------------------------------------------------------
template <int KB> struct ProbeOut {
    int match;
    typename SlotT<KB>::S mslot;
    unsigned empty, pref;
    unsigned long long meta;
};

// Position of the n-th (0-based) set bit of m; m must have more than n bits.
__host__ __device__ __forceinline__ int nth_set(unsigned m, int n) {
    int pos = 0;
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
        const unsigned low = m & ((1u << w) - 1u);
#ifdef __CUDA_ARCH__
        const int cnt = __popc(low);
#else
        const int cnt = __builtin_popcount(low);
#endif
        if (n >= cnt) {
            n -= cnt;
            m >>= w;
            pos += w;
        } else {
            m = low;
        }
    }
    return pos;
}

template <int G> __device__ __forceinline__ unsigned group_or(unsigned v) {
#pragma unroll
    for (int off = 1; off < G; off <<= 1) v |= __shfl_xor_sync(kFull, v, off);
    return v;
}

// HINT: the bucket reads carry each op's L2 cache policy (pol, see l2_policies)
template <int KB, int SB, int MODE, bool WANT_EMPTY, bool WANT_PREF, bool HINT = false>
__device__ __forceinline__ ProbeOut<KB> probe(const char *p, typename SlotT<KB>::K key, bool act,
                                              uint32_t t, uint32_t d,
                                              unsigned long long pol = 0ull) {
    using T = SlotT<KB>;
    using Sl = typename T::S;
    using K = typename T::K;
    using Gm = Geo<KB, SB>;
    constexpr int G = Gm::kG, RO = Gm::kRoundOps, SPC = Gm::kSPC, WPS = T::kBytes / 4;
    const int lane = threadIdx.x & 31;
    const int g = lane / G, r = lane % G;  // group and chunk this lane serves
    // Active ops are served in compacted order: op with rank c (among the
    // active lanes) is read in round c / RO by group c % RO, so a probe with
    // few active ops costs few rounds.
    const unsigned am = __ballot_sync(kFull, act);
    const bool all = am == kFull;
    const int nact = __popc(am);
    const int rounds = (nact + RO - 1) / RO;
    const int c = all ? lane : __popc(am & ((1u << lane) - 1u));
    const int my_q = act ? c / RO : -1, my_g = c % RO;

    ProbeOut<KB> out;
    out.match = -1;
    out.mslot = T::empty();
    out.empty = 0u;
    out.pref = 0u;
    out.meta = 0ull;
    // one round's loads per batch: fewer registers, more resident warps, and
    // more lines in flight per SM than batching rounds (measured on GB300)
    constexpr int QB = 1;
#pragma unroll 1
    for (int q0 = 0; q0 < rounds; q0 += QB) {
        uint32_t w[QB][8];
        int src[QB];
#pragma unroll
        for (int qq = 0; qq < QB; ++qq) {
            const int ci = (q0 + qq) * RO + g;  // rank of the op this group reads
            const bool have = ci < nact;
            src[qq] = all ? ci : (have ? nth_set(am, ci) : lane);
            const unsigned long long pq = shfl64((unsigned long long)p, src[qq]);
            const unsigned long long polq = HINT ? shfl64(pol, src[qq]) : 0ull;
            if (have) {
                const char *cp = (const char *)pq + r * 32;
                if (HINT) {
                    if (MODE == 1) ld_nc_pol(cp, w[qq], polq);
                    else ld_cg_pol(cp, w[qq], polq);
                } else {
                    if (MODE == 1) ld_nc(cp, w[qq]);
                    else ld_cg(cp, w[qq]);
                }
            } else {
#pragma unroll
                for (int x = 0; x < 8; ++x) w[qq][x] = 0u;
            }
        }
#pragma unroll
        for (int qq = 0; qq < QB; ++qq) {
            const int q = q0 + qq;
            if (q >= rounds) break;  // uniform across the warp
            const bool have = q * RO + g < nact;
            const K kq = (KB == 4) ? (K)__shfl_sync(kFull, (uint32_t)key, src[qq])
                                   : (K)shfl64((unsigned long long)key, src[qq]);
            Sl s[SPC];
#pragma unroll
            for (int j = 0; j < SPC; ++j) T::from_words(w[qq] + j * WPS, s[j]);
            unsigned mb = 0u, eb = 0u, pb = 0u;
            uint32_t tq = 0u, dq = d;
            if (WANT_PREF) {
                // the bucket's owner: its subtable and (for a bucket of
                // another table in a multi-table batch) its subtable count
                tq = __shfl_sync(kFull, t, src[qq]);
                dq = __shfl_sync(kFull, d, src[qq]);
            }
#pragma unroll
            for (int j = 0; j < SPC; ++j) {
                const int idx = r * SPC + j;
                if (idx < Gm::kSlots) {
                    if (T::key(s[j]) == kq) mb |= 1u << idx;
                    if (WANT_EMPTY && T::is_empty(s[j])) eb |= 1u << idx;
                    if (WANT_PREF && !T::is_empty(s[j]) &&
                        pair_of(fold(T::key(s[j])), dq).first != tq)
                        pb |= 1u << idx;
                }
            }
            if (!have) mb = eb = pb = 0u;
            const unsigned gmb = group_or<G>(mb);  // the group's match mask
            // content of the group's lowest matching slot, from the lane holding it
            const int jm = gmb ? __ffs(gmb) - 1 : 0;
            const int lj = jm % SPC;
            Sl sel = s[0];
#pragma unroll
            for (int j = 1; j < SPC; ++j)
                if (j == lj) sel = s[j];
            const Sl gslot = shfl_slot(sel, g * G + jm / SPC);
            // deliver to the owners served in round q (from their group's lead)
            const int lead = my_g * G;
            const unsigned omb = __shfl_sync(kFull, gmb, lead);
            const Sl oslot = shfl_slot(gslot, lead);
            unsigned oe = 0u, op = 0u;
            if (WANT_EMPTY) oe = __shfl_sync(kFull, group_or<G>(eb), lead);
            if (WANT_PREF) op = __shfl_sync(kFull, group_or<G>(pb), lead);
            unsigned long long ometa = 0ull;
            if (Gm::kMeta) {
                uint32_t mw[4];
                T::to_words(s[SPC - 1], mw);
                ometa = shfl64((unsigned long long)mw[0] | ((unsigned long long)mw[1] << 32),
                               lead + G - 1);
            }
            if (my_q == q) {
                if (omb) {
                    out.match = __ffs(omb) - 1;
                    out.mslot = oslot;
                }
                out.empty = oe;
                out.pref = op;
                out.meta = ometa;
            }
        }
    }
    return out;
}

// ----------------------------------------------------------------------------
// Staged probe for find and erase. The buckets of a warp's ops are copied
// into a warp-private shared-memory stage with cp.async (the destination is
// shared memory, so no registers are held while the loads are in flight and
// all rounds are in flight at once); then every lane scans its own bucket.
// Global reads stay line-shaped: in round q the group of kG lanes g copies
// the bucket of op q*(32/kG)+g, lane r the 16-byte pieces r and r+kG, so one
// instruction fetches the first half of 32/kG buckets and the next the
// second half. The 16-byte pieces of a bucket are XOR-swizzled by the
// owner's lane so that the scan's 16-byte shared loads are conflict-free.
// ----------------------------------------------------------------------------
struct KvOut {
    int match;
    uint64_t value;
    bool overflow;
    unsigned empty;  // empty entry slots (probe_staged with WANT_EMPTY)
};

constexpr int kBlockThreads = 256;
constexpr int kWarpsPerBlock = kBlockThreads / 32;

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16_pol(uint32_t dst, const void *src,
                                               unsigned long long pol) {
    asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;" ::"r"(dst),
                 "l"(src), "l"(pol)
                 : "memory");
}

template <int SB> __device__ __forceinline__ uint32_t piece_off(int o, int s) {
    constexpr int P = SB / 16;  // 16-byte pieces per bucket
    return (uint32_t)(o * SB + ((s ^ (o & (P - 1))) * 16));
}

// Copy the bucket at p of every active lane into stage (lane-indexed).
// ALL: every lane is active; otherwise active lanes are served in rank order
// so few active lanes cost few rounds.
template <int SB, bool ALL, bool HINT = false>
__device__ __forceinline__ void stage_rounds(const char *p, unsigned am, unsigned char *stage,
                                             unsigned long long pol = 0ull) {
    constexpr int G = SB / 32, RO = 32 / G;
    const int lane = threadIdx.x & 31, g = lane / G, r = lane % G;
    const int nact = ALL ? 32 : __popc(am);
    const int rounds = ALL ? G : (nact + RO - 1) / RO;
    const uint32_t base = (uint32_t)__cvta_generic_to_shared(stage);
#pragma unroll 1
    for (int q = 0; q < rounds; ++q) {
        const int ci = q * RO + g;
        const bool have = ALL ? true : ci < nact;
        const int o = ALL ? ci : (have ? nth_set(am, ci) : lane);
        const unsigned long long pq = shfl64((unsigned long long)p, o);
        if (HINT) {
            const unsigned long long polq = shfl64(pol, o);
            if (have) {
                cp_async16_pol(base + piece_off<SB>(o, r), (const char *)pq + r * 16, polq);
                cp_async16_pol(base + piece_off<SB>(o, r + G), (const char *)pq + (r + G) * 16,
                               polq);
            }
        } else if (have) {
            cp_async16(base + piece_off<SB>(o, r), (const char *)pq + r * 16);
            cp_async16(base + piece_off<SB>(o, r + G), (const char *)pq + (r + G) * 16);
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncwarp();  // other lanes' copies are visible after the warp barrier
}

template <int KB, int SB, bool WANT_EMPTY = false, bool HINT = false>
__device__ __forceinline__ KvOut probe_staged(const char *p, typename SlotT<KB>::K key, bool act,
                                              unsigned char *stage,
                                              unsigned long long pol = 0ull) {
    using T = SlotT<KB>;
    using Gm = Geo<KB, SB>;
    constexpr int P = SB / 16, SPP = 16 / T::kBytes > 0 ? 16 / T::kBytes : 1;
    const unsigned am = __ballot_sync(kFull, act);
    __syncwarp();  // the previous use of the stage is finished in every lane
    if (am == kFull) stage_rounds<SB, true, HINT>(p, am, stage, pol);
    else if (am) stage_rounds<SB, false, HINT>(p, am, stage, pol);
    KvOut out{-1, 0ull, false, 0u};
    if (!act) return out;
    const int lane = threadIdx.x & 31;
    const uint32_t base = (uint32_t)__cvta_generic_to_shared(stage);
#pragma unroll
    for (int s = 0; s < P; ++s) {
        uint32_t v[4];
        asm volatile("ld.shared.v4.u32 {%0,%1,%2,%3}, [%4];"
                     : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
                     : "r"(base + piece_off<SB>(lane, s)));
#pragma unroll
        for (int j = 0; j < SPP; ++j) {
            const int idx = s * SPP + j;
            typename T::S sl;
            T::from_words(v + j * (T::kBytes / 4), sl);
            if (idx < Gm::kSlots) {
                if (out.match < 0 && T::key(sl) == key) {
                    out.match = idx;
                    out.value = T::val(sl);
                }
                if (WANT_EMPTY && T::is_empty(sl)) out.empty |= 1u << idx;
            } else if (Gm::kMeta && idx == Gm::kTotal - 1) {
                const unsigned long long meta = (unsigned long long)v[j * (T::kBytes / 4)] |
                                                ((unsigned long long)v[j * (T::kBytes / 4) + 1] << 32);
                out.overflow = (meta & fp_bit(fold(key))) != 0ull;  // key's fingerprint
            }
        }
    }
    return out;
}

// Key/value probe used by find and erase: staged for 64- and 128-byte
// buckets; 32-byte buckets (one lane per bucket, a single 256-bit load) read
// straight into registers, since staging them would split each sector over
// two 16-byte copies.
template <int KB, int SB, int MODE, bool HINT = false>
__device__ __forceinline__ KvOut kv_probe(const char *p, typename SlotT<KB>::K key, bool act,
                                          unsigned char *stage, unsigned long long pol = 0ull) {
    if constexpr (SB >= 64) {
        return probe_staged<KB, SB, false, HINT>(p, key, act, stage, pol);
    } else {
        const ProbeOut<KB> r = probe<KB, SB, MODE, false, false, HINT>(p, key, act, 0u, 0u, pol);
        KvOut o;
        o.match = r.match;
        o.value = SlotT<KB>::val(r.mslot);
        o.overflow = false;
        o.empty = 0u;
        return o;
    }
}

// Probe used by insert placement: matching slot, empty entry slots and the
// overflow bit, through the shared-memory stage for 64- and 128-byte buckets
// (a coherent L2 snapshot: cp.async.cg), the register probe for 32-byte ones.
template <int KB, int SB, bool HINT = false>
__device__ __forceinline__ KvOut place_probe(const char *p, typename SlotT<KB>::K key, bool act,
                                             uint32_t t, uint32_t d, unsigned char *stage,
                                             unsigned long long pol = 0ull) {
    if constexpr (SB >= 64) {
        return probe_staged<KB, SB, true, HINT>(p, key, act, stage, pol);
    } else {
        const ProbeOut<KB> r = probe<KB, SB, 2, true, false, HINT>(p, key, act, t, d, pol);
        KvOut o;
        o.match = r.match;
        o.value = SlotT<KB>::val(r.mslot);
        o.overflow = (r.meta & fp_bit(fold(key))) != 0ull;
        o.empty = r.empty;
        return o;
    }
}

// ----------------------------------------------------------------------------
// Batch dedup: an open-addressing scratch table maps each key of the batch to
// its last (insert) or first (erase) op index.
// ----------------------------------------------------------------------------
template <int KB> struct Dedup;

template <> struct Dedup<4> {
    // one 64-bit cell: key << 32 | op index; 0 = free
    __device__ static __forceinline__ void claim(const Scratch &S, uint32_t k, uint32_t i,
                                                 DedupMode mode) {
        unsigned long long *tab = (unsigned long long *)S.dedup;
        const uint64_t mask = S.dedup_cap - 1;
        const unsigned long long mine = ((unsigned long long)k << 32) | i;
        uint64_t h = mix32(k) & mask;
        for (uint64_t probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
            unsigned long long old = atomicCAS(&tab[h], 0ull, mine);
            if (old == 0ull) return;
            if ((uint32_t)(old >> 32) == k) {
                if (mode == kKeepLast) atomicMax(&tab[h], mine);
                else atomicMin(&tab[h], mine);
                if (S.dupseen) *(volatile uint32_t *)S.dupseen = 1u;
                return;
            }
        }
    }
    __device__ static __forceinline__ bool winner(const Scratch &S, uint32_t k, uint32_t i) {
        if (S.dupseen && *S.dupseen == 0u) return true;  // no key repeats in the chunk
        if (winners_pass(S)) return (S.winbits[i >> 5] >> (i & 31)) & 1u;
        const unsigned long long *tab = (const unsigned long long *)S.dedup;
        const uint64_t mask = S.dedup_cap - 1;
        uint64_t h = mix32(k) & mask;
        for (uint64_t probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
            unsigned long long c = tab[h];
            if (c == 0ull) return false;
            if ((uint32_t)(c >> 32) == k) return (uint32_t)c == i;
        }
        return false;
    }
};

template <> struct Dedup<8> {
    // key array + op-index array; key 0 = free
    __device__ static __forceinline__ void claim(const Scratch &S, uint64_t k, uint32_t i,
                                                 DedupMode mode) {
        unsigned long long *tab = (unsigned long long *)S.dedup;
        const uint64_t mask = S.dedup_cap - 1;
        uint64_t h = mix32(fold(k) ^ (uint32_t)(k >> 32)) & mask;
        for (uint64_t probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
            unsigned long long old = atomicCAS(&tab[h], 0ull, (unsigned long long)k);
            if (old == 0ull || old == k) {
                if (mode == kKeepLast) atomicMax(&S.dedup_idx[h], i);
                else atomicMin(&S.dedup_idx[h], i);
                if (old == k && S.dupseen) *(volatile uint32_t *)S.dupseen = 1u;
                return;
            }
        }
    }
    __device__ static __forceinline__ bool winner(const Scratch &S, uint64_t k, uint32_t i) {
        if (S.dupseen && *S.dupseen == 0u) return true;  // no key repeats in the chunk
        if (winners_pass(S)) return (S.winbits[i >> 5] >> (i & 31)) & 1u;
        const unsigned long long *tab = (const unsigned long long *)S.dedup;
        const uint64_t mask = S.dedup_cap - 1;
        uint64_t h = mix32(fold(k) ^ (uint32_t)(k >> 32)) & mask;
        for (uint64_t probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
            unsigned long long c = tab[h];
            if (c == 0ull) return false;
            if (c == k) return S.dedup_idx[h] == i;
        }
        return false;
    }
};

// Clears one chunk's dedup state in one launch: the key cells (16-byte
// stores; dedup_cap is a power of two >= 32 and the cells are 256-byte
// aligned), the op-index cells of 8-byte keys (to idx_fill), win_words
// winner-bit words, the repeat flag, and nzero 64-bit words at zero.
template <int KB>
__global__ void __launch_bounds__(256) k_dedup_clear(const __grid_constant__ Scratch S,
                                                     uint32_t idx_fill, uint64_t win_words,
                                                     unsigned long long *zero, uint32_t nzero) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint4 *cells = (uint4 *)S.dedup;
    const uint64_t n16 = S.dedup_cap / 2;  // two 8-byte cells per store
    for (uint64_t i = tid; i < n16; i += stride) cells[i] = make_uint4(0u, 0u, 0u, 0u);
    if (KB == 8 && S.dedup_idx != nullptr) {
        uint4 *ix = (uint4 *)S.dedup_idx;
        const uint4 f = make_uint4(idx_fill, idx_fill, idx_fill, idx_fill);
        for (uint64_t i = tid; i < S.dedup_cap / 4; i += stride) ix[i] = f;
    }
    if (S.winbits != nullptr)
        for (uint64_t i = tid; i < win_words; i += stride) S.winbits[i] = 0u;
    if (tid == 0 && S.dupseen != nullptr) *S.dupseen = 0u;
    if (tid < nzero) zero[tid] = 0ull;
}

template <int KB>
__global__ void __launch_bounds__(256) k_dedup(const __grid_constant__ Scratch S,
                                               const void *__restrict__ keys, uint64_t n,
                                               DedupMode mode) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        typename SlotT<KB>::K k = load_key<KB>(keys, i);
        if (k != 0) Dedup<KB>::claim(S, k, (uint32_t)i, mode);
    }
}

// After the claims: one pass over the dedup cells (sequential reads) sets
// the winner bit of the op each used cell names (L2 atomics into a bitmap of
// n bits), so the place and erase kernels read their op's bit coalesced
// instead of probing the dedup table at random once more (the table of a
// 4M-op chunk is 64 MB; those probes cost DRAM accesses beside the bucket
// reads). A chunk whose claims met no key twice skips the pass: every op
// wins (dupseen).
template <int KB>
__global__ void __launch_bounds__(256) k_dedup_winners(const __grid_constant__ Scratch S) {
    if (S.dupseen && *S.dupseen == 0u) return;  // every op is its key's only one
    const unsigned long long *tab = (const unsigned long long *)S.dedup;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t h = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; h < S.dedup_cap;
         h += stride) {
        const unsigned long long c = tab[h];
        if (c == 0ull) continue;
        const uint32_t i = KB == 4 ? (uint32_t)c : S.dedup_idx[h];
        atomicOr(&S.winbits[i >> 5], 1u << (i & 31));
    }
}

// ----------------------------------------------------------------------------
// find (cuckoo_search, cuckoo.cu:460-520): probe the first-probe bucket; probe
// the second one only on a miss whose first bucket has its overflow bit set
// (32/64-byte buckets carry no metadata and always probe both on a miss).
// Writes the value (0 on a miss) and one hit bit per key. (Queueing second
// probes per warp, or prefetching the next tile's keys, measured slower.)
// Five resident blocks per SM for 4-byte keys (48 registers, a 16-byte
// spill): +1.7 % on uniform hits at 2^28 keys, 10 %-hit finds unchanged;
// six blocks and larger or smaller tiles per block measured no better.
// HINT (a table that keeps its lines in the L2, Desc::l2_keep): loads and
// stores carry L2 eviction-priority hints. Other tables use plain accesses:
// hinted loads of a line many warps read at once (the hot keys of a Zipf
// batch) measured 2.5x slower than plain ones (15.6 vs 39.4 G finds/s at
// Zipf 0.99 on 2^28 keys; uniform 39.3 vs 40.4).
// ----------------------------------------------------------------------------
template <int KB, int SB, bool HINT>
__global__ void __launch_bounds__(256, KB == 4 ? 5 : 1) k_find(const __grid_constant__ Desc D,
                                              const void *__restrict__ keys,
                                              void *__restrict__ vals, uint32_t vb,
                                              uint32_t *__restrict__ hits, uint64_t n) {
    using T = SlotT<KB>;
    using Gm = Geo<KB, SB>;
    __shared__ __align__(128) unsigned char s_stage[kWarpsPerBlock][32 * SB];
    unsigned char *stage = s_stage[threadIdx.x >> 5];
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t step = warp_stride();
    L2Pol pol{0ull, 0ull};
    if constexpr (HINT) pol = l2_policies(true);
    for (uint64_t base = warp_base(); base < n; base += step) {
        const uint64_t i = base + lane;
        typename T::K k = 0;
        if (i < n) {
            if constexpr (HINT) k = load_key_pol<KB>(keys, i, pol.stream);
            else k = load_key<KB>(keys, i);
        }
        const bool act = k != 0;
        const uint32_t hk = fold(k);
        const Pair p = pair_of(hk, D.d);
        const char *p1 = bucket_ptr<KB, SB>(D, p.first, bucket_index(D, p.first, hk));
        const KvOut r1 = kv_probe<KB, SB, 1, HINT>(p1, k, act, stage, pol.table);
        bool hit = act && r1.match >= 0;
        uint64_t v = hit ? r1.value : 0ull;
        const bool need2 = act && !hit && (!Gm::kMeta || r1.overflow);
        if (__any_sync(kFull, need2)) {
            const char *p2 = bucket_ptr<KB, SB>(D, p.second, bucket_index(D, p.second, hk));
            const KvOut r2 = kv_probe<KB, SB, 1, HINT>(p2, k, need2, stage, pol.table);
            if (need2 && r2.match >= 0) {
                hit = true;
                v = r2.value;
            }
        }
        const unsigned m = __ballot_sync(kFull, hit);
        if constexpr (HINT) {
            if (i < n) store_val_pol(vals, vb, i, v, pol.stream);
            if (hits != nullptr && lane == 0) store_u32_pol(hits + (base >> 5), m, pol.stream);
        } else {
            if (i < n) store_val(vals, vb, i, v);
            if (hits != nullptr && lane == 0) hits[base >> 5] = m;
        }
    }
}

// ----------------------------------------------------------------------------
// insert phase 2: update present keys in place, else claim an empty slot in
// the first-probe bucket, else in the second (marking the first bucket's
// overflow bit first); ops left without a slot go to list_a.
// ----------------------------------------------------------------------------
template <int KB, int SB, bool HINT>
__global__ void __launch_bounds__(256) k_place(const __grid_constant__ Desc D,
                                               const __grid_constant__ Scratch S, int use_dedup,
                                               int new_keys, const void *__restrict__ keys,
                                               const void *__restrict__ vals, uint32_t vb,
                                               uint64_t n, Counters *ctr) {
    using T = SlotT<KB>;
    using Sl = typename T::S;
    using Gm = Geo<KB, SB>;
    __shared__ __align__(128) unsigned char s_stage[SB >= 64 ? kWarpsPerBlock : 1][32 * SB];
    unsigned char *stage = s_stage[SB >= 64 ? (threadIdx.x >> 5) : 0];
    const uint64_t step = warp_stride();
    const unsigned long long tpol = HINT ? l2_policies(true).table : 0ull;
    uint32_t n_ins = 0, n_upd = 0, n_rej = 0, n_sup = 0;
    for (uint64_t base = warp_base(); base < n; base += step) {
        const uint64_t i = base + (threadIdx.x & 31);
        typename T::K k = 0;
        bool act = false;
        Sl e = T::empty();
        if (i < n) {
            k = load_key<KB>(keys, i);
            if (k == 0) {
                ++n_rej;
            } else if (use_dedup && !Dedup<KB>::winner(S, k, (uint32_t)i)) {
                ++n_sup;
            } else {
                act = true;
                e = T::make(k, load_val(vals, vb, i));
            }
        }
        const uint32_t hk = fold(k);
        const Pair p = pair_of(hk, D.d);
        char *p1 = bucket_ptr<KB, SB>(D, p.first, bucket_index(D, p.first, hk));
        char *p2 = bucket_ptr<KB, SB>(D, p.second, bucket_index(D, p.second, hk));
        const KvOut r1 = place_probe<KB, SB, HINT>(p1, k, act, p.first, D.d, stage, tpol);
        const bool found1 = act && r1.match >= 0;
        // the second bucket is needed to look for the key (upsert, unless the
        // first bucket's overflow bit rules it out) or for an empty slot
        const bool check2 =
            act && !found1 && ((!new_keys && (!Gm::kMeta || r1.overflow)) || r1.empty == 0u);
        KvOut r2{-1, 0ull, false, 0u};
        if (__any_sync(kFull, check2))
            r2 = place_probe<KB, SB, HINT>(p2, k, check2, p.second, D.d, stage, tpol);
        // An update rewrites the key's own slot with a plain store: the keys
        // of the kernel are distinct (dedup, or the caller's promise) and
        // its other writes only claim empty slots, so nothing else writes
        // that slot while the kernel runs (a store does not wait for an L2
        // round trip as an exchange does).
        bool pend = false;
        if (found1) {
            T::store(slot_ptr<KB, SB>(p1, r1.match), e);
            ++n_upd;
        } else if (check2 && !new_keys && r2.match >= 0) {
            T::store(slot_ptr<KB, SB>(p2, r2.match), e);
            ++n_upd;
        } else if (act) {
            bool ok = claim_empty<KB, SB>(p1, r1.empty, e);
            if (!ok && check2 && r2.empty) {
                mark_overflow<KB, SB>(p1, hk);
                ok = claim_empty<KB, SB>(p2, r2.empty, e);
            }
            if (ok) ++n_ins;
            else pend = true;
        }
        __syncwarp();
        const unsigned long long at = agg_inc(&ctr->pending, pend);
        if (pend) {
            if (at < S.list_cap) ((Sl *)S.list_a)[at] = e;
            else atomicAdd(&ctr->spill, 1ull);
        }
    }
    // one atomic per counter per block (the grid has many short-lived blocks)
    __shared__ unsigned long long s_sum[4];
    if (threadIdx.x < 4) s_sum[threadIdx.x] = 0ull;
    __syncthreads();
    const uint32_t w_ins = __reduce_add_sync(kFull, n_ins), w_upd = __reduce_add_sync(kFull, n_upd);
    const uint32_t w_rej = __reduce_add_sync(kFull, n_rej), w_sup = __reduce_add_sync(kFull, n_sup);
    if ((threadIdx.x & 31) == 0) {
        if (w_ins) atomicAdd(&s_sum[0], (unsigned long long)w_ins);
        if (w_upd) atomicAdd(&s_sum[1], (unsigned long long)w_upd);
        if (w_rej) atomicAdd(&s_sum[2], (unsigned long long)w_rej);
        if (w_sup) atomicAdd(&s_sum[3], (unsigned long long)w_sup);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_sum[0]) {
            atomicAdd(&ctr->inserted, s_sum[0]);
            atomicAdd(&ctr->size, s_sum[0]);
        }
        if (s_sum[1]) atomicAdd(&ctr->updated, s_sum[1]);
        if (s_sum[2]) atomicAdd(&ctr->rejected, s_sum[2]);
        if (s_sum[3]) atomicAdd(&ctr->superseded, s_sum[3]);
    }
}

// Victim when a bucket is full: prefer a resident sitting in its second
// bucket (evicting it sends it back to its first-probe bucket); the start
// is a pseudo-random slot (victim_rot, mixed from the key and the step). The
// preference holds for the first kPrefSteps steps of a chain (victim_pref):
// a cluster of full buckets whose second-bucket residents all point at each
// other can trap a walk that always takes them (at load 0.94 on 7-slot
// buckets some walks ran out all 2048 steps), so a chain that long walks at
// random. (Dropping the preference after 4 steps cost 32-byte buckets a
// tenth of their first-probe hits.)
constexpr uint32_t kPrefSteps = 32;
__device__ __forceinline__ uint32_t victim_rot(uint32_t hk, uint32_t step) {
    return mix32(hk ^ (step * 0x9E3779B9u));
}
__device__ __forceinline__ unsigned victim_pref(unsigned pref, uint32_t step) {
    return step < kPrefSteps ? pref : 0u;
}
template <int KB, int SB>
__device__ __forceinline__ int pick_victim(unsigned pref, uint32_t rot) {
    constexpr int B = Geo<KB, SB>::kSlots;
    rot %= (uint32_t)B;
    if (!pref) return (int)rot;
    const unsigned all = (B == 32) ? kFull : ((1u << B) - 1u);
    const unsigned rotated = ((pref >> rot) | (pref << ((B - rot) & 31))) & all;
    return (int)((__ffs(rotated) - 1 + rot) % (uint32_t)B);
}


// ----------------------------------------------------------------------------
// Eviction walk with one-level lookahead, one entry per warp. A plain walk
// exchanges the entry into its full bucket and carries the resident to that
// resident's other bucket, which is full again with the probability of the
// load factor, so the longest of a batch's chains (a dozen steps of
// dependent memory round trips at load 0.8) sets the walk kernel's time.
// Here the warp reads the full bucket, then the other buckets of all its
// residents at once (group g of kG lanes reads resident g's, kRoundOps per
// round), and evicts a resident whose other bucket has an empty slot: that
// resident is placed by the next atomic, and a chain rarely needs a second
// level. Without such a resident it evicts as the plain walk does (a
// resident in its second bucket first). The same atomics as the plain walk
// keep concurrent walks safe: an exchange hands the warp whatever was in the
// slot, a claim succeeds only on a slot still empty, and the lookahead only
// guides the choice.
// Returns whether the carried entry was placed, the exchanges made and, if
// not placed, the entry carried at the end (the caller re-places it).
// Walk kernels switch to cooperative probing of 32 entries per warp when the
// list holds more than this many entries per warp of the grid.
constexpr int kCoopWalk = 4;

template <int KB> struct WalkOut {
    bool ok;
    uint32_t steps;
    typename SlotT<KB>::S left;
};

template <int KB, int SB>
__device__ __forceinline__ WalkOut<KB> walk_lookahead(const Desc &D, typename SlotT<KB>::S e,
                                                      uint32_t max_evict) {
    using T = SlotT<KB>;
    using Sl = typename T::S;
    using K = typename T::K;
    using Gm = Geo<KB, SB>;
    constexpr int G = Gm::kG, RO = Gm::kRoundOps, NS = Gm::kSlots;
    constexpr int LR = (NS + RO - 1) / RO;  // lookahead rounds
    const int lane = threadIdx.x & 31, g = lane / G, r = lane % G;
    uint32_t hk;
    Pair pe;
    char *fb = first_bucket<KB, SB>(D, T::key(e), pe, hk);
    uint32_t t = pe.first;
    char *bp = fb;
    uint32_t steps = 0;
    for (uint32_t level = 0; level <= max_evict; ++level) {
        Bucket<KB, SB> B;
        B.template load<2>(bp);  // every lane: the same lines, one request
        const unsigned em = B.empty_mask();
        if (em) {
            bool ok = false;
            if (lane == 0) {
                if (t != pe.first) mark_overflow<KB, SB>(fb, hk);
                ok = claim_empty<KB, SB>(bp, em, e);
            }
            if (__shfl_sync(kFull, ok, 0)) return {true, steps, T::empty()};
            continue;  // the slots were taken meanwhile: read again
        }
        if (level == max_evict) break;
        // lookahead: resident j = q * RO + g's other bucket, chunk r per lane
        unsigned cand = 0u, pref = 0u;
        char *alt[LR];
        unsigned alt_em[LR];
#pragma unroll
        for (int q = 0; q < LR; ++q) {
            const int j = q * RO + g;
            K kj = 0;
#pragma unroll
            for (int x = 0; x < NS; ++x)
                if (x == j) kj = T::key(B.s[x]);
            const uint32_t hj = fold(kj);
            const Pair pj = pair_of(hj, D.d);
            const uint32_t tj = other_of(pj, t);
            alt[q] = bucket_ptr<KB, SB>(D, tj, bucket_index(D, tj, hj));
            unsigned m = 0u;
            if (j < NS) {
                uint32_t w[8];
                ld_cg(alt[q] + r * 32, w);
                constexpr int SPC = Gm::kSPC, WPS = T::kBytes / 4;
#pragma unroll
                for (int x = 0; x < SPC; ++x) {
                    Sl sx;
                    T::from_words(w + x * WPS, sx);
                    const int idx = r * SPC + x;
                    if (idx < NS && T::is_empty(sx)) m |= 1u << idx;
                }
            }
#pragma unroll
            for (int o = 1; o < G; o <<= 1) m |= __shfl_xor_sync(kFull, m, o);
            alt_em[q] = m;
            const unsigned have = __ballot_sync(kFull, r == 0 && j < NS && m != 0u);
            const unsigned second = __ballot_sync(kFull, r == 0 && j < NS && pj.first != t);
#pragma unroll
            for (int x = 0; x < RO; ++x) {
                if (q * RO + x >= NS) break;
                cand |= ((have >> (x * G)) & 1u) << (q * RO + x);
                pref |= ((second >> (x * G)) & 1u) << (q * RO + x);
            }
        }
        const int j = cand ? pick_victim<KB, SB>(cand, hk + level)
                           : pick_victim<KB, SB>(victim_pref(pref, level), victim_rot(hk, level));
        const int src = (j % RO) * G;
        char *aj = nullptr;
        unsigned aem = 0u;
#pragma unroll
        for (int q = 0; q < LR; ++q) {
            char *a = (char *)shfl64((unsigned long long)alt[q], src);
            const unsigned am = __shfl_sync(kFull, alt_em[q], src);
            if (q == j / RO) {
                aj = a;
                aem = am;
            }
        }
        K kj = 0;
#pragma unroll
        for (int x = 0; x < NS; ++x)
            if (x == j) kj = T::key(B.s[x]);
        // exchange the carried entry into slot j
        Sl old = T::empty();
        if (lane == 0) {
            if (t != pe.first) mark_overflow<KB, SB>(fb, hk);
            old = T::exch(slot_ptr<KB, SB>(bp, j), e);
        }
        old = shfl_slot(old, 0);
        ++steps;
        if (T::is_empty(old)) return {true, steps, T::empty()};
        // carry the resident to its other bucket
        e = old;
        const uint32_t from = t;
        fb = first_bucket<KB, SB>(D, T::key(e), pe, hk);
        t = other_of(pe, from);
        bp = bucket_ptr<KB, SB>(D, t, bucket_index(D, t, hk));
        if (((cand >> j) & 1u) && T::key(old) == kj) {  // bp == aj: its empty slots are known
            bool ok = false;
            if (lane == 0) {
                if (t != pe.first) mark_overflow<KB, SB>(fb, hk);
                ok = claim_empty<KB, SB>(aj, aem, e);
            }
            if (__shfl_sync(kFull, ok, 0)) return {true, steps, T::empty()};
        }
    }
    return {false, steps, e};
}

// ----------------------------------------------------------------------------
// insert phase 3: eviction walks (warp_insert, cuckoo.cu:365-432). The
// reference walks one entry per thread: exchange into the current bucket,
// carry the resident to the other bucket of its own pair. Here each entry of
// `src` is walked by a whole warp with one-level lookahead (walk_lookahead):
// the first-probe bucket's empty slots first, then an exchange that
// preferably evicts a resident whose other bucket has room. An entry whose
// walk reaches max_evict exchanges goes to `dst` for the host to place after
// an upsize.
// ----------------------------------------------------------------------------
template <int KB, int SB>
__global__ void __launch_bounds__(256) k_walk(const __grid_constant__ Desc D,
                                              const void *__restrict__ src,
                                              const unsigned long long *src_count, void *dst,
                                              unsigned long long *dst_count, uint64_t dst_cap,
                                              uint32_t max_evict, int count_new, Counters *ctr,
                                              uint64_t max_entries) {
    using T = SlotT<KB>;
    using Sl = typename T::S;
    __shared__ unsigned long long s_sum[2];
    if (threadIdx.x < 2) s_sum[threadIdx.x] = 0ull;
    __syncthreads();
    uint64_t n = *src_count;
    if (n > max_entries) n = max_entries;
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t wid = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    const bool lead = lane == 0;
    uint32_t n_ok = 0, n_steps = 0;
    if (n > (uint64_t)kCoopWalk * warps) {
        // long list: 32 entries per warp, probed cooperatively (throughput)
        const uint32_t max_iter = 2u * max_evict + 8u;
        for (uint64_t base = wid * 32; base < n; base += warps * 32) {
            const uint64_t i = base + lane;
            bool live = i < n;
            Sl e = live ? ((const Sl *)src)[i] : T::empty();
            uint32_t hk = 0;
            Pair pe{0u, 0u};
            char *fb = first_bucket<KB, SB>(D, T::key(e), pe, hk);  // first bucket of e
            uint32_t t = pe.first;
            char *bp = fb;
            int mode = 0;  // 0: empties of the first bucket, 1: of the second, 2: walking
            uint32_t evictions = 0;
            bool fail = false;
            for (uint32_t it = 0; it < max_iter; ++it) {
                if (!__any_sync(kFull, live)) break;
                const ProbeOut<KB> r = probe<KB, SB, 2, true, true>(bp, T::key(e), live, t, D.d);
                if (!live) continue;
                bool placed = false;
                if (r.empty) {
                    if (t != pe.first) mark_overflow<KB, SB>(fb, hk);
                    placed = claim_empty<KB, SB>(bp, r.empty, e);
                }
                if (placed) {
                    live = false;
                    ++n_ok;
                } else if (mode == 0) {
                    mode = 1;
                    t = pe.second;
                    bp = bucket_ptr<KB, SB>(D, t, bucket_index(D, t, hk));
                } else if (mode == 1) {
                    mode = 2;
                    t = pe.first;
                    bp = fb;
                } else if (r.empty) {
                    // every empty slot was taken by another lane: look again
                } else if (evictions >= max_evict) {
                    live = false;
                    fail = true;
                } else {
                    const int j = pick_victim<KB, SB>(victim_pref(r.pref, evictions),
                                                      victim_rot(hk, evictions));
                    if (t != pe.first) mark_overflow<KB, SB>(fb, hk);
                    const Sl old = T::exch(slot_ptr<KB, SB>(bp, j), e);
                    ++evictions;
                    ++n_steps;
                    if (T::is_empty(old)) {
                        live = false;
                        ++n_ok;
                    } else {
                        e = old;
                        fb = first_bucket<KB, SB>(D, T::key(e), pe, hk);
                        t = other_of(pe, t);
                        bp = bucket_ptr<KB, SB>(D, t, bucket_index(D, t, hk));
                    }
                }
            }
            if (live) fail = true;  // iteration bound reached
            __syncwarp();
            const unsigned long long at = agg_inc(dst_count, fail);
            if (fail) {
                if (at < dst_cap) ((Sl *)dst)[at] = e;
                else atomicAdd(&ctr->spill, 1ull);
            }
        }
    } else {
        for (uint64_t i = wid; i < n; i += warps) {
            const WalkOut<KB> w = walk_lookahead<KB, SB>(D, ((const Sl *)src)[i], max_evict);
            if (!lead) continue;
            n_steps += w.steps;
            if (w.ok) {
                ++n_ok;
            } else {
                const unsigned long long at = atomicAdd(dst_count, 1ull);
                if (at < dst_cap) ((Sl *)dst)[at] = w.left;
                else atomicAdd(&ctr->spill, 1ull);
            }
        }
    }
    n_ok = __reduce_add_sync(kFull, n_ok);
    n_steps = __reduce_add_sync(kFull, n_steps);
    if (lead && (n_ok | n_steps)) {
        atomicAdd(&s_sum[0], (unsigned long long)n_ok);
        atomicAdd(&s_sum[1], (unsigned long long)n_steps);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (count_new && s_sum[0]) {
            atomicAdd(&ctr->inserted, s_sum[0]);
            atomicAdd(&ctr->size, s_sum[0]);
        }
        if (s_sum[1]) atomicAdd(&ctr->evict_steps, s_sum[1]);
    }
}

// ----------------------------------------------------------------------------
// erase (cuckoo_delete, cuckoo.cu:524-587): the slot holding the key is
// cleared with a CAS; the second bucket is only probed when the first one's
// overflow bit allows the key to be there.
// ----------------------------------------------------------------------------
template <int KB, int SB, bool HINT>
__global__ void __launch_bounds__(256) k_erase(const __grid_constant__ Desc D,
                                               const __grid_constant__ Scratch S, int use_dedup,
                                               const void *__restrict__ keys, uint64_t n,
                                               uint32_t *__restrict__ bits, Counters *ctr) {
    using T = SlotT<KB>;
    using Gm = Geo<KB, SB>;
    __shared__ __align__(128) unsigned char s_stage[kWarpsPerBlock][32 * SB];
    unsigned char *stage = s_stage[threadIdx.x >> 5];
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t step = warp_stride();
    const unsigned long long tpol = HINT ? l2_policies(true).table : 0ull;
    uint32_t n_del = 0, n_sup = 0;
    for (uint64_t base = warp_base(); base < n; base += step) {
        const uint64_t i = base + lane;
        typename T::K k = 0;
        bool act = false;
        if (i < n) {
            k = load_key<KB>(keys, i);
            if (k != 0) {
                if (use_dedup && !Dedup<KB>::winner(S, k, (uint32_t)i)) ++n_sup;
                else act = true;
            }
        }
        const uint32_t hk = fold(k);
        const Pair p = pair_of(hk, D.d);
        char *p1 = bucket_ptr<KB, SB>(D, p.first, bucket_index(D, p.first, hk));
        const KvOut r1 = kv_probe<KB, SB, 2, HINT>(p1, k, act, stage, tpol);
        // A found key's slot is emptied with a plain store, as the reference
        // does (cuckoo.cu:551): the kernel's keys are distinct (dedup, or the
        // caller's promise) and nothing else runs on the table, so no other
        // thread writes that slot; the store does not wait on an L2 round
        // trip as a compare-and-swap does.
        bool erased = false;
        if (act && r1.match >= 0) {
            T::store(slot_ptr<KB, SB>(p1, r1.match), T::empty());
            erased = true;
        }
        const bool need2 = act && r1.match < 0 && (!Gm::kMeta || r1.overflow);
        if (__any_sync(kFull, need2)) {
            char *p2 = bucket_ptr<KB, SB>(D, p.second, bucket_index(D, p.second, hk));
            const KvOut r2 = kv_probe<KB, SB, 2, HINT>(p2, k, need2, stage, tpol);
            if (need2 && r2.match >= 0) {
                T::store(slot_ptr<KB, SB>(p2, r2.match), T::empty());
                erased = true;
            }
        }
        const unsigned m = __ballot_sync(kFull, erased);
        if (bits != nullptr && lane == 0) bits[base >> 5] = m;
        n_del += erased ? 1u : 0u;
    }
    // loops are warp-uniform, so every lane of the warp is here; one atomic
    // per counter per block (the grid has many short-lived blocks)
    __shared__ unsigned long long s_sum[2];
    if (threadIdx.x < 2) s_sum[threadIdx.x] = 0ull;
    __syncthreads();
    const uint32_t del = __reduce_add_sync(kFull, n_del);
    const uint32_t sup = __reduce_add_sync(kFull, n_sup);
    if (lane == 0) {
        if (del) atomicAdd(&s_sum[0], (unsigned long long)del);
        if (sup) atomicAdd(&s_sum[1], (unsigned long long)sup);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_sum[0]) {
            atomicAdd(&ctr->erased, s_sum[0]);
            atomicAdd(&ctr->size, (unsigned long long)(-(long long)s_sum[0]));  // size -= erased
        }
        if (s_sum[1]) atomicAdd(&ctr->superseded, s_sum[1]);
    }
}

// ----------------------------------------------------------------------------
// upsize: subtable t goes from nb to 2nb buckets. hash % 2nb of an entry in
// old bucket b is b or b+nb, so every slot keeps its index and each old
// bucket writes exactly two new buckets: a pure stream, read S / write 2S,
// no zero-fill pass and no atomics (cuckoo_resize_up, cuckoo.cu:600-627).
// One thread per 32-byte chunk; the metadata word is copied to both halves
// (keys displaced from old bucket b now have b or b+nb as first bucket).
// ----------------------------------------------------------------------------
// Chunks x0, x0 + step, ... below x1 of old subtable t (old_nb buckets) into
// their low and high images in new_sub (2 * old_nb buckets, fastmod
// reciprocal new_magic).
template <int KB, int SB>
__device__ __forceinline__ void upsize_chunks(uint32_t t, const char *__restrict__ old_sub,
                                              uint32_t old_nb, char *__restrict__ new_sub,
                                              uint64_t new_magic, uint64_t x0, uint64_t x1,
                                              uint64_t step) {
    using T = SlotT<KB>;
    using Gm = Geo<KB, SB>;
    constexpr int G = Gm::kG, SPC = Gm::kSPC, WPS = T::kBytes / 4;
    const uint32_t new_nb = 2u * old_nb;
    for (uint64_t x = x0; x < x1; x += step) {
        const uint64_t b = x / G;
        const int r = (int)(x % G);
        uint32_t w[8], lo[8], hi[8];
        ld_nc(old_sub + x * 32, w);
#pragma unroll
        for (int j = 0; j < SPC; ++j) {
            typename T::S s;
            T::from_words(w + j * WPS, s);
            const int idx = r * SPC + j;
            const bool is_meta = Gm::kMeta && idx == Gm::kTotal - 1;
            bool to_lo = is_meta, to_hi = is_meta;
            if (!is_meta && !T::is_empty(s)) {
                const uint32_t nbk = fastmod(subtable_hash(fold(T::key(s)), t), new_magic, new_nb);
                to_lo = nbk == (uint32_t)b;
                to_hi = !to_lo;
            }
#pragma unroll
            for (int x2 = 0; x2 < WPS; ++x2) {
                lo[j * WPS + x2] = to_lo ? w[j * WPS + x2] : 0u;
                hi[j * WPS + x2] = to_hi ? w[j * WPS + x2] : 0u;
            }
        }
        st_v8(new_sub + b * SB + r * 32, lo);
        st_v8(new_sub + (b + old_nb) * SB + r * 32, hi);
    }
}

template <int KB, int SB>
__global__ void __launch_bounds__(256) k_resize_up(uint32_t t, const char *__restrict__ old_sub,
                                                   uint32_t old_nb, char *__restrict__ new_sub,
                                                   uint64_t new_magic) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    upsize_chunks<KB, SB>(t, old_sub, old_nb, new_sub, new_magic,
                          (uint64_t)blockIdx.x * blockDim.x + threadIdx.x,
                          (uint64_t)old_nb * Geo<KB, SB>::kG, stride);
}

// The same split for many subtables in one launch: each block finds its job
// (a binary search over the jobs' first blocks, the same for every thread of
// the block) and moves up to kResizeChunksPerBlock chunks of it.
template <int KB, int SB>
__device__ __forceinline__ void upsize_task(const ResizeJob &jb, uint32_t task) {
    const uint64_t chunks = (uint64_t)jb.old_nb * Geo<KB, SB>::kG;
    const uint64_t x0 = (uint64_t)(task - jb.block0) * kResizeChunksPerBlock;
    const uint64_t x1 = x0 + kResizeChunksPerBlock < chunks ? x0 + kResizeChunksPerBlock : chunks;
    upsize_chunks<KB, SB>(jb.t, (const char *)jb.old_sub, jb.old_nb, (char *)jb.new_sub, jb.magic,
                          x0 + threadIdx.x, x1, blockDim.x);
}

template <int KB, int SB>
__global__ void __launch_bounds__(256) k_resize_up_many(const __grid_constant__ ResizeJobs J) {
    uint32_t lo_j = 0, hi_j = J.n;
    while (hi_j - lo_j > 1) {
        const uint32_t mid = (lo_j + hi_j) >> 1;
        if (J.j[mid].block0 <= blockIdx.x) lo_j = mid;
        else hi_j = mid;
    }
    upsize_task<KB, SB>(J.j[lo_j], blockIdx.x);
}

// The jobs a table set's device policy listed (k_set_policy): their count
// and task total are read on the device, so the grid is fixed and each
// block takes tasks blockIdx.x, blockIdx.x + gridDim.x, ... The job count is
// clamped to the list's capacity (max_jobs).
template <int KB, int SB>
__global__ void __launch_bounds__(256) k_resize_up_list(const ResizeJob *__restrict__ jobs,
                                                        const SetPolicyOut *__restrict__ out,
                                                        uint32_t max_jobs) {
    const uint32_t nj = out->njobs < max_jobs ? out->njobs : max_jobs;
    if (nj == 0) return;
    const uint32_t ntask = out->ntasks;
    for (uint32_t task = blockIdx.x; task < ntask; task += gridDim.x) {
        uint32_t lo_j = 0, hi_j = nj;
        while (hi_j - lo_j > 1) {
            const uint32_t mid = (lo_j + hi_j) >> 1;
            if (jobs[mid].block0 <= task) lo_j = mid;
            else hi_j = mid;
        }
        const ResizeJob jb = jobs[lo_j];
        if (task >= jb.block0) upsize_task<KB, SB>(jb, task);
    }
}

// ----------------------------------------------------------------------------
// Bulk-copy helpers (cp.async.bulk through an mbarrier) for streaming a
// subtable through shared memory. Waits are bounded: a wait that gives up
// is counted in *timeouts and the caller stops using the buffer.
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes,
                                          uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void bulk_store(void *dst, uint32_t src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src),
                 "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// true when phase `parity` of the barrier completed within `tries` polls
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity,
                                          uint32_t tries = kWaitTries) {
    for (uint32_t i = 0; i < tries; ++i) {
        uint32_t done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; "
            "selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// ----------------------------------------------------------------------------
// even downsize: new bucket j = old bucket j merged with old bucket j + nb/2
// (both halves of old bucket j's upsize image); entries that do not fit go to
// the list for eviction walks (cuckoo_resize_down, cuckoo.cu:638-728, whose
// residuals are dropped; here they are placed again). Tiles of kMergeTile
// buckets stream through shared memory by bulk copies: two loads (the tile
// of each half) completing on an mbarrier, a merge by one thread per bucket
// in place, one bulk store of the merged tile. The metadata words are OR-ed.
// A tile wait that gives up after tile_wait_tries polls (kWaitTries unless a
// test lowers it) is counted in *timeouts and the block stops; the old
// subtable is only read, so the caller can keep it.
// ----------------------------------------------------------------------------
constexpr int kMergeTile = 128;  // buckets per tile = threads per block

template <int KB, int SB>
__global__ void __launch_bounds__(kMergeTile) k_resize_down(const char *__restrict__ old_sub,
                                                            uint32_t new_nb,
                                                            char *__restrict__ new_sub,
                                                            void *list,
                                                            unsigned long long *list_count,
                                                            uint64_t list_cap,
                                                            unsigned long long *spill,
                                                            unsigned long long *timeouts,
                                                            uint32_t tile_wait_tries) {
    using T = SlotT<KB>;
    using Sl = typename T::S;
    using Gm = Geo<KB, SB>;
    constexpr int B = Gm::kSlots, W = T::kBytes / 4;
    __shared__ __align__(128) unsigned char sa[kMergeTile * SB];
    __shared__ __align__(128) unsigned char sc[kMergeTile * SB];
    __shared__ __align__(8) unsigned long long bar_storage;
    __shared__ int failed;
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&bar_storage);
    const uint32_t sa_addr = (uint32_t)__cvta_generic_to_shared(sa);
    const uint32_t sc_addr = (uint32_t)__cvta_generic_to_shared(sc);
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(bar, 1);
        failed = 0;
    }
    __syncthreads();
    uint32_t parity = 0;
    const uint64_t tiles = ((uint64_t)new_nb + kMergeTile - 1) / kMergeTile;
    for (uint64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint64_t j0 = tile * kMergeTile;
        const uint32_t cnt = (uint32_t)((uint64_t)new_nb - j0 < kMergeTile ? new_nb - j0 : kMergeTile);
        const uint32_t bytes = cnt * SB;
        if (tid == 0) {
            // the previous tile's store has read sa; generic accesses before
            // the barrier are ordered before the async proxy's writes
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_expect_tx(bar, 2 * bytes);
            bulk_load(sa_addr, old_sub + j0 * SB, bytes, bar);
            bulk_load(sc_addr, old_sub + (j0 + new_nb) * SB, bytes, bar);
        }
        const bool ok = mbar_wait(bar, parity, tile_wait_tries);
        parity ^= 1u;
        if (!ok) {
            if (tid == 0) atomicAdd(timeouts, 1ull);
            failed = 1;
        }
        __syncthreads();
        if (failed) break;
        // merge: a group of G = SB/32 lanes per bucket, 32 bytes (SPC slots)
        // per lane, 32/G buckets per warp step (contiguous shared reads); the
        // second half's entries move into the first half's empty slots by
        // shuffles, SPC rounds of one slot per lane
        {
            constexpr int G = Gm::kG, SPC = Gm::kSPC, BPS = 32 / G;
            const int lane = tid & 31, g = lane / G, r = lane % G;
            const unsigned entry_mask = (B == 32) ? kFull : ((1u << B) - 1u);
            for (uint32_t b0 = (uint32_t)(tid >> 5) * BPS; b0 < cnt; b0 += 4 * BPS) {
                const uint32_t bk = b0 + g;
                const bool valid = bk < cnt;
                Sl a[SPC], c[SPC];
                unsigned my_a = 0u, my_c = 0u;
#pragma unroll
                for (int j = 0; j < SPC; ++j) {
                    if (valid) {
                        T::from_words((const uint32_t *)(sa + bk * SB + r * 32) + j * W, a[j]);
                        T::from_words((const uint32_t *)(sc + bk * SB + r * 32) + j * W, c[j]);
                    } else {
                        a[j] = T::empty();
                        c[j] = T::empty();
                    }
                    if (!T::is_empty(a[j])) my_a |= 1u << (r * SPC + j);
                    if (!T::is_empty(c[j])) my_c |= 1u << (r * SPC + j);
                }
                const unsigned occ_a = group_or<G>(my_a) & entry_mask;
                const unsigned cocc = group_or<G>(my_c) & entry_mask;
                const unsigned freem = ~occ_a & entry_mask;
                const int nfree = __popc(freem), nc = __popc(cocc);
                // which c slot (lane of the group, slot in the lane) each of my
                // empty slots takes
                int src_lane[SPC], src_j[SPC];
#pragma unroll
                for (int j = 0; j < SPC; ++j) {
                    const int idx = r * SPC + j;
                    src_lane[j] = -1;
                    src_j[j] = 0;
                    if (idx < B && ((freem >> idx) & 1u)) {
                        const int rank = __popc(freem & ((1u << idx) - 1u));
                        if (rank < nc) {
                            const int si = nth_set(cocc, rank);
                            src_lane[j] = g * G + si / SPC;
                            src_j[j] = si % SPC;
                        }
                    }
                }
#pragma unroll
                for (int jj = 0; jj < SPC; ++jj) {
#pragma unroll
                    for (int j = 0; j < SPC; ++j) {
                        const Sl v = shfl_slot(c[jj], src_lane[j] < 0 ? lane : src_lane[j]);
                        if (src_lane[j] >= 0 && src_j[j] == jj) a[j] = v;
                    }
                }
                // c entries beyond the free slots go to the list
#pragma unroll
                for (int j = 0; j < SPC; ++j) {
                    const int idx = r * SPC + j;
                    if (valid && idx < B && ((cocc >> idx) & 1u) &&
                        __popc(cocc & ((1u << idx) - 1u)) >= nfree) {
                        const unsigned long long at = atomicAdd(list_count, 1ull);
                        if (at < list_cap) ((Sl *)list)[at] = c[j];
                        else atomicAdd(spill, 1ull);
                    }
                }
                if (Gm::kMeta && r == G - 1) {  // metadata word: last slot of the bucket
                    uint32_t ma[4], mc[4];
                    T::to_words(a[SPC - 1], ma);
                    T::to_words(c[SPC - 1], mc);
                    uint32_t mw[4] = {ma[0] | mc[0], ma[1] | mc[1], 0u, 0u};
                    T::from_words(mw, a[SPC - 1]);
                }
                if (valid) {
#pragma unroll
                    for (int j = 0; j < SPC; ++j)
                        T::to_words(a[j], (uint32_t *)(sa + bk * SB + r * 32) + j * W);
                }
            }
        }
        // the merged tile (written by generic stores) goes out by the async proxy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) bulk_store(new_sub + j0 * SB, sa_addr, bytes);
    }
    if (tid == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    // the loads of a tile whose wait gave up are still in flight: wait for
    // them (full bound) before the block's shared memory goes away
    if (failed && tid == 0) mbar_wait(bar, parity ^ 1u);
}

// every live slot of one subtable into a list (odd-size downsize)
template <int KB, int SB>
__global__ void __launch_bounds__(256) k_collect(const char *__restrict__ sub, uint32_t nb,
                                                 void *list, unsigned long long *list_count,
                                                 uint64_t list_cap, unsigned long long *spill) {
    using T = SlotT<KB>;
    using Sl = typename T::S;
    constexpr int B = Geo<KB, SB>::kSlots;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nb; j += stride) {
        Bucket<KB, SB> a;
        a.template load<0>(sub + j * SB);
        const unsigned live = ((B == 32) ? kFull : ((1u << B) - 1u)) & ~a.empty_mask();
        if (!live) continue;
        unsigned long long at = atomicAdd(list_count, (unsigned long long)__popc(live));
#pragma unroll
        for (int q = 0; q < B; ++q) {
            if (T::is_empty(a.s[q])) continue;
            if (at < list_cap) ((Sl *)list)[at] = a.s[q];
            else atomicAdd(spill, 1ull);
            ++at;
        }
    }
}

// set the overflow bit of every bucket of a subtable (after an odd-size
// downsize the bits of the old buckets no longer map onto the new ones)
template <int KB, int SB>
__global__ void __launch_bounds__(256) k_mark_all(char *__restrict__ sub, uint32_t nb) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nb; j += stride)
        if (Geo<KB, SB>::kMeta) *meta_ptr<KB, SB>(sub + j * SB) = kAllFingerprints;
}

// every live (key, value) of one subtable
template <int KB, int SB>
__global__ void __launch_bounds__(256) k_export(const char *__restrict__ sub, uint32_t nb,
                                                void *keys, void *vals, uint32_t vb, uint64_t cap,
                                                unsigned long long *count) {
    using T = SlotT<KB>;
    constexpr int B = Geo<KB, SB>::kSlots;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nb; j += stride) {
        Bucket<KB, SB> a;
        a.template load<0>(sub + j * SB);
        const unsigned live = ((B == 32) ? kFull : ((1u << B) - 1u)) & ~a.empty_mask();
        if (!live) continue;
        unsigned long long at = atomicAdd(count, (unsigned long long)__popc(live));
#pragma unroll
        for (int q = 0; q < B; ++q) {
            if (T::is_empty(a.s[q])) continue;
            if (at < cap) {
                ((typename T::K *)keys)[at] = T::key(a.s[q]);
                store_val(vals, vb, at, T::val(a.s[q]));
            }
            ++at;
        }
    }
}

}  // namespace dyc
