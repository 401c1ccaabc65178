// dyc_kernels.cuh -- the sm_103a kernels of the DyCuckoo table, templated on
// key width KB (4 or 8 bytes) and bucket size SB (32, 64 or 128 bytes).
//
// Design (GB300):
//   * One thread per op; a bucket is one to four 32-byte sectors read with
//     256-bit loads, so a probe costs exactly the sectors of its bucket.
//     (The reference uses 16-lane groups over 128-byte buckets:
//     GPU/dyhash/cuckoo.cu:365-520.)
//   * Loops are warp-uniform (every lane of a warp runs the same iterations),
//     so ballots and warp-aggregated counters always use the full mask.
//   * Insert runs in phases separated by kernel boundaries: (1) resolve
//     repeated keys of the batch, (2) update present keys / claim empty
//     slots -- nothing moves while keys are being searched, (3) eviction
//     walks for the ops whose two buckets were full. Phase 3 only places keys
//     known to be absent, so a concurrently evicted entry can never be
//     mistaken for a missing key.
//   * Every loop is bounded: probe loops by the table size, eviction walks by
//     max_evict. Nothing spins on another thread.
#pragma once

#include "dyc_device.cuh"

namespace dyc {

__device__ __forceinline__ uint64_t warp_base() {
    return (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) << 5;
}
__device__ __forceinline__ uint64_t warp_stride() {
    return ((uint64_t)gridDim.x * blockDim.x) & ~31ull;
}

// Slot j of a register bucket, selected without dynamic register indexing.
template <int KB, int SB>
__device__ __forceinline__ typename SlotT<KB>::S slot_at(const Bucket<KB, SB> &b, int j) {
    typename SlotT<KB>::S r = SlotT<KB>::empty();
#pragma unroll
    for (int q = 0; q < Bucket<KB, SB>::kSlots; ++q)
        if (q == j) r = b.s[q];
    return r;
}

template <int KB, int SB>
__device__ __forceinline__ typename SlotT<KB>::S *slot_ptr(char *bucket, int j) {
    return reinterpret_cast<typename SlotT<KB>::S *>(bucket + j * SlotT<KB>::kBytes);
}

// Value of key k in bucket b; returns whether it was there.
template <int KB, int SB>
__device__ __forceinline__ bool bucket_get(const Bucket<KB, SB> &b, typename SlotT<KB>::K k,
                                           uint64_t &v) {
    bool hit = false;
#pragma unroll
    for (int q = 0; q < Bucket<KB, SB>::kSlots; ++q)
        if (SlotT<KB>::key(b.s[q]) == k) {
            hit = true;
            v = SlotT<KB>::val(b.s[q]);
        }
    return hit;
}

// Claim an empty slot of the bucket at p (snapshot b) for e with CAS.
template <int KB, int SB>
__device__ __forceinline__ bool try_empty(char *p, const Bucket<KB, SB> &b,
                                          const typename SlotT<KB>::S &e) {
    using T = SlotT<KB>;
#pragma unroll
    for (int q = 0; q < Bucket<KB, SB>::kSlots; ++q) {
        if (T::is_empty(b.s[q])) {
            typename T::S old = T::cas(slot_ptr<KB, SB>(p, q), T::empty(), e);
            if (T::same(old, T::empty())) return true;
        }
    }
    return false;
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
                return;
            }
        }
    }
    __device__ static __forceinline__ bool winner(const Scratch &S, uint32_t k, uint32_t i) {
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
                return;
            }
        }
    }
    __device__ static __forceinline__ bool winner(const Scratch &S, uint64_t k, uint32_t i) {
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

template <int KB>
__global__ void __launch_bounds__(256) k_dedup(const __grid_constant__ Scratch S, const void *__restrict__ keys,
                                               uint64_t n, DedupMode mode) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        typename SlotT<KB>::K k = load_key<KB>(keys, i);
        if (k != 0) Dedup<KB>::claim(S, k, (uint32_t)i, mode);
    }
}

// ----------------------------------------------------------------------------
// find: probe the first subtable of the key's pair, then the second
// (cuckoo_search, cuckoo.cu:460-520). Writes the value (0 on a miss) and one
// hit bit per key.
// ----------------------------------------------------------------------------
template <int KB, int SB>
__global__ void __launch_bounds__(256) k_find(const __grid_constant__ Desc D, const void *__restrict__ keys,
                                              void *__restrict__ vals, uint32_t vb,
                                              uint32_t *__restrict__ hits, uint64_t n) {
    using T = SlotT<KB>;
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t step = warp_stride();
    for (uint64_t base = warp_base(); base < n; base += step) {
        const uint64_t i = base + lane;
        typename T::K k = 0;
        if (i < n) k = load_key<KB>(keys, i);
        bool hit = false;
        uint64_t v = 0;
        if (k != 0) {
            const uint32_t hk = fold(k);
            const Pair p = pair_of(hk, D.d);
            Bucket<KB, SB> b;
            b.load_nc(bucket_ptr<KB, SB>(D, p.first, bucket_index(D, p.first, hk)));
            hit = bucket_get(b, k, v);
            if (!hit) {
                b.load_nc(bucket_ptr<KB, SB>(D, p.second, bucket_index(D, p.second, hk)));
                hit = bucket_get(b, k, v);
            }
        }
        if (i < n) store_val(vals, vb, i, v);
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (hits != nullptr && lane == 0) hits[base >> 5] = m;
    }
}

// ----------------------------------------------------------------------------
// insert phase 2: update present keys in place, else claim an empty slot in
// the first or second bucket; ops with both buckets full go to list_a.
// ----------------------------------------------------------------------------
template <int KB, int SB>
__global__ void __launch_bounds__(256) k_place(const __grid_constant__ Desc D, const __grid_constant__ Scratch S, int use_dedup,
                                               int new_keys, const void *__restrict__ keys,
                                               const void *__restrict__ vals, uint32_t vb,
                                               uint64_t n, Counters *ctr) {
    using T = SlotT<KB>;
    using Sl = typename T::S;
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t step = warp_stride();
    uint32_t n_ins = 0, n_upd = 0, n_rej = 0, n_sup = 0;
    for (uint64_t base = warp_base(); base < n; base += step) {
        const uint64_t i = base + lane;
        bool pend = false;
        Sl e = T::empty();
        if (i < n) {
            const typename T::K k = load_key<KB>(keys, i);
            if (k == 0) {
                ++n_rej;
            } else if (use_dedup && !Dedup<KB>::winner(S, k, (uint32_t)i)) {
                ++n_sup;
            } else {
                e = T::make(k, load_val(vals, vb, i));
                const uint32_t hk = fold(k);
                const Pair p = pair_of(hk, D.d);
                char *p1 = bucket_ptr<KB, SB>(D, p.first, bucket_index(D, p.first, hk));
                char *p2 = bucket_ptr<KB, SB>(D, p.second, bucket_index(D, p.second, hk));
                Bucket<KB, SB> b1, b2;
                b1.load_cg(p1);
                int r = 0;  // 1 updated, 2 inserted
                if (!new_keys) {
                    int j = b1.find(k);
                    if (j >= 0) {
                        T::exch(slot_ptr<KB, SB>(p1, j), e);
                        r = 1;
                    } else {
                        b2.load_cg(p2);
                        j = b2.find(k);
                        if (j >= 0) {
                            T::exch(slot_ptr<KB, SB>(p2, j), e);
                            r = 1;
                        } else if (try_empty<KB, SB>(p1, b1, e) || try_empty<KB, SB>(p2, b2, e)) {
                            r = 2;
                        }
                    }
                } else {
                    if (try_empty<KB, SB>(p1, b1, e)) {
                        r = 2;
                    } else {
                        b2.load_cg(p2);
                        if (try_empty<KB, SB>(p2, b2, e)) r = 2;
                    }
                }
                if (r == 1) ++n_upd;
                else if (r == 2) ++n_ins;
                else pend = true;
            }
        }
        __syncwarp();
        const unsigned long long at = agg_inc(&ctr->pending, pend);
        if (pend) {
            if (at < S.list_cap) ((Sl *)S.list_a)[at] = e;
            else atomicAdd(&ctr->spill, 1ull);
        }
    }
    agg_add(&ctr->inserted, n_ins);
    agg_add(&ctr->size, n_ins);
    agg_add(&ctr->updated, n_upd);
    agg_add(&ctr->rejected, n_rej);
    agg_add(&ctr->superseded, n_sup);
}

// Victim choice when a bucket is full: prefer a resident that sits in the
// second subtable of its own pair (evicting it moves it back to its first,
// where finds look first); rotate the start so chains do not cycle.
template <int KB, int SB>
__device__ __forceinline__ int pick_victim(const Bucket<KB, SB> &b, uint32_t t, uint32_t d,
                                           uint32_t rot) {
    constexpr int B = Bucket<KB, SB>::kSlots;
    unsigned pref = 0;
#pragma unroll
    for (int q = 0; q < B; ++q) {
        const Pair pr = pair_of(fold(SlotT<KB>::key(b.s[q])), d);
        if (pr.first != t) pref |= 1u << q;
    }
    rot &= (B - 1);
    if (!pref) return (int)rot;
    const unsigned rotated = ((pref >> rot) | (pref << (B - rot))) & ((1u << B) - 1u);
    return (int)((__ffs(rotated) - 1 + rot) & (B - 1));
}

// One bounded eviction walk; on failure `e` holds the entry left over.
template <int KB, int SB>
__device__ __forceinline__ bool walk_one(const Desc &D, typename SlotT<KB>::S &e,
                                         uint32_t max_evict, uint32_t &steps) {
    using T = SlotT<KB>;
    uint32_t hk = fold(T::key(e));
    Pair p = pair_of(hk, D.d);
    char *p1 = bucket_ptr<KB, SB>(D, p.first, bucket_index(D, p.first, hk));
    char *p2 = bucket_ptr<KB, SB>(D, p.second, bucket_index(D, p.second, hk));
    Bucket<KB, SB> b;
    b.load_cg(p1);
    if (try_empty<KB, SB>(p1, b, e)) return true;
    b.load_cg(p2);
    if (try_empty<KB, SB>(p2, b, e)) return true;
    uint32_t t = p.first;
    char *bp = p1;
    const uint32_t seed = hk;
    for (uint32_t s = 0; s < max_evict; ++s) {
        b.load_cg(bp);
        if (try_empty<KB, SB>(bp, b, e)) return true;
        const int j = pick_victim<KB, SB>(b, t, D.d, seed + s);
        typename T::S old = T::exch(slot_ptr<KB, SB>(bp, j), e);
        ++steps;
        if (T::is_empty(old)) return true;
        e = old;
        hk = fold(T::key(e));
        p = pair_of(hk, D.d);
        t = other_of(p, t);
        bp = bucket_ptr<KB, SB>(D, t, bucket_index(D, t, hk));
    }
    return false;
}

// insert phase 3: eviction walks. Entries come from `src`; an entry whose
// walk reaches max_evict goes to `dst` for the host to place after an upsize.
template <int KB, int SB>
__global__ void __launch_bounds__(256) k_walk(const __grid_constant__ Desc D, const void *__restrict__ src,
                                              const unsigned long long *src_count, void *dst,
                                              unsigned long long *dst_count, uint64_t dst_cap,
                                              uint32_t max_evict, int count_new, Counters *ctr,
                                              uint64_t max_entries) {
    using T = SlotT<KB>;
    using Sl = typename T::S;
    const uint32_t lane = threadIdx.x & 31;
    uint64_t n = *src_count;
    if (n > max_entries) n = max_entries;
    const uint64_t step = warp_stride();
    uint32_t n_ok = 0, n_steps = 0;
    for (uint64_t base = warp_base(); base < n; base += step) {
        const uint64_t i = base + lane;
        bool fail = false;
        Sl e = T::empty();
        if (i < n) {
            e = ((const Sl *)src)[i];
            if (walk_one<KB, SB>(D, e, max_evict, n_steps)) ++n_ok;
            else fail = true;
        }
        __syncwarp();
        const unsigned long long at = agg_inc(dst_count, fail);
        if (fail) {
            if (at < dst_cap) ((Sl *)dst)[at] = e;
            else atomicAdd(&ctr->spill, 1ull);
        }
    }
    if (count_new) {
        agg_add(&ctr->inserted, n_ok);
        agg_add(&ctr->size, n_ok);
    }
    agg_add(&ctr->evict_steps, n_steps);
}

// ----------------------------------------------------------------------------
// erase: probe both buckets; the slot holding the key is cleared with a CAS
// (the reference clears with a plain store and returns nothing,
// cuckoo.cu:524-587).
// ----------------------------------------------------------------------------
template <int KB, int SB>
__global__ void __launch_bounds__(256) k_erase(const __grid_constant__ Desc D, const __grid_constant__ Scratch S, int use_dedup,
                                               const void *__restrict__ keys, uint64_t n,
                                               uint32_t *__restrict__ bits, Counters *ctr) {
    using T = SlotT<KB>;
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t step = warp_stride();
    uint32_t n_del = 0, n_sup = 0;
    for (uint64_t base = warp_base(); base < n; base += step) {
        const uint64_t i = base + lane;
        bool erased = false;
        if (i < n) {
            const typename T::K k = load_key<KB>(keys, i);
            if (k != 0) {
                if (use_dedup && !Dedup<KB>::winner(S, k, (uint32_t)i)) {
                    ++n_sup;
                } else {
                    const uint32_t hk = fold(k);
                    const Pair p = pair_of(hk, D.d);
#pragma unroll 1
                    for (int r = 0; r < 2 && !erased; ++r) {
                        const uint32_t t = r ? p.second : p.first;
                        char *bp = bucket_ptr<KB, SB>(D, t, bucket_index(D, t, hk));
                        Bucket<KB, SB> b;
                        b.load_cg(bp);
                        const int j = b.find(k);
                        if (j >= 0) {
                            const typename T::S cur = slot_at(b, j);
                            const typename T::S old = T::cas(slot_ptr<KB, SB>(bp, j), cur, T::empty());
                            erased = T::same(old, cur);
                            break;
                        }
                    }
                }
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, erased);
        if (bits != nullptr && lane == 0) bits[base >> 5] = m;
        n_del += erased ? 1u : 0u;
    }
    // loops are warp-uniform, so every lane of the warp is here
    const uint32_t del = __reduce_add_sync(0xffffffffu, n_del);
    const uint32_t sup = __reduce_add_sync(0xffffffffu, n_sup);
    if (lane == 0) {
        if (del) {
            atomicAdd(&ctr->erased, (unsigned long long)del);
            atomicAdd(&ctr->size, (unsigned long long)(-(long long)del));  // size -= del
        }
        if (sup) atomicAdd(&ctr->superseded, (unsigned long long)sup);
    }
}

// ----------------------------------------------------------------------------
// upsize: subtable t goes from nb to 2nb buckets. hash % 2nb of an entry in
// old bucket b is b or b+nb, so every slot keeps its index and each old
// bucket writes exactly two new buckets: a pure stream, read S / write 2S,
// no zero-fill pass and no atomics (cuckoo_resize_up, cuckoo.cu:600-627).
// ----------------------------------------------------------------------------
template <int KB, int SB>
__global__ void __launch_bounds__(256) k_resize_up(uint32_t t, const char *__restrict__ old_sub,
                                                   uint32_t old_nb, char *__restrict__ new_sub,
                                                   uint64_t new_magic, uint32_t new_nb) {
    using T = SlotT<KB>;
    constexpr int B = Bucket<KB, SB>::kSlots;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < old_nb; b += stride) {
        Bucket<KB, SB> src, lo, hi;
        src.load_nc(old_sub + b * SB);
#pragma unroll
        for (int q = 0; q < B; ++q) {
            lo.s[q] = T::empty();
            hi.s[q] = T::empty();
            if (!T::is_empty(src.s[q])) {
                const uint32_t nbk =
                    fastmod(subtable_hash(fold(T::key(src.s[q])), t), new_magic, new_nb);
                if (nbk == (uint32_t)b) lo.s[q] = src.s[q];
                else hi.s[q] = src.s[q];
            }
        }
        lo.store(new_sub + b * SB);
        hi.store(new_sub + (b + old_nb) * SB);
    }
}

// ----------------------------------------------------------------------------
// downsize of an even subtable: new bucket j = old buckets j and j+nb/2
// merged; entries that do not fit are listed for eviction walks
// (cuckoo_resize_down, cuckoo.cu:638-728, which drops the ones its walks
// cannot place).
// ----------------------------------------------------------------------------
template <int KB, int SB>
__global__ void __launch_bounds__(256) k_resize_down(const char *__restrict__ old_sub,
                                                     uint32_t new_nb, char *__restrict__ new_sub,
                                                     void *list, unsigned long long *list_count,
                                                     uint64_t list_cap,
                                                     unsigned long long *spill) {
    using T = SlotT<KB>;
    using Sl = typename T::S;
    constexpr int B = Bucket<KB, SB>::kSlots;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < new_nb; j += stride) {
        Bucket<KB, SB> a, c;
        a.load_nc(old_sub + j * SB);
        c.load_nc(old_sub + (j + new_nb) * SB);
        unsigned freem = a.empty_mask();
#pragma unroll
        for (int q = 0; q < B; ++q) {
            if (T::is_empty(c.s[q])) continue;
            if (freem) {
                const int pos = __ffs(freem) - 1;
                freem &= freem - 1;
#pragma unroll
                for (int r = 0; r < B; ++r)
                    if (r == pos) a.s[r] = c.s[q];
            } else {
                const unsigned long long at = atomicAdd(list_count, 1ull);
                if (at < list_cap) ((Sl *)list)[at] = c.s[q];
                else atomicAdd(spill, 1ull);
            }
        }
        a.store(new_sub + j * SB);
    }
}

// every live slot of one subtable into a list (odd-size downsize)
template <int KB, int SB>
__global__ void __launch_bounds__(256) k_collect(const char *__restrict__ sub, uint32_t nb,
                                                 void *list, unsigned long long *list_count,
                                                 uint64_t list_cap, unsigned long long *spill) {
    using T = SlotT<KB>;
    using Sl = typename T::S;
    constexpr int B = Bucket<KB, SB>::kSlots;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nb; j += stride) {
        Bucket<KB, SB> a;
        a.load_nc(sub + j * SB);
        const unsigned live = ((1u << B) - 1u) & ~a.empty_mask();
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

// every live (key, value) of one subtable
template <int KB, int SB>
__global__ void __launch_bounds__(256) k_export(const char *__restrict__ sub, uint32_t nb,
                                                void *keys, void *vals, uint32_t vb, uint64_t cap,
                                                unsigned long long *count) {
    using T = SlotT<KB>;
    constexpr int B = Bucket<KB, SB>::kSlots;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nb; j += stride) {
        Bucket<KB, SB> a;
        a.load_nc(sub + j * SB);
        const unsigned live = ((1u << B) - 1u) & ~a.empty_mask();
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
