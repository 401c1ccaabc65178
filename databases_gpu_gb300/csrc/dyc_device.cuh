// dyc_device.cuh -- device building blocks of the GB300 DyCuckoo table:
// the reference's hash functions and pair maps, bucket addressing, slot
// formats, 256-bit bucket loads/stores and 64/128-bit slot atomics.
#pragma once

#include <cstdint>

#include "dyc_internal.h"

namespace dyc {

// ----------------------------------------------------------------------------
// Hash functions. The same integer mixers as GPU/dyhash/cuckoo.cu:27-64
// (get_hash1..4: Thomas Wang's 32-bit mix, Bob Jenkins' 6-step mix, an
// xor-add-mod, and the 0x27d4eb2d multiply-xorshift) and :110-120 (get_hash5,
// the shift-subtract mix that chooses the subtable pair). They must match
// bit for bit so that keys land in the buckets the reference computes.
// ----------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint32_t hash1(uint32_t k) {
    k = ~k + (k << 15);
    k ^= k >> 12;
    k += k << 2;
    k ^= k >> 4;
    k *= 2057u;
    k ^= k >> 16;
    return k;
}
__host__ __device__ __forceinline__ uint32_t hash2(uint32_t a) {
    a = (a + 0x7ed55d16u) + (a << 12);
    a = (a ^ 0xc761c23cu) ^ (a >> 19);
    a = (a + 0x165667b1u) + (a << 5);
    a = (a + 0xd3a2646cu) ^ (a << 9);
    a = (a + 0xfd7046c5u) + (a << 3);
    a = (a ^ 0xb55a4f09u) ^ (a >> 16);
    return a;
}
__host__ __device__ __forceinline__ uint32_t hash3(uint32_t s) {
    return ((s ^ 59064253u) + 72355969u) % kPrime;
}
__host__ __device__ __forceinline__ uint32_t hash4(uint32_t a) {
    a = (a ^ 61u) ^ (a >> 16);
    a += a << 3;
    a ^= a >> 4;
    a *= 0x27d4eb2du;
    a ^= a >> 15;
    return a;
}
__host__ __device__ __forceinline__ uint32_t hash5(uint32_t a) {
    a -= a << 6;
    a ^= a >> 17;
    a -= a << 9;
    a ^= a << 4;
    a -= a << 3;
    a ^= a << 10;
    a ^= a >> 15;
    return a;
}

// Subtable t uses get_hash{t%4+1}(k) % 294967291 % nbuckets (cuckoo.cu:76-90).
// The final modulo by the runtime bucket count uses a precomputed 64-bit
// reciprocal (Lemire, Kaser & Kurz 2019, "Faster remainder by direct
// computation"): exact for every 32-bit numerator and divisor.
__host__ __device__ __forceinline__ uint64_t fastmod_magic(uint32_t d) {
    return ~0ull / d + 1ull;
}
__device__ __forceinline__ uint32_t fastmod(uint32_t a, uint64_t magic, uint32_t d) {
    return (uint32_t)__umul64hi(magic * a, d);
}
// Branch-free: lanes of a warp ask for different subtables, and a switch on
// t would run all four hash paths one after another. All four are computed
// (the compiler shares them between the two buckets of a key) and one is
// selected; hash3 already ends in % kPrime, so the common % is a no-op for it.
__device__ __forceinline__ uint32_t subtable_hash(uint32_t hk, uint32_t t) {
    const uint32_t a = hash1(hk), b = hash2(hk), c = hash3(hk), e = hash4(hk);
    const uint32_t lo = (t & 1u) ? b : a;
    const uint32_t hi = (t & 1u) ? e : c;
    return ((t & 2u) ? hi : lo) % kPrime;
}

// 64-bit keys fold to the 32-bit hash input; equality uses all 64 bits.
__host__ __device__ __forceinline__ uint32_t fold(uint32_t k) { return k; }
__host__ __device__ __forceinline__ uint32_t fold(uint64_t k) {
    uint32_t lo = (uint32_t)k, hi = (uint32_t)(k >> 32);
    return lo ^ hi ^ (0x9e3779b9u * hi);
}

// Pair map: key -> the two subtables it may live in. d = 4 is
// cuckoo.cu:190-213 (choose_hash = hash5 % 6, pos1, pos2); d = 2, 3, 5, 6
// are the variants of GPU/dyhash/diff_hash_num_pos_fun.cpp:14-188.
struct Pair {
    uint32_t first, second;  // probe order: `first` is looked at first
};
__device__ __forceinline__ Pair ref_pair(uint32_t hk, uint32_t h5, uint32_t d) {
    uint32_t p;
    switch (d) {
    case 2: p = hk & 1u; return {p, p ^ 1u};
    case 3:
        p = h5 % 3u;
        return {(p & 1u) ? 1u : 0u, (p & 1u) ? 2u : (p >> 1) + 1u};
    case 5:
        p = h5 % 10u;
        if (p == 9u) return {3u, 4u};
        if (p & 1u) return {0u, (p >> 1) + 1u};
        if (p & 2u) return {2u, (p >> 2) + 3u};
        return {1u, (p >> 2) + 2u};
    case 6:
        p = h5 % 15u;
        if (p <= 4u) return {0u, p + 1u};
        if (p <= 8u) return {1u, p - 3u};
        if (p <= 11u) return {2u, p - 6u};
        if (p <= 13u) return {3u, p - 8u};
        return {4u, 5u};
    default:
        p = h5 % 6u;
        if (p & 1u) return {0u, (p >> 1) + 1u};
        if (p & 2u) return {2u, 3u};
        return {1u, (p >> 2) + 2u};
    }
}
// Probe order. The reference always probes pos1 first (cuckoo.cu:482), but
// its pair map makes subtable 0 the first choice of half of all keys and the
// last subtable of none (d = 4), so at high load a large share of hits needs
// a second probe. Here bit 16 of hash5 picks which member of the pair is
// probed first, giving every subtable the same first-probe share; the two
// candidate buckets are still exactly the reference's.
__device__ __forceinline__ bool probe_swap(uint32_t h5) { return (h5 >> 16) & 1u; }
__device__ __forceinline__ Pair pair_of(uint32_t hk, uint32_t d) {
    const uint32_t h5 = hash5(hk);
    const Pair r = ref_pair(hk, h5, d);
    return probe_swap(h5) ? Pair{r.second, r.first} : r;
}
// The other subtable of a key's pair, seen from subtable `t` (get_pos,
// cuckoo.cu:310-312).
__device__ __forceinline__ uint32_t other_of(Pair p, uint32_t t) {
    return t == p.first ? p.second : p.first;
}

__device__ __forceinline__ uint32_t bucket_index(const Desc &D, uint32_t t, uint32_t hk) {
    return fastmod(subtable_hash(hk, t), D.magic[t], D.nb[t]);
}

// ----------------------------------------------------------------------------
// Slot formats. A 4-byte-key slot is one 64-bit word: key in the low half,
// value in the high half; 0 is empty. An 8-byte-key slot is 16 bytes
// {key, value}; key 0 (and value 0) is empty. Updates are single 64-bit or
// 128-bit atomics (atom.cas/exch.b128 exist on sm_90 and later).
// ----------------------------------------------------------------------------
struct alignas(16) u128 {
    unsigned long long lo, hi;
};

template <int KB> struct SlotT;

template <> struct SlotT<4> {
    using S = unsigned long long;
    using K = uint32_t;
    static constexpr int kBytes = 8;
    __device__ static __forceinline__ K key(S s) { return (uint32_t)s; }
    __device__ static __forceinline__ uint64_t val(S s) { return s >> 32; }
    __device__ static __forceinline__ S make(K k, uint64_t v) {
        return (S)k | ((S)(uint32_t)v << 32);
    }
    __device__ static __forceinline__ S empty() { return 0ull; }
    __device__ static __forceinline__ bool is_empty(S s) { return (uint32_t)s == 0u; }
    __device__ static __forceinline__ bool same(S a, S b) { return a == b; }
    __device__ static __forceinline__ S cas(S *p, S cmp, S v) { return atomicCAS(p, cmp, v); }
    __device__ static __forceinline__ S exch(S *p, S v) { return atomicExch(p, v); }
    // plain store of a whole slot: for a slot no other thread of the kernel
    // can write (it holds a key the batch names once)
    __device__ static __forceinline__ void store(S *p, S v) {
        asm volatile("st.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
    }
    __device__ static __forceinline__ void from_words(const uint32_t *w, S &s) {
        s = (S)w[0] | ((S)w[1] << 32);
    }
    __device__ static __forceinline__ void to_words(S s, uint32_t *w) {
        w[0] = (uint32_t)s;
        w[1] = (uint32_t)(s >> 32);
    }
};

template <> struct SlotT<8> {
    using S = u128;
    using K = uint64_t;
    static constexpr int kBytes = 16;
    __device__ static __forceinline__ K key(S s) { return s.lo; }
    __device__ static __forceinline__ uint64_t val(S s) { return s.hi; }
    __device__ static __forceinline__ S make(K k, uint64_t v) { return {k, v}; }
    __device__ static __forceinline__ S empty() { return {0ull, 0ull}; }
    __device__ static __forceinline__ bool is_empty(S s) { return s.lo == 0ull; }
    __device__ static __forceinline__ bool same(S a, S b) { return a.lo == b.lo && a.hi == b.hi; }
    __device__ static __forceinline__ S cas(S *p, S cmp, S v) {
        S r;
        asm volatile(
            "{\n\t.reg .b128 d, c, s;\n\t"
            "mov.b128 c, {%2, %3};\n\t"
            "mov.b128 s, {%4, %5};\n\t"
            "atom.global.cas.b128 d, [%6], c, s;\n\t"
            "mov.b128 {%0, %1}, d;\n\t}"
            : "=l"(r.lo), "=l"(r.hi)
            : "l"(cmp.lo), "l"(cmp.hi), "l"(v.lo), "l"(v.hi), "l"(p)
            : "memory");
        return r;
    }
    __device__ static __forceinline__ S exch(S *p, S v) {
        S r;
        asm volatile(
            "{\n\t.reg .b128 d, s;\n\t"
            "mov.b128 s, {%2, %3};\n\t"
            "atom.global.exch.b128 d, [%4], s;\n\t"
            "mov.b128 {%0, %1}, d;\n\t}"
            : "=l"(r.lo), "=l"(r.hi)
            : "l"(v.lo), "l"(v.hi), "l"(p)
            : "memory");
        return r;
    }
    __device__ static __forceinline__ void store(S *p, S v) {
        asm volatile("st.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(v.lo), "l"(v.hi) : "memory");
    }
    __device__ static __forceinline__ void from_words(const uint32_t *w, S &s) {
        s.lo = (unsigned long long)w[0] | ((unsigned long long)w[1] << 32);
        s.hi = (unsigned long long)w[2] | ((unsigned long long)w[3] << 32);
    }
    __device__ static __forceinline__ void to_words(S s, uint32_t *w) {
        w[0] = (uint32_t)s.lo;
        w[1] = (uint32_t)(s.lo >> 32);
        w[2] = (uint32_t)s.hi;
        w[3] = (uint32_t)(s.hi >> 32);
    }
};

// ----------------------------------------------------------------------------
// 256-bit global accesses (one 32-byte DRAM sector per instruction).
//   ld_nc:  read-only path, no L1 allocation -- tables nobody writes during
//           the kernel (find, resize sources).
//   ld_cg:  L2-coherent load -- tables that other threads update with atomics
//           in the same kernel (insert, erase).
// ----------------------------------------------------------------------------
__device__ __forceinline__ void ld_nc(const void *p, uint32_t (&w)[8]) {
    asm volatile("ld.global.nc.L1::no_allocate.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]),
                   "=r"(w[6]), "=r"(w[7])
                 : "l"(p));
}
__device__ __forceinline__ void ld_cg(const void *p, uint32_t (&w)[8]) {
    asm volatile("ld.global.cg.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]),
                   "=r"(w[6]), "=r"(w[7])
                 : "l"(p)
                 : "memory");
}
__device__ __forceinline__ void st_v8(void *p, const uint32_t (&w)[8]) {
    asm volatile("st.global.v8.u32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(p), "r"(w[0]),
                 "r"(w[1]), "r"(w[2]), "r"(w[3]), "r"(w[4]), "r"(w[5]), "r"(w[6]), "r"(w[7])
                 : "memory");
}

// ----------------------------------------------------------------------------
// L2 residency. A table whose subtables fit in the L2 (Desc::l2_keep) reads
// its buckets with an evict_last cache policy, and the kernels that stream a
// batch through (find's keys, values and hit words) use evict_first, so the
// batch does not push the table out of the L2 between probes (PTX
// createpolicy + .L2::cache_hint: the eviction priorities an access-policy
// window applies, given per access, so tables need not be contiguous and no
// L2 set-aside is taken from the process). Other tables use evict_normal.
// ----------------------------------------------------------------------------
struct L2Pol {
    unsigned long long table, stream;
};
__device__ __forceinline__ L2Pol l2_policies(bool keep) {
    unsigned long long a, b;
    if (keep) {
        asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(a));
        asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(b));
    } else {
        asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(a));
        b = a;
    }
    return {a, b};
}
__device__ __forceinline__ void ld_nc_pol(const void *p, uint32_t (&w)[8], unsigned long long pol) {
    asm volatile(
        "ld.global.nc.L1::no_allocate.L2::cache_hint.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
        : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]), "=r"(w[6]),
          "=r"(w[7])
        : "l"(p), "l"(pol));
}
__device__ __forceinline__ void ld_cg_pol(const void *p, uint32_t (&w)[8], unsigned long long pol) {
    asm volatile("ld.global.cg.L2::cache_hint.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
                 : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]),
                   "=r"(w[6]), "=r"(w[7])
                 : "l"(p), "l"(pol)
                 : "memory");
}

__device__ __forceinline__ void ld_ca(const void *p, uint32_t (&w)[8]) {
    asm volatile("ld.global.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]),
                   "=r"(w[6]), "=r"(w[7])
                 : "l"(p));
}

// ----------------------------------------------------------------------------
// Bucket geometry. A bucket of SB bytes is SB/32 chunks of 32 bytes. A group
// of kG = SB/32 lanes reads one bucket with one 256-bit load per lane (lane r
// of the group reads chunk r), so a warp instruction fetches 32/kG whole
// buckets and every DRAM line it touches is used in full.
//
// A 128-byte bucket keeps its last slot as a metadata word of displacement
// fingerprints: bit fp(k) of its low 64 bits is set once a key k whose
// first-probe bucket this is has been stored in its second bucket, with fp(k)
// the top 6 bits of fold(k) * 0x9E3779B1 (bits the bucket index does not
// use). While k's bit is clear, k missing from this bucket is missing from the
// table, so a find or erase stops after one probe; a single "something was
// displaced" bit, set in most buckets at load factor 0.9, sent nearly every
// miss to a second line. Bits are only ever set (erase leaves them, a full
// rehash sets all), so a set bit is a hint that costs one extra probe, never a
// wrong answer.
// ----------------------------------------------------------------------------
__host__ __device__ __forceinline__ unsigned long long fp_bit(uint32_t hk) {
    return 1ull << ((hk * 0x9E3779B1u) >> 26);
}
constexpr unsigned long long kAllFingerprints = ~0ull;

template <int KB, int SB> struct Geo {
    using T = SlotT<KB>;
    static constexpr int kG = SB / 32;             // lanes per bucket
    static constexpr int kRoundOps = 32 / kG;      // buckets per warp instruction
    static constexpr int kSPC = 32 / T::kBytes;    // slots per 32-byte chunk
    static constexpr int kTotal = SB / T::kBytes;  // slots including the metadata slot
    static constexpr int kMeta = SB == 128 ? 1 : 0;
    static constexpr int kSlots = kTotal - kMeta;  // slots that hold entries
};

template <int KB, int SB>
__device__ __forceinline__ unsigned long long *meta_ptr(char *bucket) {
    return reinterpret_cast<unsigned long long *>(bucket + (Geo<KB, SB>::kTotal - 1) * SlotT<KB>::kBytes);
}

// A whole bucket in one thread's registers (streaming kernels: resize, export).
template <int KB, int SB> struct Bucket {
    using T = SlotT<KB>;
    using S = typename T::S;
    using G = Geo<KB, SB>;
    static constexpr int kSlots = G::kSlots;
    static constexpr int kChunks = SB / 32;
    static constexpr int kPerChunk = G::kSPC;
    S s[G::kTotal];

    template <int MODE>  // 0: default caching, 1: read-only no-allocate, 2: L2 only
    __device__ __forceinline__ void load(const void *p) {
#pragma unroll
        for (int c = 0; c < kChunks; ++c) {
            uint32_t w[8];
            if (MODE == 0) ld_ca((const char *)p + 32 * c, w);
            else if (MODE == 1) ld_nc((const char *)p + 32 * c, w);
            else ld_cg((const char *)p + 32 * c, w);
#pragma unroll
            for (int j = 0; j < kPerChunk; ++j) T::from_words(w + j * (T::kBytes / 4), s[c * kPerChunk + j]);
        }
    }
    __device__ __forceinline__ void store(void *p) const {
#pragma unroll
        for (int c = 0; c < kChunks; ++c) {
            uint32_t w[8];
#pragma unroll
            for (int j = 0; j < kPerChunk; ++j) T::to_words(s[c * kPerChunk + j], w + j * (T::kBytes / 4));
            st_v8((char *)p + 32 * c, w);
        }
    }
    __device__ __forceinline__ unsigned empty_mask() const {
        unsigned m = 0;
#pragma unroll
        for (int j = 0; j < kSlots; ++j)
            if (T::is_empty(s[j])) m |= 1u << j;
        return m;
    }
    __device__ __forceinline__ unsigned long long meta() const {
        if (!G::kMeta) return 0ull;
        uint32_t w[4];
        T::to_words(s[G::kTotal - 1], w);
        return (unsigned long long)w[0] | ((unsigned long long)w[1] << 32);
    }
};

template <int KB, int SB>
__device__ __forceinline__ char *bucket_ptr(const Desc &D, uint32_t t, uint32_t b) {
    return (char *)D.sub[t] + (uint64_t)b * SB;
}

// ----------------------------------------------------------------------------
// Batch I/O helpers (keys / values of either width, dense arrays).
// ----------------------------------------------------------------------------
template <int KB> __device__ __forceinline__ typename SlotT<KB>::K load_key(const void *k, uint64_t i);
template <> __device__ __forceinline__ uint32_t load_key<4>(const void *k, uint64_t i) {
    return __ldg((const uint32_t *)k + i);
}
template <> __device__ __forceinline__ uint64_t load_key<8>(const void *k, uint64_t i) {
    return __ldg((const unsigned long long *)k + i);
}
__device__ __forceinline__ uint64_t load_val(const void *v, uint32_t vb, uint64_t i) {
    return vb == 4 ? (uint64_t)__ldg((const uint32_t *)v + i)
                   : (uint64_t)__ldg((const unsigned long long *)v + i);
}
__device__ __forceinline__ void store_val(void *v, uint32_t vb, uint64_t i, uint64_t x) {
    if (vb == 4) ((uint32_t *)v)[i] = (uint32_t)x;
    else ((unsigned long long *)v)[i] = x;
}
// the same, with an L2 cache policy (a batch streaming past an L2-resident table)
template <int KB>
__device__ __forceinline__ typename SlotT<KB>::K load_key_pol(const void *k, uint64_t i,
                                                             unsigned long long pol) {
    if constexpr (KB == 4) {
        uint32_t r;
        asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;"
                     : "=r"(r)
                     : "l"((const uint32_t *)k + i), "l"(pol));
        return r;
    } else {
        unsigned long long r;
        asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u64 %0, [%1], %2;"
                     : "=l"(r)
                     : "l"((const unsigned long long *)k + i), "l"(pol));
        return r;
    }
}
__device__ __forceinline__ void store_u32_pol(uint32_t *p, uint32_t x, unsigned long long pol) {
    asm volatile("st.global.L2::cache_hint.u32 [%0], %1, %2;" ::"l"(p), "r"(x), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ void store_val_pol(void *v, uint32_t vb, uint64_t i, uint64_t x,
                                              unsigned long long pol) {
    if (vb == 4) {
        store_u32_pol((uint32_t *)v + i, (uint32_t)x, pol);
    } else {
        asm volatile("st.global.L2::cache_hint.u64 [%0], %1, %2;" ::"l"((unsigned long long *)v + i),
                     "l"(x), "l"(pol)
                     : "memory");
    }
}

// Warp-aggregated counter increment: one atomic per warp for the lanes that
// pass `pred`; returns this lane's slot (valid only where pred is true).
__device__ __forceinline__ unsigned long long agg_inc(unsigned long long *ctr, bool pred) {
    const unsigned mask = __activemask();
    const unsigned vote = __ballot_sync(mask, pred);
    if (!vote) return 0ull;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(vote) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(ctr, (unsigned long long)__popc(vote));
    base = __shfl_sync(mask, base, leader);
    return base + __popc(vote & ((1u << lane) - 1u));
}

// Mixing hash of the batch-dedup table, the grouping cells and the eviction
// victim choice (independent of the subtable hashes).
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

}  // namespace dyc
