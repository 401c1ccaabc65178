// dyc_set.cuh -- probe kernels of a multi-table batch (a table set): the find
// of the distinct keys, one pass for the erases and upserts, and the eviction
// walks, with the logic of the single-table kernels in dyc_kernels.cuh, but
// every item carries a table id and reads that
// table's descriptor from a device array, so one grid-stride launch serves
// the work of every table in the set. Item counts are read on the device
// (the counters the mixed-batch kernels fill), so a batch's launch sequence
// needs no host reads and can be captured as a CUDA graph. Such a count is
// clamped to the capacity of the list behind it and a table id at or above
// the table count skips its item; both are counted in *bad, which the host
// turns into an error, so a wrong count can never index past a buffer. A
// null table-id array means table 0 for every item: a single table's mixed
// batch runs through the same kernels with a one-entry descriptor array.
#pragma once

#include "dyc_apply.cuh"

namespace dyc {

// Per-table size change by `sign` for every lane with pred; one atomic per
// distinct table in the warp. All 32 lanes must call.
__device__ __forceinline__ void warp_size_add(Counters *tctr, uint32_t t, bool pred,
                                              long long sign) {
    const unsigned peers = __match_any_sync(kFull, pred ? t : 0xffffffffu);
    if (pred && (__ffs(peers) - 1) == (int)(threadIdx.x & 31))
        atomicAdd(&tctr[t].size, (unsigned long long)(sign * (long long)__popc(peers)));
}

// A count read on the device, clamped to cap (the capacity of the list it
// counts); an excess is recorded in *bad by one thread.
__device__ __forceinline__ uint64_t clamped_count(const unsigned long long *p, uint64_t cap,
                                                  unsigned long long *bad) {
    const uint64_t n = *p;
    if (n <= cap) return n;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(bad, 1ull);
    return cap;
}

// Table id of item i (0 without an id array); an id at or above ntables is
// recorded in *bad and the item is dropped from the pass (ok = false).
__device__ __forceinline__ uint32_t checked_tid(const uint32_t *tids, uint64_t i,
                                                uint32_t ntables, unsigned long long *bad,
                                                bool &ok) {
    const uint32_t t = tids ? tids[i] : 0u;
    if (t < ntables) return t;
    atomicAdd(bad, 1ull);
    ok = false;
    return 0u;
}

// find of keys[i] in table tids[i], i < *n_ptr (k_find per table)
template <int KB, int SB, bool HINT>
__global__ void __launch_bounds__(256) k_set_find(const Desc *__restrict__ descs, uint32_t ntables,
                                                  const void *__restrict__ keys,
                                                  const uint32_t *__restrict__ tids,
                                                  const unsigned long long *__restrict__ n_ptr,
                                                  uint64_t max_n, void *__restrict__ vals,
                                                  uint32_t vb, uint32_t *__restrict__ hits,
                                                  unsigned long long *bad) {
    using T = SlotT<KB>;
    using Gm = Geo<KB, SB>;
    __shared__ __align__(128) unsigned char s_stage[kWarpsPerBlock][32 * SB];
    unsigned char *stage = s_stage[threadIdx.x >> 5];
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t n = clamped_count(n_ptr, max_n, bad);
    const uint64_t step = warp_stride();
    for (uint64_t base = warp_base(); base < n; base += step) {
        const uint64_t i = base + lane;
        typename T::K k = 0;
        uint32_t tb = 0u;
        bool ok = true;
        if (i < n) {
            k = load_key<KB>(keys, i);
            tb = checked_tid(tids, i, ntables, bad, ok);
        }
        const Desc &D = descs[tb];
        const bool act = ok && k != 0;
        const unsigned long long tpol = HINT ? l2_policies(D.l2_keep != 0u).table : 0ull;
        const uint32_t hk = fold(k);
        const Pair p = pair_of(hk, D.d);
        const char *p1 = bucket_ptr<KB, SB>(D, p.first, bucket_index(D, p.first, hk));
        const KvOut r1 = kv_probe<KB, SB, 1, HINT>(p1, k, act, stage, tpol);
        bool hit = act && r1.match >= 0;
        uint64_t v = hit ? r1.value : 0ull;
        const bool need2 = act && !hit && (!Gm::kMeta || r1.overflow);
        if (__any_sync(kFull, need2)) {
            const char *p2 = bucket_ptr<KB, SB>(D, p.second, bucket_index(D, p.second, hk));
            const KvOut r2 = kv_probe<KB, SB, 1, HINT>(p2, k, need2, stage, tpol);
            if (need2 && r2.match >= 0) {
                hit = true;
                v = r2.value;
            }
        }
        if (i < n) store_val(vals, vb, i, v);
        const unsigned m = __ballot_sync(kFull, hit);
        if (hits != nullptr && lane == 0) hits[base >> 5] = m;
    }
}

// erase of unique keys[i] from table tids[i], i in [base, base + 32) and
// below n (k_erase per table, no dedup). Warp-collective; returns whether
// this lane erased its key.
template <int KB, int SB, bool HINT>
__device__ __forceinline__ bool set_erase_warp(const Desc *__restrict__ descs, uint32_t ntables,
                                               Counters *__restrict__ tctr,
                                               const void *__restrict__ keys,
                                               const uint32_t *__restrict__ tids, uint64_t n,
                                               uint64_t base, unsigned char *stage,
                                               unsigned long long *bad) {
    using T = SlotT<KB>;
    using Gm = Geo<KB, SB>;
    const uint64_t i = base + (threadIdx.x & 31);
    typename T::K k = 0;
    uint32_t tb = 0u;
    bool ok = true;
    if (i < n) {
        k = load_key<KB>(keys, i);
        tb = checked_tid(tids, i, ntables, bad, ok);
    }
    const Desc &D = descs[tb];
    const bool act = ok && k != 0;
    const unsigned long long tpol = HINT ? l2_policies(D.l2_keep != 0u).table : 0ull;
    const uint32_t hk = fold(k);
    const Pair p = pair_of(hk, D.d);
    char *p1 = bucket_ptr<KB, SB>(D, p.first, bucket_index(D, p.first, hk));
    const KvOut r1 = kv_probe<KB, SB, 2, HINT>(p1, k, act, stage, tpol);
    // plain stores, as in k_erase: the erase and upsert lists name distinct
    // keys, so no other thread of the pass writes a found key's slot
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
    warp_size_add(tctr, tb, erased, -1);
    return erased;
}

// upsert of unique keys[i] -> vals[i] into table tids[i], i in [base,
// base + 32) and below n (k_place per table); ops left without a slot go to
// list_a / list_a_tid. Warp-collective; adds to n_ins / n_upd.
template <int KB, int SB, bool HINT>
__device__ __forceinline__ void set_place_warp(const Desc *__restrict__ descs, uint32_t ntables,
                                               Counters *__restrict__ tctr,
                                               const void *__restrict__ keys,
                                               const void *__restrict__ vals, uint32_t vb,
                                               const uint32_t *__restrict__ tids, uint64_t n,
                                               uint64_t base, void *list_a, uint32_t *list_a_tid,
                                               uint64_t list_cap, Counters *gctr,
                                               unsigned char *stage, uint32_t &n_ins,
                                               uint32_t &n_upd, unsigned long long *bad) {
    using T = SlotT<KB>;
    using Sl = typename T::S;
    using Gm = Geo<KB, SB>;
    const uint64_t i = base + (threadIdx.x & 31);
    typename T::K k = 0;
    bool act = false;
    uint32_t tb = 0u;
    Sl e = T::empty();
    if (i < n) {
        bool ok = true;
        k = load_key<KB>(keys, i);
        tb = checked_tid(tids, i, ntables, bad, ok);
        act = ok && k != 0;
        if (act) e = T::make(k, load_val(vals, vb, i));
    }
    const Desc &D = descs[tb];
    const unsigned long long tpol = HINT ? l2_policies(D.l2_keep != 0u).table : 0ull;
    const uint32_t hk = fold(k);
    const Pair p = pair_of(hk, D.d);
    char *p1 = bucket_ptr<KB, SB>(D, p.first, bucket_index(D, p.first, hk));
    char *p2 = bucket_ptr<KB, SB>(D, p.second, bucket_index(D, p.second, hk));
    const KvOut r1 = place_probe<KB, SB, HINT>(p1, k, act, p.first, D.d, stage, tpol);
    const bool found1 = act && r1.match >= 0;
    const bool check2 = act && !found1 && ((!Gm::kMeta || r1.overflow) || r1.empty == 0u);
    KvOut r2{-1, 0ull, false, 0u};
    if (__any_sync(kFull, check2))
        r2 = place_probe<KB, SB, HINT>(p2, k, check2, p.second, D.d, stage, tpol);
    bool pend = false, ins = false;
    if (found1) {  // the key's own slot: a plain store (distinct keys, as in k_place)
        T::store(slot_ptr<KB, SB>(p1, r1.match), e);
        ++n_upd;
    } else if (check2 && r2.match >= 0) {
        T::store(slot_ptr<KB, SB>(p2, r2.match), e);
        ++n_upd;
    } else if (act) {
        bool ok = claim_empty<KB, SB>(p1, r1.empty, e);
        if (!ok && check2 && r2.empty) {
            mark_overflow<KB, SB>(p1, hk);
            ok = claim_empty<KB, SB>(p2, r2.empty, e);
        }
        if (ok) {
            ++n_ins;
            ins = true;
        } else {
            pend = true;
        }
    }
    __syncwarp();
    warp_size_add(tctr, tb, ins, 1);
    const unsigned long long at = agg_inc(&gctr->pending, pend);
    if (pend) {
        if (at < list_cap) {
            ((Sl *)list_a)[at] = e;
            if (list_a_tid) list_a_tid[at] = tb;
        } else {
            atomicAdd(&gctr->spill, 1ull);
        }
    }
}

// The batch's erases (er_keys, *ne_ptr of them) and upserts (up_keys,
// *nu_ptr) in one grid-stride pass: warp items [0, ceil32(ne)) erase, the
// rest upsert. The keys of the two lists are distinct, so the two kinds may
// run concurrently (an upsert only claims empty slots or rewrites its own
// key; an erase only empties its own key's slot).
template <int KB, int SB, bool HINT>
__global__ void __launch_bounds__(256) k_set_mutate(
    const Desc *__restrict__ descs, uint32_t ntables, Counters *__restrict__ tctr,
    const void *__restrict__ er_keys, const uint32_t *__restrict__ er_tids,
    const unsigned long long *__restrict__ ne_ptr, const void *__restrict__ up_keys,
    const void *__restrict__ up_vals, uint32_t vb, const uint32_t *__restrict__ up_tids,
    const unsigned long long *__restrict__ nu_ptr, uint64_t max_n, void *list_a,
    uint32_t *list_a_tid, uint64_t list_cap, Counters *gctr, unsigned long long *bad,
    const uint32_t *hold) {
    if (hold != nullptr && *hold != 0u) return;  // the host applies the rest of the policy first
    __shared__ __align__(128) unsigned char s_stage[kWarpsPerBlock][32 * SB];
    unsigned char *stage = s_stage[threadIdx.x >> 5];
    const uint64_t ne = clamped_count(ne_ptr, max_n, bad), nu = clamped_count(nu_ptr, max_n, bad);
    const uint64_t ne32 = (ne + 31) & ~(uint64_t)31;
    const uint64_t step = warp_stride();
    uint32_t n_del = 0, n_ins = 0, n_upd = 0;
    for (uint64_t base = warp_base(); base < ne32 + nu; base += step) {
        if (base < ne32) {  // warp-uniform: base is a multiple of 32
            n_del += set_erase_warp<KB, SB, HINT>(descs, ntables, tctr, er_keys, er_tids, ne, base,
                                            stage, bad)
                         ? 1u
                         : 0u;
        } else {
            set_place_warp<KB, SB, HINT>(descs, ntables, tctr, up_keys, up_vals, vb, up_tids, nu,
                                   base - ne32, list_a, list_a_tid, list_cap, gctr, stage, n_ins,
                                   n_upd, bad);
        }
    }
    // one atomic per counter per block (the grid has many short-lived blocks)
    __shared__ unsigned long long s_sum[3];
    if (threadIdx.x < 3) s_sum[threadIdx.x] = 0ull;
    __syncthreads();
    n_del = __reduce_add_sync(kFull, n_del);
    n_ins = __reduce_add_sync(kFull, n_ins);
    n_upd = __reduce_add_sync(kFull, n_upd);
    if ((threadIdx.x & 31) == 0) {
        if (n_del) atomicAdd(&s_sum[0], (unsigned long long)n_del);
        if (n_ins) atomicAdd(&s_sum[1], (unsigned long long)n_ins);
        if (n_upd) atomicAdd(&s_sum[2], (unsigned long long)n_upd);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_sum[0]) atomicAdd(&gctr->erased, s_sum[0]);
        if (s_sum[1]) atomicAdd(&gctr->inserted, s_sum[1]);
        if (s_sum[2]) atomicAdd(&gctr->updated, s_sum[2]);
    }
}

// The ops of a set batch whose key has no other op in it (and key-0 ops),
// after the device policy's upsizes and before the mutation of the repeated
// keys (ApplyScratch::single_pass): each resolved in one probe of its
// table's buckets, as k_apply_unique does for one table. The result is the
// key's state before the batch; an insert updates in place or claims an
// empty slot, else goes to list_a with its table; an erase of a present key
// clears its slot. Hit bits are ORed in (the scatter and the replays wrote
// the repeated keys' bits). The other phase-B kernels touch only repeated
// keys, so no key is probed by two kernels at once.
template <int KB, int SB, bool HINT>
__global__ void __launch_bounds__(256) k_set_unique(
    const __grid_constant__ ApplyScratch A, const uint32_t *__restrict__ off,
    const Desc *__restrict__ descs, uint32_t ntables, Counters *__restrict__ tctr,
    const uint8_t *__restrict__ ops, const void *__restrict__ keys, const void *__restrict__ vals,
    uint32_t vb, void *__restrict__ vals_out, uint32_t *__restrict__ bits_out, void *list_a,
    uint32_t *list_a_tid, uint64_t list_cap, Counters *gctr, const uint32_t *hold) {
    using T = SlotT<KB>;
    using Sl = typename T::S;
    using Gm = Geo<KB, SB>;
    if (hold != nullptr && *hold != 0u) return;  // the host applies the rest of the policy first
    __shared__ __align__(128) unsigned char s_stage[kWarpsPerBlock][32 * SB];
    unsigned char *stage = s_stage[threadIdx.x >> 5];
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t n = set_op_count(A, off);
    const uint64_t step = warp_stride();
    uint32_t n_ins = 0, n_upd = 0, n_del = 0;
    for (uint64_t base = warp_base(); base < n; base += step) {
        const uint64_t i = base + lane;
        bool mine = i < n && ((A.single[i >> 5] >> (i & 31)) & 1u);  // the scatter's bitmap
        uint32_t tb = 0u;
        typename T::K k = 0;
        uint8_t op = kOpFind;
        Sl e = T::empty();
        if (mine) {
            tb = table_at(A.tidx, off, (uint32_t)i, (uint32_t)i);
            if (tb >= ntables) {
                note_bad(A);
                mine = false;
                tb = 0u;
            } else {
                k = load_key<KB>(keys, i);
                op = ops[i];
            }
        }
        const Desc &D = descs[tb];
        const unsigned long long tpol = HINT ? l2_policies(D.l2_keep != 0u).table : 0ull;
        const bool act = mine && k != 0;  // ops on key 0 miss and change nothing
        const bool ins = act && op == kOpInsert, del = act && op == kOpErase;
        if (ins) e = T::make(k, load_val(vals, vb, i));
        const uint32_t hk = fold(k);
        const Pair p = pair_of(hk, D.d);
        char *p1 = bucket_ptr<KB, SB>(D, p.first, bucket_index(D, p.first, hk));
        char *p2 = bucket_ptr<KB, SB>(D, p.second, bucket_index(D, p.second, hk));
        const KvOut r1 = place_probe<KB, SB, HINT>(p1, k, act, p.first, D.d, stage, tpol);
        const bool found1 = act && r1.match >= 0;
        const bool check2 =
            act && !found1 && ((!Gm::kMeta || r1.overflow) || (ins && r1.empty == 0u));
        KvOut r2{-1, 0ull, false, 0u};
        if (__any_sync(kFull, check2))
            r2 = place_probe<KB, SB, HINT>(p2, k, check2, p.second, D.d, stage, tpol);
        const bool found2 = check2 && r2.match >= 0;
        const bool present = found1 || found2;
        const uint64_t before = found1 ? r1.value : (found2 ? r2.value : 0ull);
        bool pend = false, placed = false, gone = false;
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
                if (ok) {
                    ++n_ins;
                    placed = true;
                } else {
                    pend = true;
                }
            }
        } else if (del && present) {
            T::store(found1 ? slot_ptr<KB, SB>(p1, r1.match) : slot_ptr<KB, SB>(p2, r2.match),
                     T::empty());
            ++n_del;
            gone = true;
        }
        if (vals_out != nullptr && mine) store_val(vals_out, vb, i, before);
        const unsigned m = __ballot_sync(kFull, present);
        if (bits_out != nullptr && lane == 0 && m) atomicOr(&bits_out[base >> 5], m);
        __syncwarp();
        warp_size_add(tctr, tb, placed, 1);
        warp_size_add(tctr, tb, gone, -1);
        const unsigned long long at = agg_inc(&gctr->pending, pend);
        if (pend) {
            if (at < list_cap) {
                ((Sl *)list_a)[at] = e;
                if (list_a_tid) list_a_tid[at] = tb;
            } else {
                atomicAdd(&gctr->spill, 1ull);
            }
        }
    }
    // one atomic per counter per block
    __shared__ unsigned long long s_sum[3];
    if (threadIdx.x < 3) s_sum[threadIdx.x] = 0ull;
    __syncthreads();
    n_del = __reduce_add_sync(kFull, n_del);
    n_ins = __reduce_add_sync(kFull, n_ins);
    n_upd = __reduce_add_sync(kFull, n_upd);
    if (lane == 0) {
        if (n_del) atomicAdd(&s_sum[0], (unsigned long long)n_del);
        if (n_ins) atomicAdd(&s_sum[1], (unsigned long long)n_ins);
        if (n_upd) atomicAdd(&s_sum[2], (unsigned long long)n_upd);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_sum[0]) atomicAdd(&gctr->erased, s_sum[0]);
        if (s_sum[1]) atomicAdd(&gctr->inserted, s_sum[1]);
        if (s_sum[2]) atomicAdd(&gctr->updated, s_sum[2]);
    }
}

// eviction walks of src entries (k_walk per table, each with its own
// eviction bound; max_evict, the largest, bounds the cooperative loop);
// failures go to dst
template <int KB, int SB>
__global__ void __launch_bounds__(256) k_set_walk(const Desc *__restrict__ descs, uint32_t ntables,
                                                  Counters *__restrict__ tctr,
                                                  const void *__restrict__ src,
                                                  const uint32_t *__restrict__ src_tid,
                                                  const unsigned long long *src_count, void *dst,
                                                  uint32_t *dst_tid, unsigned long long *dst_count,
                                                  uint64_t dst_cap, uint32_t max_evict,
                                                  Counters *gctr, uint64_t max_entries,
                                                  unsigned long long *bad) {
    using T = SlotT<KB>;
    using Sl = typename T::S;
    __shared__ unsigned long long s_sum[2];
    if (threadIdx.x < 2) s_sum[threadIdx.x] = 0ull;
    __syncthreads();
    // (more entries than max_entries means entries were already counted in
    // spill by the kernel that listed them)
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
            const uint32_t tb = live ? checked_tid(src_tid, i, ntables, bad, live) : 0u;
            const Desc &D = descs[tb];
            uint32_t hk = 0;
            Pair pe{0u, 0u};
            char *fb = first_bucket<KB, SB>(D, T::key(e), pe, hk);
            uint32_t t = pe.first;
            char *bp = fb;
            // 0: empties of the first bucket, 1: of the second, 2: walking. The
            // entries come from the upsert pass, which found both buckets full:
            // the walk starts at the first bucket (still taking an empty slot
            // there if one has appeared since).
            int mode = 2;
            uint32_t evictions = 0;
            bool fail = false, ok = false;
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
                    ok = true;
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
                } else if (evictions >= D.max_evict) {  // this table's bound
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
                        ok = true;
                    } else {
                        e = old;  // a resident of the same table
                        fb = first_bucket<KB, SB>(D, T::key(e), pe, hk);
                        t = other_of(pe, t);
                        bp = bucket_ptr<KB, SB>(D, t, bucket_index(D, t, hk));
                    }
                }
            }
            if (live) fail = true;  // iteration bound reached
            __syncwarp();
            n_ok += ok ? 1u : 0u;
            warp_size_add(tctr, tb, ok, 1);
            const unsigned long long at = agg_inc(dst_count, fail);
            if (fail) {
                if (at < dst_cap) {
                    ((Sl *)dst)[at] = e;
                    if (dst_tid) dst_tid[at] = tb;
                } else {
                    atomicAdd(&gctr->spill, 1ull);
                }
            }
        }
    } else {
        for (uint64_t i = wid; i < n; i += warps) {
            const Sl e = ((const Sl *)src)[i];
            const uint32_t tb = src_tid ? src_tid[i] : 0u;  // warp-uniform
            if (tb >= ntables) {
                if (lead) atomicAdd(bad, 1ull);
                continue;
            }
            const Desc &D = descs[tb];
            const WalkOut<KB> w = walk_lookahead<KB, SB>(D, e, D.max_evict);
            if (!lead) continue;
            n_steps += w.steps;
            if (w.ok) {
                ++n_ok;
                atomicAdd(&tctr[tb].size, 1ull);
            } else {
                const unsigned long long at = atomicAdd(dst_count, 1ull);
                if (at < dst_cap) {
                    ((Sl *)dst)[at] = w.left;
                    if (dst_tid) dst_tid[at] = tb;
                } else {
                    atomicAdd(&gctr->spill, 1ull);
                }
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
        if (s_sum[0]) atomicAdd(&gctr->inserted, s_sum[0]);
        if (s_sum[1]) atomicAdd(&gctr->evict_steps, s_sum[1]);
    }
}

// ----------------------------------------------------------------------------
// Device half of a set round's upsize policy, between phase A (which counted
// each member's upserts tup[t] and erases ter[t]) and phase B (which applies
// them). The rule is the host's (hash_insert_batch, api.cpp:359-369, per
// member): upsize while size - erases + upserts > upper x capacity. Here a
// member over the bound is upsized once, into its spare (Spare: a subtable
// of twice the buckets of the one pick_up_index names, allocated by the
// host before the round); its descriptor switches to the spare at once and
// the move is listed for k_resize_up_list, which runs before phase B. A
// member still over the bound after that upsize, or without a fitting
// spare, sets out->host: phase B's mutate kernel then does nothing and the
// host applies the rest of the policy before running phase B itself. The
// capacity and the comparison are the host's, in doubles. One block walks
// the members in tiles of blockDim.x (a scan gives each listed move its
// place and its first task).
// ----------------------------------------------------------------------------
template <int KB>
__global__ void __launch_bounds__(1024) k_set_policy(Desc *__restrict__ descs, uint32_t ntables,
                                                     const Counters *__restrict__ tctr,
                                                     const uint32_t *__restrict__ tup,
                                                     const uint32_t *__restrict__ ter,
                                                     const Spare *__restrict__ spares, double upper,
                                                     uint32_t slots, uint32_t chunks_per_bucket,
                                                     ResizeJob *__restrict__ jobs,
                                                     uint8_t *__restrict__ grew,
                                                     SetPolicyOut *__restrict__ out) {
    __shared__ uint32_t s_wj[32], s_wt[32];  // per-warp inclusive sums of the tile
    __shared__ uint32_t s_cj, s_ct, s_host;   // jobs / tasks before the tile; host needed
    const uint32_t tid = threadIdx.x, lane = tid & 31u, w = tid >> 5, nw = blockDim.x >> 5;
    if (tid == 0) {
        s_cj = 0u;
        s_ct = 0u;
        s_host = 0u;
    }
    __syncthreads();
    for (uint32_t base = 0; base < ntables; base += blockDim.x) {
        const uint32_t t = base + tid;
        uint32_t want = 0u, tasks = 0u, ti = 0u, onb = 0u;
        if (t < ntables) {
            const Desc &D = descs[t];
            const uint32_t d = D.d < (uint32_t)kMaxSub ? D.d : (uint32_t)kMaxSub;
            uint64_t nbs = 0;
            for (uint32_t i = 0; i < d; ++i) nbs += D.nb[i];
            const double cap = (double)(nbs * slots);
            const double bse = (double)tctr[t].size - (double)ter[t];
            const double up = (double)tup[t];
            if (tup[t] != 0u && bse + up > upper * cap) {
                ti = pick_up_index(D.nb, d);
                onb = D.nb[ti];
                const Spare sp = spares[t];
                if (sp.new_sub != nullptr && sp.ti == ti && sp.old_nb == onb && onb != 0u &&
                    onb <= 0x7fffffffu) {
                    want = 1u;
                    tasks = (uint32_t)(((uint64_t)onb * chunks_per_bucket + kResizeChunksPerBlock -
                                        1) / kResizeChunksPerBlock);
                    if (bse + up > upper * (cap + (double)((uint64_t)onb * slots))) s_host = 1u;
                } else {
                    s_host = 1u;
                }
            }
            grew[t] = (uint8_t)want;
        }
        // place of this member's move among the tile's (exclusive scans)
        uint32_t ij = want, it = tasks;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t a = __shfl_up_sync(kFull, ij, o), b = __shfl_up_sync(kFull, it, o);
            if (lane >= (uint32_t)o) {
                ij += a;
                it += b;
            }
        }
        if (lane == 31u) {
            s_wj[w] = ij;
            s_wt[w] = it;
        }
        __syncthreads();
        if (w == 0) {
            uint32_t vj = lane < nw ? s_wj[lane] : 0u, vt = lane < nw ? s_wt[lane] : 0u;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t a = __shfl_up_sync(kFull, vj, o), b = __shfl_up_sync(kFull, vt, o);
                if (lane >= (uint32_t)o) {
                    vj += a;
                    vt += b;
                }
            }
            if (lane < nw) {
                s_wj[lane] = vj;
                s_wt[lane] = vt;
            }
        }
        __syncthreads();
        if (want) {
            const uint32_t pj = s_cj + (w ? s_wj[w - 1] : 0u) + ij - want;
            const uint32_t pt = s_ct + (w ? s_wt[w - 1] : 0u) + it - tasks;
            Desc &D = descs[t];
            void *nw_sub = spares[t].new_sub;
            const uint32_t nnb = 2u * onb;
            const uint64_t mg = fastmod_magic(nnb);
            jobs[pj] = ResizeJob{D.sub[ti], nw_sub, mg, onb, ti, pt, t};
            D.sub[ti] = nw_sub;
            D.nb[ti] = nnb;
            D.magic[ti] = mg;
        }
        __syncthreads();  // the carries and the warp sums are read above
        if (tid == 0) {
            s_cj += s_wj[nw - 1];
            s_ct += s_wt[nw - 1];
        }
        __syncthreads();
    }
    if (tid == 0) {
        out->njobs = s_cj;
        out->ntasks = s_ct;
        out->host = s_host;
        out->pad = 0u;
    }
}

}  // namespace dyc
