// dyc_ops.cuh -- host launchers for the kernels of one key width. Included by
// dyc_ops4.cu and dyc_ops8.cu, which instantiate Ops<4> and Ops<8>, so the
// two widths compile as separate translation units in parallel.
#pragma once

#include <algorithm>
#include <mutex>
#include <unordered_map>

#include "dyc_set.cuh"
#include "dyc_kernels.cuh"

namespace dyc {

// Grid of a random-access kernel: one block of 256 threads per 2048 items,
// so each warp takes eight 32-item tiles. Block
// turnover keeps the SMs' fetch phases out of step, which sustains more
// random line accesses than one resident wave (find on GB300: 39.3 vs 34.2
// G/s).
// A tuner's blocks-per-SM cap (L.max_blocks_per_sm) still bounds the grid;
// the kernels are grid-stride loops.
inline int tile_grid(const LaunchCtx &L, uint64_t n) {
    uint64_t g = (n + 2047) / 2048;
    // a small batch keeps one item per thread up to a full wave of 256-thread
    // blocks (8 per SM): its latency, not the fetch rate, sets the time
    const uint64_t one_each = (n + 255) / 256, wave = 8ull * (uint64_t)(L.sms > 0 ? L.sms : 1);
    const uint64_t floor_g = one_each < wave ? one_each : wave;
    if (g < floor_g) g = floor_g;
    if (L.max_blocks_per_sm > 0) {
        const uint64_t cap = (uint64_t)L.max_blocks_per_sm * (uint64_t)(L.sms > 0 ? L.sms : 1);
        if (g > cap) g = cap;
    }
    return (int)(g < 1 ? 1 : (g > 0x7fffffffull ? 0x7fffffffull : g));
}

// Compaction: one block per tile of 256 * kCompactRun cells (a block's tile
// ends in two barriers and two atomics, so many short blocks keep more tiles
// in flight than one resident wave looping over them); the tuner's cap
// applies as for tile_grid.
inline int compact_grid(const LaunchCtx &L, uint64_t cells) {
    const uint64_t tile = 256ull * kCompactRun;
    uint64_t g = (cells + tile - 1) / tile;
    if (L.max_blocks_per_sm > 0) {
        const uint64_t cap = (uint64_t)L.max_blocks_per_sm * (uint64_t)(L.sms > 0 ? L.sms : 1);
        if (g > cap) g = cap;
    }
    return (int)(g < 1 ? 1 : (g > 0x7fffffffull ? 0x7fffffffull : g));
}

// Grid size for a grid-stride kernel: enough blocks for `work` threads, at
// most one full wave of resident blocks (occupancy x SM count).
inline int grid_for(const void *kernel, const LaunchCtx &L, uint64_t work, int block = 256) {
    static std::mutex mu;
    static std::unordered_map<const void *, int> occ;
    int per_sm;
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = occ.find(kernel);
        if (it == occ.end()) {
            int v = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kernel, block, 0) != cudaSuccess ||
                v < 1)
                v = 1;
            occ[kernel] = v;
            per_sm = v;
        } else {
            per_sm = it->second;
        }
    }
    if (L.max_blocks_per_sm > 0 && L.max_blocks_per_sm < per_sm) per_sm = L.max_blocks_per_sm;
    const uint64_t need = (work + block - 1) / block;
    const uint64_t wave = (uint64_t)per_sm * (uint64_t)(L.sms > 0 ? L.sms : 1);
    uint64_t g = need < wave ? need : wave;
    if (g < 1) g = 1;
    return (int)g;
}

#define DYC_SB_DISPATCH(sb, ...)                              \
    switch (sb) {                                             \
    case 32: { constexpr int SB = 32; __VA_ARGS__; } break;   \
    case 64: { constexpr int SB = 64; __VA_ARGS__; } break;   \
    case 128: { constexpr int SB = 128; __VA_ARGS__; } break; \
    default: return cudaErrorInvalidValue;                    \
    }

template <int KB>
cudaError_t Ops<KB>::find(const LaunchCtx &L, const Desc &D, int sb, const void *keys, void *vals,
                          uint32_t vb, uint32_t *hits, uint64_t n) {
    if (n == 0) return cudaSuccess;
    DYC_SB_DISPATCH(sb, {
        auto k = D.l2_keep ? k_find<KB, SB, true> : k_find<KB, SB, false>;
        k<<<tile_grid(L, n), 256, 0, L.stream>>>(D, keys, vals, vb, hits, n);
    });
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::dedup(const LaunchCtx &L, const Scratch &S, const void *keys, uint64_t n,
                           DedupMode mode, unsigned long long *zero, uint32_t nzero) {
    if (n == 0) return cudaSuccess;
    if (S.winbits) {
        auto c = k_dedup_clear<KB>;
        c<<<grid_for((const void *)c, L, S.dedup_cap / 2), 256, 0, L.stream>>>(
            S, mode == kKeepLast ? 0u : 0xFFFFFFFFu, n / 32 + 1, zero, nzero);
    }
    auto k = k_dedup<KB>;
    k<<<grid_for((const void *)k, L, n), 256, 0, L.stream>>>(S, keys, n, mode);
    if (winners_pass(S)) {
        auto w = k_dedup_winners<KB>;
        w<<<grid_for((const void *)w, L, S.dedup_cap), 256, 0, L.stream>>>(S);
    }
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::place(const LaunchCtx &L, const Desc &D, int sb, const Scratch &S,
                           bool use_dedup, bool new_keys, const void *keys, const void *vals,
                           uint32_t vb, uint64_t n, Counters *ctr) {
    if (n == 0) return cudaSuccess;
    DYC_SB_DISPATCH(sb, {
        auto k = D.l2_keep ? k_place<KB, SB, true> : k_place<KB, SB, false>;
        k<<<tile_grid(L, n), 256, 0, L.stream>>>(D, S, use_dedup ? 1 : 0, new_keys ? 1 : 0, keys,
                                                  vals, vb, n, ctr);
    });
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::walk(const LaunchCtx &L, const Desc &D, int sb, const void *src,
                          const unsigned long long *src_count, void *dst,
                          unsigned long long *dst_count, uint64_t dst_cap, uint32_t max_evict,
                          bool count_new, Counters *ctr, uint64_t max_entries) {
    if (max_entries == 0) return cudaSuccess;
    DYC_SB_DISPATCH(sb, {
        auto k = k_walk<KB, SB>;
        k<<<grid_for((const void *)k, L, max_entries), 256, 0, L.stream>>>(
            D, src, src_count, dst, dst_count, dst_cap, max_evict, count_new ? 1 : 0, ctr,
            max_entries);
    });
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::erase(const LaunchCtx &L, const Desc &D, int sb, const Scratch &S,
                           bool use_dedup, const void *keys, uint64_t n, uint32_t *bits,
                           Counters *ctr) {
    if (n == 0) return cudaSuccess;
    DYC_SB_DISPATCH(sb, {
        auto k = D.l2_keep ? k_erase<KB, SB, true> : k_erase<KB, SB, false>;
        k<<<tile_grid(L, n), 256, 0, L.stream>>>(D, S, use_dedup ? 1 : 0, keys, n, bits, ctr);
    });
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::apply_unique(const LaunchCtx &L, const Desc &D, int sb, const Scratch &S,
                                  const uint8_t *ops, const void *keys, const void *vals,
                                  uint32_t vb, void *vals_out, uint32_t *bits_out, uint64_t n,
                                  Counters *ctr, const uint32_t *single,
                                  const unsigned long long *gate) {
    if (n == 0) return cudaSuccess;
    DYC_SB_DISPATCH(sb, {
        auto k = D.l2_keep ? k_apply_unique<KB, SB, true> : k_apply_unique<KB, SB, false>;
        k<<<tile_grid(L, n), 256, 0, L.stream>>>(D, S, ops, keys, vals, vb, vals_out, bits_out, n,
                                                  ctr, single, gate);
    });
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::count_inserts(const LaunchCtx &L, const uint8_t *ops, uint64_t n,
                                   unsigned long long *count) {
    if (n == 0) return cudaSuccess;
    auto k = k_count_inserts<KB>;
    k<<<grid_for((const void *)k, L, n), 256, 0, L.stream>>>(ops, n, count);
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::resize_up_many(const LaunchCtx &L, int sb, const ResizeJobs &J) {
    if (J.n == 0 || J.blocks == 0) return cudaSuccess;
    DYC_SB_DISPATCH(sb, {
        auto k = k_resize_up_many<KB, SB>;
        k<<<J.blocks, 256, 0, L.stream>>>(J);
    });
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::resize_up(const LaunchCtx &L, int sb, uint32_t t, const void *old_sub,
                               uint32_t old_nb, void *new_sub) {
    if (old_nb == 0) return cudaSuccess;
    const uint32_t new_nb = 2u * old_nb;
    const uint64_t magic = fastmod_magic(new_nb);
    DYC_SB_DISPATCH(sb, {
        auto k = k_resize_up<KB, SB>;
        k<<<grid_for((const void *)k, L, (uint64_t)old_nb * (SB / 32)), 256, 0, L.stream>>>(
            t, (const char *)old_sub, old_nb, (char *)new_sub, magic);
    });
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::resize_up_list(const LaunchCtx &L, int sb, const ResizeJob *jobs,
                                    const SetPolicyOut *out, uint32_t max_jobs) {
    if (max_jobs == 0) return cudaSuccess;
    DYC_SB_DISPATCH(sb, {
        auto k = k_resize_up_list<KB, SB>;
        // one full wave; blocks loop over the listed tasks
        k<<<grid_for((const void *)k, L, ~0ull >> 1), 256, 0, L.stream>>>(jobs, out, max_jobs);
    });
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::set_policy(const LaunchCtx &L, Desc *descs, uint32_t ntables,
                                const Counters *tctr, const uint32_t *tup, const uint32_t *ter,
                                const Spare *spares, double upper, uint32_t slots, int sb,
                                ResizeJob *jobs, uint8_t *grew, SetPolicyOut *out) {
    k_set_policy<KB><<<1, 1024, 0, L.stream>>>(descs, ntables, tctr, tup, ter, spares, upper, slots,
                                               (uint32_t)sb / 32u, jobs, grew, out);
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::resize_down(const LaunchCtx &L, int sb, const void *old_sub,
                                 uint32_t old_nb, void *new_sub, void *list,
                                 unsigned long long *list_count, uint64_t list_cap,
                                 unsigned long long *spill, unsigned long long *timeouts,
                                 uint32_t tile_wait_tries) {
    const uint32_t new_nb = old_nb / 2u;
    if (new_nb == 0) return cudaSuccess;
    DYC_SB_DISPATCH(sb, {
        auto k = k_resize_down<KB, SB>;
        k<<<grid_for((const void *)k, L, new_nb, kMergeTile), kMergeTile, 0, L.stream>>>(
            (const char *)old_sub, new_nb, (char *)new_sub, list, list_count, list_cap, spill,
            timeouts, tile_wait_tries);
    });
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::collect(const LaunchCtx &L, int sb, const void *sub, uint32_t nb, void *list,
                             unsigned long long *list_count, uint64_t list_cap,
                             unsigned long long *spill) {
    if (nb == 0) return cudaSuccess;
    DYC_SB_DISPATCH(sb, {
        auto k = k_collect<KB, SB>;
        k<<<grid_for((const void *)k, L, nb), 256, 0, L.stream>>>((const char *)sub, nb, list,
                                                                  list_count, list_cap, spill);
    });
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::apply_group(const LaunchCtx &L, const ApplyScratch &A, const void *keys,
                                 uint64_t n) {
    if (n == 0) return cudaSuccess;
    auto g = k_apply_group<KB>;
    g<<<tile_grid(L, n), 256, 0, L.stream>>>(A, keys, n);
    auto c = k_apply_compact<KB>;
    c<<<compact_grid(L, 2 * n), 256, 0, L.stream>>>(A, 2 * n);
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::apply_scatter(const LaunchCtx &L, const ApplyScratch &A, uint64_t n,
                                   const uint32_t *n_ptr, const uint8_t *ops, const void *vals,
                                   uint32_t vb, void *vals_out, uint32_t *bits_out) {
    if (n == 0) return cudaSuccess;
    auto sc = k_apply_scatter<KB>;
    sc<<<tile_grid(L, n), 256, 0, L.stream>>>(A, n, n_ptr, ops, vals, vb, vals_out, bits_out);
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::apply_replay(const LaunchCtx &L, const ApplyScratch &A, const uint8_t *ops,
                                  const void *vals, uint32_t vb, void *vals_out,
                                  uint32_t *bits_out, uint64_t n, uint64_t max_distinct,
                                  const uint32_t *n_ptr) {
    if (n == 0) return cudaSuccess;
    auto r = k_apply_replay<KB>;
    const uint64_t work = n > max_distinct ? n : max_distinct;
    r<<<tile_grid(L, work), 256, 0, L.stream>>>(A, ops, vals, vb, vals_out, bits_out, n, n_ptr);
    // the segment classes are disjoint: with a side stream the warp and
    // block replays run beside the thread replay
    const bool forked = L.side != nullptr;
    cudaStream_t s2 = forked ? L.side : L.stream;
    if (forked) {
        cudaError_t e = cudaEventRecord(L.fork, L.stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(L.side, L.fork, 0);
        if (e != cudaSuccess) return e;
    }
    auto w = k_apply_replay_warp<KB>;
    // one warp per kWarpTask warp segments; at most n / (kShortSeg + 1) segments
    w<<<grid_for((const void *)w, L, (n / (kShortSeg + 1) / kWarpTask + 1) * 32), 256, 0, s2>>>(
        A, ops, vals, vb, vals_out, bits_out);
    auto m = k_apply_replay_mid<KB>;
    // one block per mid segment; at most n / (kWarpSeg + 1) of them
    m<<<grid_for((const void *)m, L, (n / (kWarpSeg + 1) + 1) * 256), 256, 0, s2>>>(
        A, ops, vals, vb, vals_out, bits_out);
    if (forked) {
        cudaError_t e = cudaEventRecord(L.join, L.side);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(L.stream, L.join, 0);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::set_group(const LaunchCtx &L, const ApplyScratch &A, const uint32_t *off,
                               const void *keys, uint64_t n, uint32_t *bits, Counters *gctr) {
    auto pr = k_set_prep<KB>;
    pr<<<grid_for((const void *)pr, L, 2 * n * (cell_bytes<KB>() / 8) + 1), 256, 0, L.stream>>>(
        A, off, bits, (unsigned long long *)gctr, (uint32_t)(sizeof(Counters) / 8));
    if (n) {  // n sizes the grids; the kernels read the op count from off[ntables]
        auto g = k_set_group<KB>;
        g<<<tile_grid(L, n), 256, 0, L.stream>>>(A, off, keys);
        auto c = k_apply_compact<KB>;
        c<<<compact_grid(L, 2 * n), 256, 0, L.stream>>>(A, 0);
    }
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::set_find(const LaunchCtx &L, const Desc *descs, uint32_t ntables, int sb,
                              const void *keys, const uint32_t *tids,
                              const unsigned long long *n_ptr, uint64_t max_n, void *vals,
                              uint32_t vb, uint32_t *hits, unsigned long long *bad, bool hint) {
    if (max_n == 0) return cudaSuccess;
    DYC_SB_DISPATCH(sb, {
        auto k = hint ? k_set_find<KB, SB, true> : k_set_find<KB, SB, false>;
        k<<<tile_grid(L, max_n), 256, 0, L.stream>>>(descs, ntables, keys, tids, n_ptr, max_n,
                                                     vals, vb, hits, bad);
    });
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::set_mutate(const LaunchCtx &L, const Desc *descs, uint32_t ntables,
                                Counters *tctr, int sb, const void *er_keys,
                                const uint32_t *er_tids, const unsigned long long *ne_ptr,
                                const void *up_keys, const void *up_vals, uint32_t vb,
                                const uint32_t *up_tids, const unsigned long long *nu_ptr,
                                uint64_t max_n, void *list_a, uint32_t *list_a_tid,
                                uint64_t list_cap, Counters *gctr, unsigned long long *bad,
                                const uint32_t *hold, bool hint) {
    if (max_n == 0) return cudaSuccess;
    DYC_SB_DISPATCH(sb, {
        auto k = hint ? k_set_mutate<KB, SB, true> : k_set_mutate<KB, SB, false>;
        k<<<tile_grid(L, max_n + 32), 256, 0, L.stream>>>(
            descs, ntables, tctr, er_keys, er_tids, ne_ptr, up_keys, up_vals, vb, up_tids, nu_ptr,
            max_n, list_a, list_a_tid, list_cap, gctr, bad, hold);
    });
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::set_unique(const LaunchCtx &L, const ApplyScratch &A, const uint32_t *off,
                                const Desc *descs, uint32_t ntables, Counters *tctr, int sb,
                                const uint8_t *ops, const void *keys, const void *vals,
                                uint32_t vb, void *vals_out, uint32_t *bits_out, uint64_t max_n,
                                void *list_a, uint32_t *list_a_tid, uint64_t list_cap,
                                Counters *gctr, const uint32_t *hold, bool hint) {
    if (max_n == 0) return cudaSuccess;
    DYC_SB_DISPATCH(sb, {
        auto k = hint ? k_set_unique<KB, SB, true> : k_set_unique<KB, SB, false>;
        k<<<tile_grid(L, max_n), 256, 0, L.stream>>>(A, off, descs, ntables, tctr, ops, keys,
                                                      vals, vb, vals_out, bits_out, list_a,
                                                      list_a_tid, list_cap, gctr, hold);
    });
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::set_walk(const LaunchCtx &L, const Desc *descs, uint32_t ntables,
                              Counters *tctr, int sb, const void *src, const uint32_t *src_tid,
                              const unsigned long long *src_count, void *dst, uint32_t *dst_tid,
                              unsigned long long *dst_count, uint64_t dst_cap, uint32_t max_evict,
                              Counters *gctr, uint64_t max_entries, unsigned long long *bad) {
    if (max_entries == 0) return cudaSuccess;
    DYC_SB_DISPATCH(sb, {
        auto k = k_set_walk<KB, SB>;
        k<<<grid_for((const void *)k, L, max_entries), 256, 0, L.stream>>>(
            descs, ntables, tctr, src, src_tid, src_count, dst, dst_tid, dst_count, dst_cap,
            max_evict, gctr, max_entries, bad);
    });
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::mark_all(const LaunchCtx &L, int sb, void *sub, uint32_t nb) {
    if (nb == 0) return cudaSuccess;
    DYC_SB_DISPATCH(sb, {
        auto k = k_mark_all<KB, SB>;
        k<<<grid_for((const void *)k, L, nb), 256, 0, L.stream>>>((char *)sub, nb);
    });
    return cudaGetLastError();
}

template <int KB>
cudaError_t Ops<KB>::export_all(const LaunchCtx &L, const Desc &D, int sb, void *keys, void *vals,
                                uint32_t vb, uint64_t cap, unsigned long long *count) {
    for (uint32_t t = 0; t < D.d; ++t) {
        const uint32_t nb = D.nb[t];
        if (nb == 0) continue;
        DYC_SB_DISPATCH(sb, {
            auto k = k_export<KB, SB>;
            k<<<grid_for((const void *)k, L, nb), 256, 0, L.stream>>>(
                (const char *)D.sub[t], nb, keys, vals, vb, cap, count);
        });
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace dyc
