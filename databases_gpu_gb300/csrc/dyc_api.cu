// dyc_api.cu -- the C ABI of include/dycuckoo.h: table lifetime, sizing and
// resize policy (GPU/dyhash/api.cpp), the library's allocation pool, batch
// chunking, the no-loss overflow loop, mixed batches, table sets (their
// launch graphs and upsize waves), snapshots, wide values, and the
// host-buffer forms of the hashAPI calls.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <memory>
#include <mutex>
#include <string>
#include <map>
#include <vector>

#include "dycuckoo.h"
#include "dyc_device.cuh"
#include "dyc_internal.h"

using dyc::Counters;
using dyc::Desc;
using dyc::LaunchCtx;
using dyc::Ops;
using dyc::Scratch;

namespace dyc {
std::atomic<unsigned long long> g_lib_allocs{0};
}

namespace {

thread_local std::string g_err;

dyc_status fail(dyc_status s, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return s;
}

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(e_ == cudaErrorMemoryAllocation ? DYC_ENOMEM : DYC_ECUDA,         \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

#define TRY(expr)                       \
    do {                                \
        dyc_status s_ = (expr);         \
        if (s_ != DYC_OK) return s_;    \
    } while (0)

// --- sizing: isPrime / nextPrime / buckets per subtable (api.cpp:4-22, :46-56)
bool is_prime_ref(int32_t num) {
    if (num == 2 || num == 3) return true;
    if (num % 6 != 1 && num % 6 != 5) return false;
    for (int32_t i = 5; (int64_t)i * i <= num; i += 6)
        if (num % i == 0 || num % (i + 2) == 0) return false;
    return true;
}
uint32_t next_prime_ref(uint32_t n) {
    while (!is_prime_ref((int32_t)n)) ++n;
    return n;
}

// resize target choice (api.cpp:115-122 and :147-153); the upsize rule is
// shared with the device half of a set's policy (dyc::pick_up_index)
uint32_t pick_up(const uint32_t *nb, uint32_t d) { return dyc::pick_up_index(nb, d); }
uint32_t pick_down(const uint32_t *nb, uint32_t d) {
    for (uint32_t i = 0; i + 1 < d; ++i)
        if (nb[i] > nb[i + 1]) return i;
    return d - 1;
}

uint64_t next_pow2(uint64_t x) {
    uint64_t p = 1;
    while (p < x) p <<= 1;
    return p;
}

// Library-owned stream-ordered memory pool per device for everything a
// resize allocates and frees (subtables, entry lists, value heaps). The
// default pool hands freed memory back to the driver at every
// synchronisation, so each resize mapped fresh physical memory (a 1.27 GB
// upsize spent most of its 4.4 ms there); this pool keeps up to a quarter of
// the device's memory cached for the next resize, and is trimmed when the
// last table on the device is destroyed.
std::mutex g_pool_mu;
constexpr int kPoolDevices = 256;
cudaMemPool_t g_pool[kPoolDevices];
int g_pool_tables[kPoolDevices];

cudaError_t lib_pool(int device, cudaMemPool_t *out) {
    if (device < 0 || device >= kPoolDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> g(g_pool_mu);
    if (!g_pool[device]) {
        cudaMemPoolProps props;
        memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        cudaMemPool_t p = nullptr;
        cudaError_t e = cudaMemPoolCreate(&p, &props);
        if (e != cudaSuccess) return e;
        size_t free_b = 0, total_b = 0;
        e = cudaMemGetInfo(&free_b, &total_b);
        if (e != cudaSuccess) return e;
        uint64_t keep = total_b / 4;
        e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
        if (e != cudaSuccess) return e;
        g_pool[device] = p;
    }
    *out = g_pool[device];
    return cudaSuccess;
}

void pool_table_count(int device, int delta) {
    if (device < 0 || device >= kPoolDevices) return;
    std::lock_guard<std::mutex> g(g_pool_mu);
    g_pool_tables[device] += delta;
    if (g_pool_tables[device] == 0 && g_pool[device]) cudaMemPoolTrimTo(g_pool[device], 0);
}

constexpr uint64_t kChunkDefault = 1ull << 22;  // ops per insert/erase pass
constexpr int kMaxOverflowRounds = 24;

}  // namespace

struct dyc_table {
    dyc_config cfg;
    int kb, vb, sb, slot_bytes, slots;
    int device, sms;
    Desc D;
    Counters *d_ctr = nullptr;
    Counters *h_ctr = nullptr;
    bool owns_ctr = true;  // false for a member of a table set (the set's arrays)
    bool counted = false;  // counted among the live tables of its device's pool
    // scratch for one chunk
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    Scratch S{};
    uint64_t chunk = kChunkDefault;
    // mixed-batch scratch (dyc_apply), allocated on first use
    void *apply_buf = nullptr;
    size_t apply_bytes = 0;
    dyc::ApplyScratch A{};
    unsigned long long *h_actr = nullptr;  // pinned copy of A.ctr
    Desc *d_desc = nullptr;  // device copy of D for the mixed-batch probe kernels
    Desc *h_desc = nullptr;  // its pinned mirror (the last pushed state)
    // host-form staging
    cudaStream_t io_stream = nullptr;
    void *d_io = nullptr;
    size_t d_io_bytes = 0;
    // dyc_find_host pipeline: one stream and one device buffer per stage
    cudaStream_t pipe_stream[3] = {nullptr, nullptr, nullptr};
    void *pipe_buf[3] = {nullptr, nullptr, nullptr};
    size_t pipe_bytes = 0;
    uint64_t size = 0, capacity = 0;
    dyc_op_stats last{};
    // entries a failed call could not place (slot images, held_n of them);
    // not in the device size counter; the next call places them first
    std::vector<unsigned char> held;
    uint64_t held_n = 0;
};

namespace {

// Desc::l2_keep from cfg.l2_resident: 2 asks the L2 to keep the table's
// bucket lines (evict_last hints on every probe, evict_first on the find's
// key and result streams); 0 and 1 use plain accesses. Measured on GB300
// with the find kernel: a table of 1.2x the L2 (2^24 keys) found 48.1 G/s
// with the hints and 51.1 G/s with plain loads (Zipf 0.99: 35.0 both); at
// 2^28 keys hinted loads even at evict_normal priority ran Zipf batches at
// 15.6 G/s against 39.4 plain (many warps reading one hot line), and tables
// of up to half the L2 stay resident under any policy. So the hints are
// opt-in, and kernels take them only through their HINT instantiation.
void refresh_l2(dyc_table *t) { t->D.l2_keep = t->cfg.l2_resident == 2u ? 1u : 0u; }

dyc_status set_device(dyc_table *t) {
    int cur = -1;
    CK(cudaGetDevice(&cur));
    if (cur != t->device) CK(cudaSetDevice(t->device));
    return DYC_OK;
}

LaunchCtx ctx(dyc_table *t, void *stream) { return LaunchCtx{t->sms, (cudaStream_t)stream}; }

// Failure injection for the tests of the error paths (dyc_debug_inject):
// the n-th pool allocation from now fails as if the device were out of
// memory; the downsize kernel's tile-copy waits give up after this many
// polls. Process-wide.
std::atomic<uint64_t> g_inject_alloc{0};
std::atomic<uint32_t> g_inject_wait_tries{dyc::kWaitTries};
std::atomic<uint64_t> g_inject_chunk{0};  // ops per insert / erase chunk of new tables (0: default)

// Stream-ordered allocation from the library pool of the table's device.
cudaError_t pool_alloc(int device, void **p, size_t bytes, cudaStream_t s) {
    for (uint64_t c = g_inject_alloc.load(); c != 0;) {
        if (g_inject_alloc.compare_exchange_weak(c, c - 1)) {
            if (c == 1) return cudaErrorMemoryAllocation;
            break;
        }
    }
    cudaMemPool_t pool = nullptr;
    cudaError_t e = lib_pool(device, &pool);
    if (e != cudaSuccess) return e;
    dyc::g_lib_allocs.fetch_add(1, std::memory_order_relaxed);
    return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

// dispatch on key width
#define KB_CALL(t, fn, ...) ((t)->kb == 4 ? Ops<4>::fn(__VA_ARGS__) : Ops<8>::fn(__VA_ARGS__))

// Make the scratch lists hold `n` ops (grow only).
// Dedup cells for a chunk of n ops: a power of two, at most half full, and
// at most a quarter full while that stays within 2^22 cells (32 MB of 8-byte
// cells, which stay in the L2 beside the bucket lines). Fewer probes per
// claim pay there: 2^19-key calls on an L2-resident table went from 5.1 to
// 5.9 G ops/s (insert) and 8.2 to 8.8 (erase). A larger table at a quarter
// load spills the L2: 4M-op chunks on a 2^28-key table lost 10 %.
uint64_t dedup_cells(uint64_t n) {
    const uint64_t m = n < 16 ? 16 : n;
    const uint64_t quarter = next_pow2(4 * m);
    return quarter <= (1ull << 22) ? quarter : next_pow2(2 * m);
}

dyc_status ensure_scratch(dyc_table *t, uint64_t n) {
    const uint64_t cap = dedup_cells(n);
    const size_t dedup_bytes = (size_t)cap * 8;
    const size_t idx_bytes = t->kb == 8 ? (size_t)cap * 4 : 0;
    const size_t list_bytes = (size_t)n * t->slot_bytes;
    const size_t win_bytes = (size_t)(n / 32 + 1) * 4;
    const size_t need = dedup_bytes + idx_bytes + 2 * list_bytes + win_bytes + 256 + 5 * 256;
    if (t->scratch && t->scratch_bytes >= need && t->S.list_cap >= n && t->S.dedup_cap >= cap)
        return DYC_OK;
    if (t->scratch) {
        CK(cudaDeviceSynchronize());
        CK(cudaFree(t->scratch));
        t->scratch = nullptr;
    }
    CK(dyc::lib_malloc(&t->scratch, need));
    t->scratch_bytes = need;
    char *p = (char *)t->scratch;
    auto carve = [&](size_t bytes) {
        char *r = p;
        p += (bytes + 255) & ~(size_t)255;
        return (void *)r;
    };
    t->S.dedup = carve(dedup_bytes);
    t->S.dedup_idx = idx_bytes ? (uint32_t *)carve(idx_bytes) : nullptr;
    t->S.dedup_cap = cap;
    t->S.list_a = carve(list_bytes);
    t->S.list_b = carve(list_bytes);
    t->S.list_cap = n;
    t->S.winbits = (uint32_t *)carve(win_bytes);
    t->S.dupseen = (uint32_t *)carve(4);
    return DYC_OK;
}

dyc_status reset_call_counters(dyc_table *t, cudaStream_t s) {
    CK(cudaMemsetAsync(&t->d_ctr->inserted, 0, sizeof(Counters) - sizeof(unsigned long long), s));
    return DYC_OK;
}

dyc_status read_counters(dyc_table *t, cudaStream_t s) {
    CK(cudaMemcpyAsync(t->h_ctr, t->d_ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (t->h_ctr->spill)
        return fail(DYC_EOVERFLOW, "internal list overflow (%llu entries)",
                    (unsigned long long)t->h_ctr->spill);
    if (t->h_ctr->timeouts)
        return fail(DYC_ETIMEOUT, "%llu bounded device wait(s) gave up",
                    (unsigned long long)t->h_ctr->timeouts);
    t->size = t->h_ctr->size;
    return DYC_OK;
}

// ---- entries held outside the table after a failed call -------------------
// An error path (an upsize the pool cannot serve, eviction overflow that
// outlasts every round) keeps the entries it has not placed: they are copied
// to the table's held list on the host instead of being dropped (the
// reference drops them, cuckoo.cu:422-431, :714-722). Held entries are not
// in the device size counter; dyc_size counts them, dyc_op_stats.held
// reports them, and every later call on the table places them first
// (settle_held).
dyc_status hold_list(dyc_table *t, cudaStream_t s, const void *d_list, uint64_t count,
                     bool counted) {
    if (count == 0) return DYC_OK;
    const size_t bytes = (size_t)count * t->slot_bytes, at = t->held.size();
    t->held.resize(at + bytes);
    cudaError_t e = cudaMemcpyAsync(t->held.data() + at, d_list, bytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        t->held.resize(at);
        return fail(DYC_ECUDA, "copying %llu unplaced entries to the host: %s",
                    (unsigned long long)count, cudaGetErrorString(e));
    }
    t->held_n += count;
    if (counted) {  // moved residents (a downsize): the device size still counts them
        t->size -= count;
        t->h_ctr->size = t->size;
        CK(cudaMemcpyAsync(&t->d_ctr->size, &t->h_ctr->size, sizeof(unsigned long long),
                           cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
    }
    return DYC_OK;
}

// Hold `count` entries of d_list and return `why` (the failure that stopped
// their placement), its message extended.
dyc_status hold_failed(dyc_table *t, cudaStream_t s, const void *d_list, uint64_t count,
                       bool counted, dyc_status why) {
    const std::string msg = g_err;
    TRY(hold_list(t, s, d_list, count, counted));
    return fail(why, "%s; %llu entries held for the next call", msg.c_str(),
                (unsigned long long)count);
}

dyc_status drain(dyc_table *t, cudaStream_t s, void *src, unsigned long long *src_ctr,
                 void *dst, unsigned long long *dst_ctr, uint64_t cap, bool count_new,
                 bool first_upsize);

// Place the held entries (eviction walks, upsizing as needed). On failure
// the ones still unplaced are held again.
dyc_status settle_held(dyc_table *t, cudaStream_t s) {
    if (t->held_n == 0) return DYC_OK;
    const uint64_t n = t->held_n;
    TRY(ensure_scratch(t, n));
    CK(cudaMemcpyAsync(t->S.list_a, t->held.data(), (size_t)n * t->slot_bytes,
                       cudaMemcpyHostToDevice, s));
    TRY(reset_call_counters(t, s));
    t->h_ctr->pending = n;
    CK(cudaMemcpyAsync(&t->d_ctr->pending, &t->h_ctr->pending, sizeof(unsigned long long),
                       cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    std::vector<unsigned char>().swap(t->held);
    t->held_n = 0;
    const dyc_op_stats keep = t->last;
    const dyc_status r = drain(t, s, t->S.list_a, &t->d_ctr->pending, t->S.list_b,
                               &t->d_ctr->overflow, t->S.list_cap, true, false);
    const uint64_t ups = t->last.resizes_up - keep.resizes_up;
    t->last = keep;
    t->last.resizes_up += ups;
    return r;
}

// Double subtable pick_up(): allocate 2nb buckets, stream the old buckets
// into their two images, retire the old buffer (all stream-ordered).
dyc_status resize_up_impl(dyc_table *t, cudaStream_t s) {
    const uint32_t ti = pick_up(t->D.nb, t->D.d);
    const uint32_t onb = t->D.nb[ti];
    if ((uint64_t)onb * 2 > 0xFFFFFFFFull) return fail(DYC_EINVAL, "subtable %u too large", ti);
    const uint32_t nnb = onb * 2;
    void *nw = nullptr;
    CK(pool_alloc(t->device, &nw, (size_t)nnb * t->sb, s));
    void *old = t->D.sub[ti];
    cudaError_t e = KB_CALL(t, resize_up, ctx(t, s), t->sb, ti, old, onb, nw);
    if (e != cudaSuccess) {
        cudaFreeAsync(nw, s);
        return fail(DYC_ECUDA, "resize_up kernel: %s", cudaGetErrorString(e));
    }
    t->D.sub[ti] = nw;
    t->D.nb[ti] = nnb;
    t->D.magic[ti] = dyc::fastmod_magic(nnb);
    CK(cudaFreeAsync(old, s));
    t->capacity += (uint64_t)onb * t->slots;
    refresh_l2(t);
    t->last.resizes_up++;
    return DYC_OK;
}

// Highest load a batch may fill a table to before its upsize policy runs
// (the policy then runs after the batch): halfway from the upper bound to
// full. Past it eviction walks lengthen and fail (at 0.94 on 7-slot buckets
// a walk of max_evictions 2048 steps took 4-6 ms before overflowing).
double deferred_fill(const dyc_table *t) { return 0.5 * (1.0 + t->cfg.upper_load); }

// Host half of an upsize of subtable pick_up(): allocate the doubled
// subtable, describe the move as a job and switch the descriptor to the new
// subtable. The caller launches the move (resize_up_flush) before freeing
// *old_out, both stream-ordered on s.
dyc_status resize_up_prepare(dyc_table *t, cudaStream_t s, dyc::ResizeJob *job, void **old_out) {
    const uint32_t ti = pick_up(t->D.nb, t->D.d);
    const uint32_t onb = t->D.nb[ti];
    if ((uint64_t)onb * 2 > 0xFFFFFFFFull) return fail(DYC_EINVAL, "subtable %u too large", ti);
    const uint32_t nnb = onb * 2;
    void *nw = nullptr;
    CK(pool_alloc(t->device, &nw, (size_t)nnb * t->sb, s));
    const uint64_t magic = dyc::fastmod_magic(nnb);
    *job = dyc::ResizeJob{t->D.sub[ti], nw, magic, onb, ti, 0u, 0u};
    *old_out = t->D.sub[ti];
    t->D.sub[ti] = nw;
    t->D.nb[ti] = nnb;
    t->D.magic[ti] = magic;
    t->capacity += (uint64_t)onb * t->slots;
    refresh_l2(t);
    t->last.resizes_up++;
    return DYC_OK;
}

// The moves of prepared upsizes, kMaxResizeJobs per launch, then the old
// subtables freed behind them.
dyc_status resize_up_flush(int kb, int sb, int sms, cudaStream_t s,
                           const std::vector<dyc::ResizeJob> &jobs, const std::vector<void *> &olds) {
    static thread_local std::unique_ptr<dyc::ResizeJobs> J(new dyc::ResizeJobs());
    const LaunchCtx L{sms, s};
    const uint64_t g = (uint64_t)sb / 32;
    for (size_t a = 0; a < jobs.size(); a += dyc::kMaxResizeJobs) {
        const size_t m = std::min<size_t>(dyc::kMaxResizeJobs, jobs.size() - a);
        uint64_t blocks = 0;
        for (size_t i = 0; i < m; ++i) {
            J->j[i] = jobs[a + i];
            J->j[i].block0 = (uint32_t)blocks;
            const uint64_t chunks = (uint64_t)J->j[i].old_nb * g;
            blocks += (chunks + dyc::kResizeChunksPerBlock - 1) / dyc::kResizeChunksPerBlock;
        }
        if (blocks >= 0x7FFFFFFFull) return fail(DYC_EINVAL, "upsize wave too large");
        J->n = (uint32_t)m;
        J->blocks = (uint32_t)blocks;
        const cudaError_t e = kb == 4 ? Ops<4>::resize_up_many(L, sb, *J)
                                      : Ops<8>::resize_up_many(L, sb, *J);
        if (e != cudaSuccess) return fail(DYC_ECUDA, "resize_up kernel: %s", cudaGetErrorString(e));
    }
    for (void *o : olds) CK(cudaFreeAsync(o, s));
    return DYC_OK;
}

// Place the entries of list `src` (count in counter *src_ctr, and in its
// host mirror in t->h_ctr on entry) by eviction walks; leftovers go to
// `dst`. Repeats with an upsize in between until nothing is left.
// count_new: successes are new keys (insert) rather than moved ones
// (downsize). If an upsize fails or the rounds run out, the entries not yet
// placed are held (hold_list) and the error is returned: nothing is dropped.
dyc_status drain(dyc_table *t, cudaStream_t s, void *src, unsigned long long *src_ctr,
                 void *dst, unsigned long long *dst_ctr, uint64_t cap, bool count_new,
                 bool first_upsize) {
    auto host_count = [&](const unsigned long long *dc) {
        return dc == &t->d_ctr->pending ? t->h_ctr->pending : t->h_ctr->overflow;
    };
    unsigned long long left = host_count(src_ctr);
    for (int round = 0; round < kMaxOverflowRounds; ++round) {
        if (round > 0 || first_upsize) {
            // grow to the upper load bound for everything placed or pending,
            // and by at least one subtable
            int guard = 0;
            do {
                const dyc_status r = resize_up_impl(t, s);
                if (r != DYC_OK) return hold_failed(t, s, src, left, !count_new, r);
            } while ((double)(t->size + left) > t->cfg.upper_load * (double)t->capacity &&
                     ++guard < 64);
        }
        CK(cudaMemsetAsync(dst_ctr, 0, sizeof(unsigned long long), s));
        cudaError_t e = KB_CALL(t, walk, ctx(t, s), t->D, t->sb, src, src_ctr, dst, dst_ctr, cap,
                                t->cfg.max_evictions, count_new, t->d_ctr, cap);
        if (e != cudaSuccess)
            return hold_failed(t, s, src, left, !count_new,
                               fail(DYC_ECUDA, "walk kernel: %s", cudaGetErrorString(e)));
        TRY(read_counters(t, s));
        left = host_count(dst_ctr);
        if (left == 0) return DYC_OK;
        std::swap(src, dst);
        std::swap(src_ctr, dst_ctr);
    }
    return hold_failed(t, s, src, left, !count_new,
                       fail(DYC_EOVERFLOW, "eviction overflow persisted after %d upsizes",
                            kMaxOverflowRounds));
}

// The table's scratch as one chunk of n ops uses it: the dedup table sized
// for n (as ensure_scratch sizes it for the largest chunk), so a small call
// on a table that once took a large batch clears and probes a small table.
Scratch chunk_scratch(const dyc_table *t, uint64_t n) {
    Scratch S = t->S;
    const uint64_t cap = dedup_cells(n);
    if (cap < S.dedup_cap) S.dedup_cap = cap;
    return S;
}

// Batch dedup of one chunk into the dedup buffers of S, on stream s:
// kKeepLast (insert) names each key's last op, kKeepFirst (erase) its first.
// One launch clears the chunk's cells and the call counters (what
// reset_call_counters does), then the claims run.
dyc_status dedup_chunk(dyc_table *t, const Scratch &S, const void *keys, uint64_t n,
                       dyc::DedupMode mode, cudaStream_t s) {
    cudaError_t e = KB_CALL(t, dedup, ctx(t, s), S, keys, n, mode, &t->d_ctr->inserted,
                            (uint32_t)(sizeof(Counters) / 8 - 1));
    if (e != cudaSuccess) return fail(DYC_ECUDA, "dedup kernel: %s", cudaGetErrorString(e));
    return DYC_OK;
}

dyc_status insert_chunk(dyc_table *t, const void *keys, const void *vals, uint64_t n,
                        uint32_t flags, cudaStream_t s) {
    const bool use_dedup = !(flags & DYC_FLAG_UNIQUE) && n > 1;
    const bool new_keys = (flags & DYC_FLAG_NEW_KEYS) != 0;
    const Scratch S = chunk_scratch(t, n);
    if (use_dedup) TRY(dedup_chunk(t, S, keys, n, dyc::kKeepLast, s));
    else TRY(reset_call_counters(t, s));
    cudaError_t e = KB_CALL(t, place, ctx(t, s), t->D, t->sb, S, use_dedup, new_keys, keys,
                            vals, (uint32_t)t->vb, n, t->d_ctr);
    if (e != cudaSuccess) return fail(DYC_ECUDA, "place kernel: %s", cudaGetErrorString(e));
    // walks for the ops whose buckets were full: list_a -> list_b
    e = KB_CALL(t, walk, ctx(t, s), t->D, t->sb, t->S.list_a, &t->d_ctr->pending, t->S.list_b,
                &t->d_ctr->overflow, t->S.list_cap, t->cfg.max_evictions, true, t->d_ctr,
                t->S.list_cap);
    if (e != cudaSuccess) return fail(DYC_ECUDA, "walk kernel: %s", cudaGetErrorString(e));
    TRY(read_counters(t, s));
    const Counters c = *t->h_ctr;
    dyc_op_stats &L = t->last;
    L.inserted += c.inserted;
    L.updated += c.updated;
    L.rejected += c.rejected;
    L.superseded += c.superseded;
    L.evict_steps += c.evict_steps;
    L.overflowed += c.overflow;
    if (c.overflow) {
        TRY(drain(t, s, t->S.list_b, &t->d_ctr->overflow, t->S.list_a, &t->d_ctr->pending,
                  t->S.list_cap, true, true));
        L.inserted += t->h_ctr->inserted - c.inserted;
        L.evict_steps += t->h_ctr->evict_steps - c.evict_steps;
    }
    return DYC_OK;
}

dyc_status erase_chunk(dyc_table *t, const void *keys, uint64_t n, uint32_t *bits,
                       uint32_t flags, cudaStream_t s) {
    const bool use_dedup = !(flags & DYC_FLAG_UNIQUE) && n > 1;
    const Scratch S = chunk_scratch(t, n);
    if (use_dedup) TRY(dedup_chunk(t, S, keys, n, dyc::kKeepFirst, s));
    else TRY(reset_call_counters(t, s));
    cudaError_t e = KB_CALL(t, erase, ctx(t, s), t->D, t->sb, S, use_dedup, keys, n, bits,
                            t->d_ctr);
    if (e != cudaSuccess) return fail(DYC_ECUDA, "erase kernel: %s", cudaGetErrorString(e));
    TRY(read_counters(t, s));
    t->last.erased += t->h_ctr->erased;
    t->last.superseded += t->h_ctr->superseded;
    return DYC_OK;
}

// Halve subtable pick_down(). Even bucket counts merge bucket j with j+nb/2;
// odd counts rehash the whole subtable into ceil(nb/2) buckets. Entries that
// do not fit are placed by eviction walks (upsizing another subtable if
// needed), so nothing is dropped. The merge only reads the old subtable, and
// the descriptor switches to the new one only after the merge's counters
// are read: a failed allocation, a merge whose copy waits gave up
// (DYC_ETIMEOUT) or a full list leave the table as it was. The lists hold
// every entry that can be left over (even: one bucket's worth per merged
// bucket; odd: the whole subtable), so a spill means a fault, not a load.
dyc_status resize_down_impl(dyc_table *t, cudaStream_t s) {
    const uint32_t ti = pick_down(t->D.nb, t->D.d);
    const uint32_t onb = t->D.nb[ti];
    if (onb < 2) return fail(DYC_EINVAL, "subtable %u has %u bucket(s); cannot halve", ti, onb);
    const bool even = (onb % 2u) == 0;
    const uint32_t nnb = even ? onb / 2 : (onb + 1) / 2;
    const uint64_t list_cap = even ? (uint64_t)nnb * t->slots : (uint64_t)onb * t->slots;
    void *nw = nullptr, *la = nullptr, *lb = nullptr;
    auto release = [&]() {
        if (nw) cudaFreeAsync(nw, s);
        if (la) cudaFreeAsync(la, s);
        if (lb) cudaFreeAsync(lb, s);
    };
    cudaError_t e = pool_alloc(t->device, &nw, (size_t)nnb * t->sb, s);
    if (e == cudaSuccess) e = pool_alloc(t->device, &la, (size_t)list_cap * t->slot_bytes, s);
    if (e == cudaSuccess) e = pool_alloc(t->device, &lb, (size_t)list_cap * t->slot_bytes, s);
    if (e != cudaSuccess) {
        release();
        return fail(e == cudaErrorMemoryAllocation ? DYC_ENOMEM : DYC_ECUDA,
                    "downsize of subtable %u: allocation: %s (table unchanged)", ti,
                    cudaGetErrorString(e));
    }
    dyc_status r = reset_call_counters(t, s);
    if (r != DYC_OK) {
        release();
        return r;
    }
    void *old = t->D.sub[ti];
    if (even) {
        e = KB_CALL(t, resize_down, ctx(t, s), t->sb, old, onb, nw, la, &t->d_ctr->pending,
                    list_cap, &t->d_ctr->spill, &t->d_ctr->timeouts, g_inject_wait_tries.load());
    } else {
        e = cudaMemsetAsync(nw, 0, (size_t)nnb * t->sb, s);
        if (e == cudaSuccess)
            e = KB_CALL(t, collect, ctx(t, s), t->sb, old, onb, la, &t->d_ctr->pending, list_cap,
                        &t->d_ctr->spill);
        // keys of other subtables may have had their first-probe bucket here:
        // start every new bucket with all fingerprint bits set
        if (e == cudaSuccess) e = KB_CALL(t, mark_all, ctx(t, s), t->sb, nw, nnb);
    }
    if (e != cudaSuccess) {
        release();
        return fail(DYC_ECUDA, "downsize kernel: %s", cudaGetErrorString(e));
    }
    e = cudaMemcpyAsync(t->h_ctr, t->d_ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        release();
        return fail(DYC_ECUDA, "downsize counters: %s", cudaGetErrorString(e));
    }
    if (t->h_ctr->timeouts || t->h_ctr->spill) {
        const bool to = t->h_ctr->timeouts != 0;
        const unsigned long long c = to ? t->h_ctr->timeouts : t->h_ctr->spill;
        release();
        CK(cudaMemsetAsync(&t->d_ctr->inserted, 0, sizeof(Counters) - sizeof(unsigned long long), s));
        CK(cudaStreamSynchronize(s));
        return fail(to ? DYC_ETIMEOUT : DYC_EOVERFLOW,
                    "downsize of subtable %u: %llu %s; the table is unchanged", ti, c,
                    to ? "bounded copy wait(s) gave up" : "leftover entries found no list slot");
    }
    t->D.sub[ti] = nw;
    t->D.nb[ti] = nnb;
    t->D.magic[ti] = dyc::fastmod_magic(nnb);
    t->capacity -= (uint64_t)(onb - nnb) * t->slots;
    refresh_l2(t);
    CK(cudaFreeAsync(old, s));
    t->last.resizes_down++;
    const dyc_status st = drain(t, s, la, &t->d_ctr->pending, lb, &t->d_ctr->overflow, list_cap,
                                false, false);
    cudaFreeAsync(la, s);
    cudaFreeAsync(lb, s);
    return st;
}

bool valid_config(const dyc_config *c, char *why, size_t n) {
    if (c->key_bytes != 4 && c->key_bytes != 8) return snprintf(why, n, "key_bytes must be 4 or 8"), false;
    if (c->value_bytes != 4 && c->value_bytes != 8) return snprintf(why, n, "value_bytes must be 4 or 8"), false;
    if (c->key_bytes == 4 && c->value_bytes != 4)
        return snprintf(why, n, "4-byte keys take 4-byte values"), false;
    if (c->num_subtables < 2 || c->num_subtables > 6)
        return snprintf(why, n, "num_subtables must be 2..6"), false;
    if (c->bucket_bytes != 32 && c->bucket_bytes != 64 && c->bucket_bytes != 128)
        return snprintf(why, n, "bucket_bytes must be 32, 64 or 128"), false;
    if (c->max_evictions < 1 || c->max_evictions > 100000)
        return snprintf(why, n, "max_evictions must be 1..100000"), false;
    if (!(c->upper_load > 0.0 && c->upper_load <= 1.0) || !(c->lower_load >= 0.0 && c->lower_load < c->upper_load))
        return snprintf(why, n, "need 0 <= lower_load < upper_load <= 1"), false;
    if (c->l2_resident > 2) return snprintf(why, n, "l2_resident must be 0, 1 or 2"), false;
    if (c->device_upsize > 1) return snprintf(why, n, "device_upsize must be 0 or 1"), false;
    return true;
}

}  // namespace

// =============================================================================
extern "C" {

void dyc_config_default(dyc_config *cfg) {
    if (!cfg) return;
    memset(cfg, 0, sizeof(*cfg));
    cfg->key_bytes = 4;
    cfg->value_bytes = 4;
    cfg->num_subtables = 4;
    cfg->bucket_bytes = 128;
    cfg->max_evictions = 64;
    cfg->auto_resize = 1;
    cfg->initial_size = 1024;
    cfg->upper_load = 0.8;
    cfg->lower_load = 0.5;
    cfg->min_downsize_capacity = (uint64_t)(4 * 1024 * 1024 * 1.2);
    cfg->device = 0;
}

const char *dyc_status_string(dyc_status s) {
    switch (s) {
    case DYC_OK: return "ok";
    case DYC_ENOMEM: return "out of memory";
    case DYC_EINVAL: return "invalid argument";
    case DYC_EOVERFLOW: return "eviction overflow";
    case DYC_ETIMEOUT: return "device wait timed out";
    case DYC_ECUDA: return "CUDA error";
    case DYC_ENOTSUP: return "not supported";
    }
    return "unknown status";
}

const char *dyc_last_error(void) { return g_err.c_str(); }

}  // extern "C"

namespace {
// Table creation. ext_d / ext_h: counters owned by a table set (the table
// then allocates none); sync: wait for the zero-fill before returning.
// nb_override: bucket count of every subtable (a restored snapshot's layout)
// instead of the sizing rule.
dyc_status create_impl(const dyc_config *cfg, Counters *ext_d, Counters *ext_h, bool sync,
                       dyc_table **out, const uint32_t *nb_override = nullptr) {
    if (!cfg || !out) return fail(DYC_EINVAL, "null argument");
    *out = nullptr;
    char why[128];
    if (!valid_config(cfg, why, sizeof(why))) return fail(DYC_EINVAL, "%s", why);
    dyc_table *t = new (std::nothrow) dyc_table();
    if (!t) return fail(DYC_ENOMEM, "host allocation");
    if (const uint64_t c = g_inject_chunk.load()) t->chunk = c;
    t->cfg = *cfg;
    t->kb = (int)cfg->key_bytes;
    t->vb = (int)cfg->value_bytes;
    t->sb = (int)cfg->bucket_bytes;
    t->slot_bytes = t->kb == 4 ? 8 : 16;
    // 128-byte buckets keep their last slot as the metadata word
    t->slots = t->sb / t->slot_bytes - (t->sb == 128 ? 1 : 0);
    t->device = cfg->device;
    auto undo = [&](dyc_status s) {
        dyc_destroy(t);
        return s;
    };
    {
        cudaError_t e = cudaSetDevice(t->device);
        if (e != cudaSuccess) return undo(fail(DYC_ECUDA, "cudaSetDevice(%d): %s", t->device, cudaGetErrorString(e)));
        e = cudaDeviceGetAttribute(&t->sms, cudaDevAttrMultiProcessorCount, t->device);
        if (e != cudaSuccess) return undo(fail(DYC_ECUDA, "device attribute: %s", cudaGetErrorString(e)));
    }
    // hashAPI::hashAPI sizing (api.cpp:47-54) with this table's slots/bucket
    const uint64_t per = (uint64_t)cfg->num_subtables * t->slots;
    const uint64_t s0 = cfg->initial_size / per;
    if (s0 >= 0x7FFFFFF0ull) return undo(fail(DYC_EINVAL, "initial_size too large"));
    uint32_t s = next_prime_ref((uint32_t)s0);
    const uint32_t nb_rule = (s & 1u) ? s + 1u : s;
    memset(&t->D, 0, sizeof(t->D));
    t->D.d = cfg->num_subtables;
    t->D.max_evict = cfg->max_evictions;
    for (uint32_t i = 0; i < t->D.d; ++i) {
        const uint32_t nb = nb_override ? nb_override[i] : nb_rule;
        cudaError_t e = dyc::lib_malloc(&t->D.sub[i], (size_t)nb * t->sb);
        if (e != cudaSuccess) return undo(fail(DYC_ENOMEM, "subtable %u: %s", i, cudaGetErrorString(e)));
        e = cudaMemsetAsync(t->D.sub[i], 0, (size_t)nb * t->sb, 0);
        if (e != cudaSuccess) return undo(fail(DYC_ECUDA, "memset: %s", cudaGetErrorString(e)));
        t->D.nb[i] = nb;
        t->D.magic[i] = dyc::fastmod_magic(nb);
        t->capacity += (uint64_t)nb * t->slots;
    }
    refresh_l2(t);
    cudaError_t e = cudaSuccess;
    if (ext_d) {
        t->owns_ctr = false;
        t->d_ctr = ext_d;
        t->h_ctr = ext_h;
    } else {
        e = dyc::lib_malloc(&t->d_ctr, sizeof(Counters));
        if (e == cudaSuccess) e = cudaMemsetAsync(t->d_ctr, 0, sizeof(Counters), 0);
        if (e == cudaSuccess) e = dyc::lib_malloc_host(&t->h_ctr, sizeof(Counters));
        if (e == cudaSuccess) memset(t->h_ctr, 0, sizeof(Counters));
    }
    if (e == cudaSuccess && sync) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return undo(fail(DYC_ECUDA, "table setup: %s", cudaGetErrorString(e)));
    t->counted = true;
    pool_table_count(t->device, 1);
    *out = t;
    return DYC_OK;
}
}  // namespace

extern "C" {

dyc_status dyc_create(const dyc_config *cfg, dyc_table **out) {
    return create_impl(cfg, nullptr, nullptr, true, out);
}

dyc_status dyc_destroy(dyc_table *t) {
    if (!t) return DYC_OK;
    cudaSetDevice(t->device);
    cudaDeviceSynchronize();
    for (uint32_t i = 0; i < dyc::kMaxSub; ++i)
        if (t->D.sub[i]) cudaFree(t->D.sub[i]);
    if (t->owns_ctr && t->d_ctr) cudaFree(t->d_ctr);
    if (t->owns_ctr && t->h_ctr) cudaFreeHost(t->h_ctr);
    if (t->scratch) cudaFree(t->scratch);
    if (t->apply_buf) cudaFree(t->apply_buf);
    if (t->h_actr) cudaFreeHost(t->h_actr);
    if (t->d_desc) cudaFree(t->d_desc);
    if (t->h_desc) cudaFreeHost(t->h_desc);
    if (t->d_io) cudaFree(t->d_io);
    if (t->io_stream) cudaStreamDestroy(t->io_stream);
    for (int i = 0; i < 3; ++i) {
        if (t->pipe_buf[i]) cudaFree(t->pipe_buf[i]);
        if (t->pipe_stream[i]) cudaStreamDestroy(t->pipe_stream[i]);
    }
    if (t->counted) pool_table_count(t->device, -1);
    delete t;
    return DYC_OK;
}

dyc_status dyc_pool_reserve(int32_t device, uint64_t bytes) {
    if (bytes == 0) return DYC_OK;
    int cur = -1;
    CK(cudaGetDevice(&cur));
    if (cur != device) CK(cudaSetDevice(device));
    cudaMemPool_t pool = nullptr;
    CK(lib_pool(device, &pool));
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const uint64_t keep = total_b / 4;  // the pool's release threshold
    if (bytes > keep) bytes = keep;
    cudaStream_t s = nullptr;
    CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    void *p = nullptr;
    dyc::g_lib_allocs.fetch_add(1, std::memory_order_relaxed);
    cudaError_t e = cudaMallocFromPoolAsync(&p, (size_t)bytes, pool, s);
    if (e == cudaSuccess) e = cudaFreeAsync(p, s);
    const cudaError_t e2 = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (cur != device) cudaSetDevice(cur);
    if (e == cudaErrorMemoryAllocation) return fail(DYC_ENOMEM, "pool reserve of %llu bytes",
                                                    (unsigned long long)bytes);
    if (e != cudaSuccess || e2 != cudaSuccess)
        return fail(DYC_ECUDA, "pool reserve: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    return DYC_OK;
}

dyc_status dyc_insert(dyc_table *t, const void *d_keys, const void *d_vals, uint64_t n,
                      uint32_t flags, void *stream) {
    if (!t) return fail(DYC_EINVAL, "null table");
    TRY(set_device(t));
    cudaStream_t s = (cudaStream_t)stream;
    t->last = dyc_op_stats{};
    TRY(settle_held(t, s));
    if (n == 0) return DYC_OK;
    if (!d_keys || !d_vals) return fail(DYC_EINVAL, "null key or value array");
    const uint64_t chunk = t->chunk;
    TRY(ensure_scratch(t, n < chunk ? n : chunk));
    for (uint64_t off = 0; off < n; off += chunk) {
        const uint64_t m = (n - off) < chunk ? (n - off) : chunk;
        // projected-size check before the batch (api.cpp:359-369)
        if (t->cfg.auto_resize && !(flags & DYC_FLAG_NO_RESIZE)) {
            int guard = 0;
            while ((double)(t->size + m) > t->cfg.upper_load * (double)t->capacity && guard++ < 64)
                TRY(resize_up_impl(t, s));
        }
        TRY(insert_chunk(t, (const char *)d_keys + off * t->kb,
                         (const char *)d_vals + off * t->vb, m, flags, s));
    }
    return DYC_OK;
}

dyc_status dyc_find(dyc_table *t, const void *d_keys, void *d_vals_out, uint32_t *d_hit_bits_out,
                    uint64_t n, void *stream) {
    if (!t) return fail(DYC_EINVAL, "null table");
    TRY(set_device(t));
    if (t->held_n) TRY(settle_held(t, (cudaStream_t)stream));
    if (n == 0) return DYC_OK;
    if (!d_keys || !d_vals_out) return fail(DYC_EINVAL, "null key or value array");
    cudaError_t e = KB_CALL(t, find, ctx(t, stream), t->D, t->sb, d_keys, d_vals_out,
                            (uint32_t)t->vb, d_hit_bits_out, n);
    if (e != cudaSuccess) return fail(DYC_ECUDA, "find kernel: %s", cudaGetErrorString(e));
    return DYC_OK;
}

dyc_status dyc_erase(dyc_table *t, const void *d_keys, uint64_t n, uint32_t *d_erased_bits_out,
                     uint64_t *h_erased_count, uint32_t flags, void *stream) {
    if (!t) return fail(DYC_EINVAL, "null table");
    if (h_erased_count) *h_erased_count = 0;
    TRY(set_device(t));
    cudaStream_t s = (cudaStream_t)stream;
    t->last = dyc_op_stats{};
    TRY(settle_held(t, s));
    if (n == 0) return DYC_OK;
    if (!d_keys) return fail(DYC_EINVAL, "null key array");
    const uint64_t chunk = t->chunk;
    TRY(ensure_scratch(t, n < chunk ? n : chunk));
    for (uint64_t off = 0; off < n; off += chunk) {
        const uint64_t m = (n - off) < chunk ? (n - off) : chunk;
        TRY(erase_chunk(t, (const char *)d_keys + off * t->kb, m,
                        d_erased_bits_out ? d_erased_bits_out + off / 32 : nullptr, flags, s));
    }
    if (h_erased_count) *h_erased_count = t->last.erased;
    // downsize check after the batch (api.cpp:494-505)
    if (t->cfg.auto_resize && !(flags & DYC_FLAG_NO_RESIZE) &&
        (double)t->size < t->cfg.lower_load * (double)t->capacity &&
        t->capacity > t->cfg.min_downsize_capacity) {
        const dyc_op_stats keep = t->last;
        dyc_status st = resize_down_impl(t, s);
        if (st != DYC_OK && st != DYC_EINVAL) return st;
        const uint64_t downs = t->last.resizes_down, ups = t->last.resizes_up;
        t->last = keep;
        t->last.resizes_down = downs;
        t->last.resizes_up = ups;
    }
    return DYC_OK;
}

dyc_status dyc_resize_up(dyc_table *t, void *stream) {
    if (!t) return fail(DYC_EINVAL, "null table");
    TRY(set_device(t));
    t->last = dyc_op_stats{};
    TRY(settle_held(t, (cudaStream_t)stream));
    TRY(resize_up_impl(t, (cudaStream_t)stream));
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    return DYC_OK;
}

dyc_status dyc_resize_down(dyc_table *t, void *stream) {
    if (!t) return fail(DYC_EINVAL, "null table");
    TRY(set_device(t));
    t->last = dyc_op_stats{};
    TRY(settle_held(t, (cudaStream_t)stream));
    return resize_down_impl(t, (cudaStream_t)stream);
}

dyc_status dyc_size(dyc_table *t, uint64_t *size) {
    if (!t || !size) return fail(DYC_EINVAL, "null argument");
    *size = t->size + t->held_n;  // held entries are keys of the table too
    return DYC_OK;
}

dyc_status dyc_capacity(dyc_table *t, uint64_t *capacity) {
    if (!t || !capacity) return fail(DYC_EINVAL, "null argument");
    *capacity = t->capacity;
    return DYC_OK;
}

dyc_status dyc_layout(dyc_table *t, uint32_t *nbuckets_out, uint32_t *num_subtables) {
    if (!t) return fail(DYC_EINVAL, "null table");
    if (num_subtables) *num_subtables = t->D.d;
    if (nbuckets_out)
        for (uint32_t i = 0; i < t->D.d; ++i) nbuckets_out[i] = t->D.nb[i];
    return DYC_OK;
}

dyc_status dyc_subtable(dyc_table *t, uint32_t i, void **d_ptr, uint64_t *bytes) {
    if (!t || i >= t->D.d) return fail(DYC_EINVAL, "bad table or subtable index");
    if (d_ptr) *d_ptr = t->D.sub[i];
    if (bytes) *bytes = (uint64_t)t->D.nb[i] * t->sb;
    return DYC_OK;
}

dyc_status dyc_export(dyc_table *t, void *d_keys_out, void *d_vals_out, uint64_t capacity,
                      uint64_t *n_out, void *stream) {
    if (!t) return fail(DYC_EINVAL, "null table");
    if (capacity && (!d_keys_out || !d_vals_out)) return fail(DYC_EINVAL, "null output array");
    TRY(set_device(t));
    cudaStream_t s = (cudaStream_t)stream;
    TRY(settle_held(t, s));
    CK(cudaMemsetAsync(&t->d_ctr->pad[0], 0, sizeof(unsigned long long), s));
    cudaError_t e = KB_CALL(t, export_all, ctx(t, s), t->D, t->sb, d_keys_out, d_vals_out,
                            (uint32_t)t->vb, capacity, &t->d_ctr->pad[0]);
    if (e != cudaSuccess) return fail(DYC_ECUDA, "export kernel: %s", cudaGetErrorString(e));
    unsigned long long cnt = 0;
    CK(cudaMemcpyAsync(t->h_ctr, t->d_ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    cnt = t->h_ctr->pad[0];
    if (n_out) *n_out = cnt;
    return DYC_OK;
}

dyc_status dyc_debug_alloc_count(uint64_t *count) {
    if (!count) return fail(DYC_EINVAL, "null argument");
    *count = dyc::g_lib_allocs.load();
    return DYC_OK;
}

dyc_status dyc_debug_inject(uint32_t kind, uint64_t n) {
    switch (kind) {
    case DYC_INJECT_RESET:
        g_inject_alloc.store(0);
        g_inject_wait_tries.store(dyc::kWaitTries);
        g_inject_chunk.store(0);
        return DYC_OK;
    case DYC_INJECT_POOL_ALLOC:
        g_inject_alloc.store(n);
        return DYC_OK;
    case DYC_INJECT_WAIT_TRIES:
        g_inject_wait_tries.store(n < dyc::kWaitTries ? (uint32_t)n : dyc::kWaitTries);
        return DYC_OK;
    case DYC_INJECT_CHUNK_OPS:
        // chunk offsets index per-op bit arrays by 32-bit word
        if (n % 32 != 0 || n > kChunkDefault)
            return fail(DYC_EINVAL, "chunk of %llu ops: a multiple of 32, at most %llu",
                        (unsigned long long)n, (unsigned long long)kChunkDefault);
        g_inject_chunk.store(n);
        return DYC_OK;
    default:
        return fail(DYC_EINVAL, "unknown injection kind %u", kind);
    }
}

dyc_status dyc_last_stats(dyc_table *t, dyc_op_stats *out) {
    if (!t || !out) return fail(DYC_EINVAL, "null argument");
    *out = t->last;
    out->held = t->held_n;
    return DYC_OK;
}

// ---- host-buffer forms (hashAPI::hash_insert / hash_search / hash_delete) ----
namespace {
constexpr uint64_t kIoChunk = 1ull << 22;  // ops staged per round trip

dyc_status ensure_io(dyc_table *t, size_t bytes) {
    if (!t->io_stream) CK(cudaStreamCreateWithFlags(&t->io_stream, cudaStreamNonBlocking));
    if (t->d_io && t->d_io_bytes >= bytes) return DYC_OK;
    if (t->d_io) {
        CK(cudaStreamSynchronize(t->io_stream));
        CK(cudaFree(t->d_io));
        t->d_io = nullptr;
    }
    CK(dyc::lib_malloc(&t->d_io, bytes));
    t->d_io_bytes = bytes;
    return DYC_OK;
}
}  // namespace

dyc_status dyc_insert_host(dyc_table *t, const void *h_keys, const void *h_vals, uint64_t n,
                           uint32_t flags) {
    if (!t) return fail(DYC_EINVAL, "null table");
    if (n == 0) return DYC_OK;
    if (!h_keys || !h_vals) return fail(DYC_EINVAL, "null key or value array");
    TRY(set_device(t));
    const uint64_t c = n < kIoChunk ? n : kIoChunk;
    TRY(ensure_io(t, (size_t)c * (t->kb + t->vb) + 256));
    char *dk = (char *)t->d_io;
    char *dv = dk + (((size_t)c * t->kb + 255) & ~(size_t)255);
    dyc_op_stats total{};
    for (uint64_t off = 0; off < n; off += c) {
        const uint64_t m = (n - off) < c ? (n - off) : c;
        CK(cudaMemcpyAsync(dk, (const char *)h_keys + off * t->kb, m * t->kb, cudaMemcpyHostToDevice, t->io_stream));
        CK(cudaMemcpyAsync(dv, (const char *)h_vals + off * t->vb, m * t->vb, cudaMemcpyHostToDevice, t->io_stream));
        TRY(dyc_insert(t, dk, dv, m, flags, t->io_stream));
        total.inserted += t->last.inserted;
        total.updated += t->last.updated;
        total.rejected += t->last.rejected;
        total.superseded += t->last.superseded;
        total.evict_steps += t->last.evict_steps;
        total.overflowed += t->last.overflowed;
        total.resizes_up += t->last.resizes_up;
    }
    t->last = total;
    return DYC_OK;
}

// Three-stage pipeline over chunks: chunk c uses stream and buffer c % 3, so
// the upload of one chunk, the find kernel of the previous one and the
// download of the one before that run at the same time (the two copy
// directions use separate engines). Stream order on each stage keeps a
// buffer from being refilled before its previous results are downloaded.
dyc_status dyc_find_host(dyc_table *t, const void *h_keys, void *h_vals_out,
                         uint32_t *h_hit_bits_out, uint64_t n) {
    if (!t) return fail(DYC_EINVAL, "null table");
    if (n == 0) return DYC_OK;
    if (!h_keys || !h_vals_out) return fail(DYC_EINVAL, "null key or value array");
    TRY(set_device(t));
    constexpr int kStages = 3;
    const uint64_t c = n < kIoChunk ? n : kIoChunk;
    const size_t kbytes = (((size_t)c * t->kb) + 255) & ~(size_t)255;
    const size_t vbytes = (((size_t)c * t->vb) + 255) & ~(size_t)255;
    const size_t need = kbytes + vbytes + (c / 32 + 1) * 4 + 256;
    if (t->pipe_bytes < need) {
        for (int i = 0; i < kStages; ++i) {
            if (t->pipe_stream[i]) CK(cudaStreamSynchronize(t->pipe_stream[i]));
            if (t->pipe_buf[i]) CK(cudaFree(t->pipe_buf[i]));
            t->pipe_buf[i] = nullptr;
        }
        t->pipe_bytes = 0;
        for (int i = 0; i < kStages; ++i) {
            if (!t->pipe_stream[i])
                CK(cudaStreamCreateWithFlags(&t->pipe_stream[i], cudaStreamNonBlocking));
            CK(dyc::lib_malloc(&t->pipe_buf[i], need));
        }
        t->pipe_bytes = need;
    }
    const uint64_t nchunks = (n + c - 1) / c;
    for (uint64_t ci = 0; ci < nchunks; ++ci) {
        const int st = (int)(ci % kStages);
        cudaStream_t s = t->pipe_stream[st];
        char *dk = (char *)t->pipe_buf[st];
        char *dv = dk + kbytes;
        uint32_t *db = (uint32_t *)(dv + vbytes);
        const uint64_t off = ci * c;
        const uint64_t m = (n - off) < c ? (n - off) : c;
        CK(cudaMemcpyAsync(dk, (const char *)h_keys + off * t->kb, m * t->kb, cudaMemcpyHostToDevice, s));
        TRY(dyc_find(t, dk, dv, h_hit_bits_out ? db : nullptr, m, s));
        CK(cudaMemcpyAsync((char *)h_vals_out + off * t->vb, dv, m * t->vb, cudaMemcpyDeviceToHost, s));
        if (h_hit_bits_out)
            CK(cudaMemcpyAsync(h_hit_bits_out + off / 32, db, ((m + 31) / 32) * 4, cudaMemcpyDeviceToHost, s));
    }
    for (int i = 0; i < kStages; ++i)
        if (t->pipe_stream[i]) CK(cudaStreamSynchronize(t->pipe_stream[i]));
    return DYC_OK;
}

dyc_status dyc_erase_host(dyc_table *t, const void *h_keys, uint64_t n,
                          uint32_t *h_erased_bits_out, uint64_t *erased_count) {
    if (!t) return fail(DYC_EINVAL, "null table");
    if (erased_count) *erased_count = 0;
    if (n == 0) return DYC_OK;
    if (!h_keys) return fail(DYC_EINVAL, "null key array");
    TRY(set_device(t));
    const uint64_t c = n < kIoChunk ? n : kIoChunk;
    const size_t kbytes = (((size_t)c * t->kb) + 255) & ~(size_t)255;
    TRY(ensure_io(t, kbytes + (c / 32 + 1) * 4 + 256));
    char *dk = (char *)t->d_io;
    uint32_t *db = (uint32_t *)(dk + kbytes);
    uint64_t total = 0;
    dyc_op_stats agg{};
    for (uint64_t off = 0; off < n; off += c) {
        const uint64_t m = (n - off) < c ? (n - off) : c;
        CK(cudaMemcpyAsync(dk, (const char *)h_keys + off * t->kb, m * t->kb, cudaMemcpyHostToDevice, t->io_stream));
        uint64_t got = 0;
        TRY(dyc_erase(t, dk, m, h_erased_bits_out ? db : nullptr, &got, 0, t->io_stream));
        total += got;
        agg.erased += t->last.erased;
        agg.superseded += t->last.superseded;
        agg.resizes_down += t->last.resizes_down;
        agg.resizes_up += t->last.resizes_up;
        if (h_erased_bits_out)
            CK(cudaMemcpyAsync(h_erased_bits_out + off / 32, db, ((m + 31) / 32) * 4, cudaMemcpyDeviceToHost, t->io_stream));
    }
    CK(cudaStreamSynchronize(t->io_stream));
    t->last = agg;
    if (erased_count) *erased_count = total;
    return DYC_OK;
}

}  // extern "C"

// =============================================================================
// dyc_apply: mixed batches of finds, inserts and erases in batch order.
// The kernels (dyc_apply.cuh) group the ops by key, read every distinct key's
// state before the batch, replay each key's ops in index order, and leave one
// list of keys to erase and one of keys to upsert; the table's own erase and
// insert phases apply those lists (unique keys), so placement, eviction walks,
// overflow handling and the resize policy are the ones dyc_insert/dyc_erase use.
// =============================================================================
namespace {

// Carve the mixed-batch scratch for `n` ops per chunk (grow only).
// Carve an ApplyScratch for `ops` ops and `cells` cells out of one device
// buffer (*buf, grown when too small). ntables > 0 adds the multi-table
// arrays.
dyc_status carve_apply(int kb, int vb, uint64_t ops, uint64_t cells, uint32_t ntables,
                       void **buf, size_t *buf_bytes, dyc::ApplyScratch *out) {
    const bool multi = ntables > 0;
    const size_t K = (size_t)kb, V = (size_t)vb;
    const size_t CB = kb == 4 ? 8 : 16;  // cell bytes
    const size_t sizes[] = {
        cells * CB,                                   // cells
        ops * 4, ops * 4, ops * K, ops * 4, ops * 8,  // op_cell, op_rank, dkey, dcnt, dseg
        ops * 4, ops * V, (ops / 32 + 1) * 4,         // seg, pre_val, pre_hit
        ops * K, ops * V, ops * K,                    // up_key, up_val, er_key
        dyc::kCtrSlots * 8, ops * 4, ops * 4,         // ctr, wseg, mid
        ops * 4,                                      // sort_tmp
        multi ? ops * 4 : 0,                          // dtid
        multi ? ops * 4 : 0, multi ? ops * 4 : 0,     // up_tid, er_tid
        multi ? (size_t)ntables * 4 : 0,              // tup
        multi ? (size_t)ntables * 4 : 0,              // ter
        multi ? ((size_t)ntables + 1) * 4 : 0,        // tcell_off
        multi ? (ops / dyc::kTidxStep + 1) * 4 : 0,   // tidx
        (ops / 32 + 1) * 4};                          // single
    size_t need = 0;
    for (size_t b : sizes) need += (b + 255) & ~(size_t)255;
    if (*buf && *buf_bytes < need) {
        CK(cudaDeviceSynchronize());
        CK(cudaFree(*buf));
        *buf = nullptr;
    }
    if (!*buf) {
        CK(dyc::lib_malloc(buf, need));
        *buf_bytes = need;
    }
    char *p = (char *)*buf;
    int k = 0;
    auto carve = [&]() {
        char *r = sizes[k] ? p : nullptr;
        p += (sizes[k++] + 255) & ~(size_t)255;
        return (void *)r;
    };
    dyc::ApplyScratch A{};
    A.cells = carve();
    A.op_cell = (uint32_t *)carve();
    A.op_rank = (uint32_t *)carve();
    A.dkey = carve();
    A.dcnt = (uint32_t *)carve();
    A.dseg = (unsigned long long *)carve();
    A.seg = (uint32_t *)carve();
    A.pre_val = carve();
    A.pre_hit = (uint32_t *)carve();
    A.up_key = carve();
    A.up_val = carve();
    A.er_key = carve();
    A.ctr = (unsigned long long *)carve();
    A.wseg = (uint32_t *)carve();
    A.mid = (uint32_t *)carve();
    A.sort_tmp = (uint32_t *)carve();
    A.dtid = (uint32_t *)carve();
    A.up_tid = (uint32_t *)carve();
    A.er_tid = (uint32_t *)carve();
    A.tup = (uint32_t *)carve();
    A.ter = (uint32_t *)carve();
    A.tcell_off = (uint32_t *)carve();
    A.tidx = (uint32_t *)carve();
    A.single = (uint32_t *)carve();
    A.ntables = ntables;
    A.cap_cells = cells;
    A.cap_ops = ops;
    *out = A;
    return DYC_OK;
}

// Mixed-batch scratch of a single table for `n` ops per chunk (grow only).
dyc_status ensure_apply(dyc_table *t, uint64_t n) {
    const uint64_t ops = n < 128 ? 128 : n;
    if (!t->d_desc) {
        CK(dyc::lib_malloc(&t->d_desc, sizeof(Desc)));
        CK(dyc::lib_malloc_host(&t->h_desc, sizeof(Desc)));
        memset(t->h_desc, 0, sizeof(Desc));  // differs from any live D: the first push copies
    }
    if (t->apply_buf && t->A.cap_ops >= ops) return DYC_OK;
    if (!t->h_actr) CK(dyc::lib_malloc_host(&t->h_actr, dyc::kCtrSlots * sizeof(unsigned long long)));
    return carve_apply(t->kb, t->vb, ops, 2 * ops, 0, &t->apply_buf, &t->apply_bytes, &t->A);
}

// Copy D to the device if it changed since the last push. The pinned mirror
// is rewritten only after the previous copy has run: every mixed-batch chunk
// ends with a host read of the stream, and a push inside a chunk follows one.
dyc_status push_desc(dyc_table *t, cudaStream_t s) {
    if (memcmp(t->h_desc, &t->D, sizeof(Desc)) == 0) return DYC_OK;
    *t->h_desc = t->D;
    CK(cudaMemcpyAsync(t->d_desc, t->h_desc, sizeof(Desc), cudaMemcpyHostToDevice, s));
    return DYC_OK;
}

dyc_status read_apply_counters(dyc_table *t, cudaStream_t s) {
    CK(cudaMemcpyAsync(t->h_actr, t->A.ctr, dyc::kCtrSlots * sizeof(unsigned long long),
                       cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return DYC_OK;
}

// A chunk of n mixed ops: grouping, scatter and replay (dyc_apply.cuh), then
// the table-set probe kernels (dyc_set.cuh) with this table's one-entry
// descriptor array: the find of the distinct keys, one pass for the erases
// and upserts, the eviction walks. Every kernel reads its item count on the
// device, so the host reads the counters once, at the end. The upsize
// policy (api.cpp:359-369: the size after the batch's erases plus its
// inserts above upper bound x capacity) needs the batch's upsert and erase
// counts: where even n inserts keep the table within deferred_fill() of its
// slots it is applied after the batch with the same counts, so the capacity
// ends as if it had run first (entries the fuller table could not place
// take the overflow path); otherwise the host reads the counts after the
// replay and upsizes first.
dyc_status apply_chunk(dyc_table *t, const uint8_t *ops, const void *keys, const void *vals,
                       uint64_t n, void *vals_out, uint32_t *bits_out, uint32_t flags,
                       cudaStream_t s) {
    const dyc::ApplyScratch &A = t->A;
    const LaunchCtx L = ctx(t, s);
    const uint32_t vb = (uint32_t)t->vb;
    const bool resize = t->cfg.auto_resize && !(flags & DYC_FLAG_NO_RESIZE);
    const bool deferred = !resize || (double)(t->size + n) <= deferred_fill(t) * (double)t->capacity;
    const uint64_t size0 = t->size;
    bool grew = false;
    // nu upserts and ne erases of present keys
    auto upsize_policy = [&](uint64_t nu, uint64_t ne) -> dyc_status {
        int guard = 0;
        while (resize && nu &&
               (double)size0 - (double)ne + (double)nu > t->cfg.upper_load * (double)t->capacity &&
               guard++ < 64) {
            TRY(resize_up_impl(t, s));
            grew = true;
        }
        return DYC_OK;
    };
    // With the policy deferred, keys with a single op in the chunk (most keys
    // of a random batch) skip the per-key passes: compaction lists only keys
    // with several ops, the find, scatter, replays and mutation handle those,
    // and after the replays the one-pass kernel resolves every other op in
    // one probe of its key's buckets (it touches no key the others do). A
    // chunk in which no key repeats (k_apply_group sets the gate) skips
    // compaction and the scatter altogether. The host reads nothing in
    // between; later kernels read counts the skipped ones leave at 0.
    dyc::ApplyScratch Ag = A;
    if (deferred) {
        Ag.gate = &A.ctr[dyc::kCtrRepeat];
        Ag.single_pass = 1u;
    }
    TRY(push_desc(t, s));
    TRY(reset_call_counters(t, s));
    CK(cudaMemsetAsync(A.cells, 0, (size_t)(2 * n) * (t->kb == 4 ? 8 : 16), s));  // 2n cells used
    CK(cudaMemsetAsync(A.ctr, 0, dyc::kCtrSlots * sizeof(unsigned long long), s));
    if (bits_out) CK(cudaMemsetAsync(bits_out, 0, (size_t)((n + 31) / 32) * 4, s));
    cudaError_t e = KB_CALL(t, apply_group, L, Ag, keys, n);
    // state of every distinct key before the batch
    if (e == cudaSuccess)
        e = KB_CALL(t, set_find, L, t->d_desc, 1u, t->sb, A.dkey, nullptr,
                    &A.ctr[dyc::kCtrDistinct], n, A.pre_val, vb, A.pre_hit, &A.ctr[dyc::kCtrBad],
                    t->D.l2_keep != 0u);
    if (e == cudaSuccess)
        e = KB_CALL(t, apply_scatter, L, Ag, n, nullptr, ops, vals, vb, vals_out, bits_out);
    if (e == cudaSuccess) e = KB_CALL(t, apply_replay, L, Ag, ops, vals, vb, vals_out, bits_out, n, n);
    if (e == cudaSuccess && deferred)
        e = KB_CALL(t, apply_unique, L, t->D, t->sb, t->S, ops, keys, vals, vb, vals_out, bits_out,
                    n, t->d_ctr, A.single, Ag.gate);
    if (e != cudaSuccess) return fail(DYC_ECUDA, "apply kernels: %s", cudaGetErrorString(e));
    if (!deferred) {
        TRY(read_apply_counters(t, s));
        TRY(upsize_policy(t->h_actr[dyc::kCtrUp], t->h_actr[dyc::kCtrEr]));
        if (grew) TRY(push_desc(t, s));
    }
    e = KB_CALL(t, set_mutate, L, t->d_desc, 1u, t->d_ctr, t->sb, A.er_key, nullptr,
                &A.ctr[dyc::kCtrEr], A.up_key, A.up_val, vb, nullptr, &A.ctr[dyc::kCtrUp], n,
                t->S.list_a, nullptr, t->S.list_cap, t->d_ctr, &A.ctr[dyc::kCtrBad], nullptr,
                t->D.l2_keep != 0u);
    if (e == cudaSuccess)
        e = KB_CALL(t, set_walk, L, t->d_desc, 1u, t->d_ctr, t->sb, t->S.list_a, nullptr,
                    &t->d_ctr->pending, t->S.list_b, nullptr, &t->d_ctr->overflow,
                    t->S.list_cap, t->cfg.max_evictions, t->d_ctr, t->S.list_cap,
                    &A.ctr[dyc::kCtrBad]);
    if (e != cudaSuccess) return fail(DYC_ECUDA, "apply probe kernels: %s", cudaGetErrorString(e));
    CK(cudaMemcpyAsync(t->h_actr, A.ctr, dyc::kCtrSlots * sizeof(unsigned long long),
                       cudaMemcpyDeviceToHost, s));
    TRY(read_counters(t, s));
    if (t->h_actr[dyc::kCtrBad])
        return fail(DYC_ECUDA, "mixed batch: %llu device counts or ids out of range",
                    t->h_actr[dyc::kCtrBad]);
    const Counters c = *t->h_ctr;
    // both paths' upserts and erases of present keys, as the table counted
    // them (the one-pass kernel counts an insert on a present key as an
    // update even when the value is the same)
    if (deferred) TRY(upsize_policy(c.inserted + c.updated, c.erased));
    dyc_op_stats &St = t->last;
    St.inserted += c.inserted;
    St.updated += c.updated;
    St.erased += c.erased;
    St.evict_steps += c.evict_steps;
    St.overflowed += c.overflow;
    if (c.overflow) {
        TRY(drain(t, s, t->S.list_b, &t->d_ctr->overflow, t->S.list_a, &t->d_ctr->pending,
                  t->S.list_cap, true, !grew));
        St.inserted += t->h_ctr->inserted - c.inserted;
        St.evict_steps += t->h_ctr->evict_steps - c.evict_steps;
    }
    return DYC_OK;
}

// One chunk of a mixed batch whose keys are all distinct (DYC_FLAG_UNIQUE):
// the one-pass kernel, then eviction walks for the inserts it left without a
// slot. The upsize policy counts every insert op of the chunk before it, as
// dyc_insert does (api.cpp:359-369), unless even a chunk of nothing but new
// keys keeps the table within deferred_fill() of its slots; then it runs
// after the chunk on the table's size.
dyc_status apply_unique_chunk(dyc_table *t, const uint8_t *ops, const void *keys, const void *vals,
                              uint64_t n, void *vals_out, uint32_t *bits_out, uint32_t flags,
                              cudaStream_t s) {
    const bool resize = t->cfg.auto_resize && !(flags & DYC_FLAG_NO_RESIZE);
    const bool before = resize && (double)(t->size + n) > deferred_fill(t) * (double)t->capacity;
    TRY(reset_call_counters(t, s));
    if (before) {
        cudaError_t e = KB_CALL(t, count_inserts, ctx(t, s), ops, n, &t->d_ctr->nins);
        if (e != cudaSuccess) return fail(DYC_ECUDA, "count kernel: %s", cudaGetErrorString(e));
        TRY(read_counters(t, s));
        const uint64_t nins = t->h_ctr->nins;
        int guard = 0;
        while (nins && (double)(t->size + nins) > t->cfg.upper_load * (double)t->capacity &&
               guard++ < 64)
            TRY(resize_up_impl(t, s));
    }
    cudaError_t e = KB_CALL(t, apply_unique, ctx(t, s), t->D, t->sb, t->S, ops, keys, vals,
                            (uint32_t)t->vb, vals_out, bits_out, n, t->d_ctr);
    if (e != cudaSuccess) return fail(DYC_ECUDA, "apply kernel: %s", cudaGetErrorString(e));
    e = KB_CALL(t, walk, ctx(t, s), t->D, t->sb, t->S.list_a, &t->d_ctr->pending, t->S.list_b,
                &t->d_ctr->overflow, t->S.list_cap, t->cfg.max_evictions, true, t->d_ctr,
                t->S.list_cap);
    if (e != cudaSuccess) return fail(DYC_ECUDA, "walk kernel: %s", cudaGetErrorString(e));
    TRY(read_counters(t, s));
    const Counters c = *t->h_ctr;
    dyc_op_stats &St = t->last;
    St.inserted += c.inserted;
    St.updated += c.updated;
    St.erased += c.erased;
    St.evict_steps += c.evict_steps;
    St.overflowed += c.overflow;
    bool grew = false;
    if (c.overflow) {
        TRY(drain(t, s, t->S.list_b, &t->d_ctr->overflow, t->S.list_a, &t->d_ctr->pending,
                  t->S.list_cap, true, true));
        St.inserted += t->h_ctr->inserted - c.inserted;
        St.evict_steps += t->h_ctr->evict_steps - c.evict_steps;
        grew = true;
    }
    if (resize && !before && !grew) {
        int guard = 0;
        while ((double)t->size > t->cfg.upper_load * (double)t->capacity && guard++ < 64)
            TRY(resize_up_impl(t, s));
    }
    return DYC_OK;
}

}  // namespace

extern "C" dyc_status dyc_apply(dyc_table *t, const uint8_t *d_ops, const void *d_keys,
                                const void *d_vals, uint64_t n, void *d_vals_out,
                                uint32_t *d_bits_out, uint32_t flags, void *stream) {
    if (!t) return fail(DYC_EINVAL, "null table");
    TRY(set_device(t));
    cudaStream_t s = (cudaStream_t)stream;
    t->last = dyc_op_stats{};
    TRY(settle_held(t, s));
    if (n == 0) return DYC_OK;
    if (!d_ops || !d_keys || !d_vals) return fail(DYC_EINVAL, "null op, key or value array");
    const uint64_t chunk = t->chunk;
    const uint64_t m0 = n < chunk ? n : chunk;
    const bool unique = (flags & DYC_FLAG_UNIQUE) != 0;
    if (!unique) TRY(ensure_apply(t, m0));
    TRY(ensure_scratch(t, m0));
    for (uint64_t off = 0; off < n; off += chunk) {
        const uint64_t m = (n - off) < chunk ? (n - off) : chunk;
        const char *k = (const char *)d_keys + off * t->kb, *v = (const char *)d_vals + off * t->vb;
        void *o = d_vals_out ? (char *)d_vals_out + off * t->vb : nullptr;
        uint32_t *b = d_bits_out ? d_bits_out + off / 32 : nullptr;
        if (unique) TRY(apply_unique_chunk(t, d_ops + off, k, v, m, o, b, flags, s));
        else TRY(apply_chunk(t, d_ops + off, k, v, m, o, b, flags, s));
    }
    // downsize check after the batch, as after an erase batch (api.cpp:494-505)
    if (t->cfg.auto_resize && !(flags & DYC_FLAG_NO_RESIZE) &&
        (double)t->size < t->cfg.lower_load * (double)t->capacity &&
        t->capacity > t->cfg.min_downsize_capacity) {
        const dyc_op_stats keep = t->last;
        dyc_status st = resize_down_impl(t, s);
        if (st != DYC_OK && st != DYC_EINVAL) return st;
        const uint64_t downs = t->last.resizes_down, ups = t->last.resizes_up;
        t->last = keep;
        t->last.resizes_down = downs;
        t->last.resizes_up = ups;
    }
    return DYC_OK;
}

// =============================================================================
// dyc_erase_noalloc: erase whose batch-dedup table lives in a fixed device
// array compiled into this file, for callers that must not allocate device
// memory during the call (see include/dycuckoo.h).
// =============================================================================
#include <mutex>

namespace {

constexpr uint64_t kNoAllocMaxKeys = 1ull << 18;         // keys per call
constexpr uint64_t kNoAllocCells = 2 * kNoAllocMaxKeys;  // dedup cells, a power of two
// key cells (8 bytes each) followed by the op-index cells 8-byte keys need
constexpr size_t kNoAllocBytes = (size_t)kNoAllocCells * 8 + (size_t)kNoAllocCells * 4;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
constexpr int kNoAllocMaxDevices = 256;
void *g_noalloc_addr[kNoAllocMaxDevices];  // device address of the array, per device

// One-time per-device set-up, with that device current: the array's name is
// only a host-side stand-in, so kernels get the address the runtime reports.
dyc_status noalloc_scratch(int device, void **out) {
    if (device < 0 || device >= kNoAllocMaxDevices)
        return fail(DYC_EINVAL, "device %d out of range for the no-alloc scratch", device);
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_addr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(DYC_ECUDA, "cudaGetSymbolAddress(no-alloc scratch) on device %d: %s",
                        device, cudaGetErrorString(e));
        g_noalloc_addr[device] = p;
    }
    *out = g_noalloc_addr[device];
    return DYC_OK;
}

}  // namespace

extern "C" dyc_status dyc_erase_noalloc(dyc_table *t, const void *d_keys, uint64_t n,
                                        uint32_t *d_erased_bits_out, uint64_t *h_erased_count,
                                        uint32_t flags, void *stream) {
    if (!t) return fail(DYC_EINVAL, "null table");
    if (h_erased_count) *h_erased_count = 0;
    if (n > kNoAllocMaxKeys)
        return fail(DYC_EINVAL, "dyc_erase_noalloc takes at most %llu keys per call, got %llu",
                    (unsigned long long)kNoAllocMaxKeys, (unsigned long long)n);
    if (n == 0) return DYC_OK;
    if (!d_keys) return fail(DYC_EINVAL, "null key array");
    if (t->held_n)  // placing them may need memory: an allocating call must come first
        return fail(DYC_ENOMEM, "%llu entries are held from a failed call; an allocating "
                    "call on the table places them first", (unsigned long long)t->held_n);
    TRY(set_device(t));
    void *base = nullptr;
    TRY(noalloc_scratch(t->device, &base));
    cudaStream_t s = (cudaStream_t)stream;
    // this call's dedup table: the first dedup_cap cells of the array (the
    // kernels take their mask from dedup_cap), as the allocating path sizes
    // its own; the index array of 8-byte keys keeps its fixed offset
    Scratch S{};
    S.dedup = base;
    S.dedup_cap = next_pow2(2 * (n < 16 ? 16 : n));  // <= kNoAllocCells for n <= the limit
    S.dedup_idx = t->kb == 8 ? (uint32_t *)((char *)base + kNoAllocCells * 8) : nullptr;
    const bool use_dedup = !(flags & DYC_FLAG_UNIQUE) && n > 1;
    t->last = dyc_op_stats{};
    TRY(reset_call_counters(t, s));
    if (use_dedup) {
        // the array keeps the previous call's cells: clear the ones this call uses
        CK(cudaMemsetAsync(S.dedup, 0, (size_t)S.dedup_cap * 8, s));
        if (S.dedup_idx) CK(cudaMemsetAsync(S.dedup_idx, 0xFF, (size_t)S.dedup_cap * 4, s));
        cudaError_t e = KB_CALL(t, dedup, ctx(t, s), S, d_keys, n, dyc::kKeepFirst);
        if (e != cudaSuccess) return fail(DYC_ECUDA, "dedup kernel: %s", cudaGetErrorString(e));
    }
    cudaError_t e = KB_CALL(t, erase, ctx(t, s), t->D, t->sb, S, use_dedup, d_keys, n,
                            d_erased_bits_out, t->d_ctr);
    if (e != cudaSuccess) return fail(DYC_ECUDA, "erase kernel: %s", cudaGetErrorString(e));
    TRY(read_counters(t, s));
    t->last.erased = t->h_ctr->erased;
    t->last.superseded = t->h_ctr->superseded;
    if (h_erased_count) *h_erased_count = t->h_ctr->erased;
    return DYC_OK;
}

// =============================================================================
// Table sets: many independent tables whose mixed batches are served by one
// launch sequence (include/dycuckoo.h, dyc_set_*). Each phase is one
// grid-stride launch over a work list that spans every table; an item reads
// its table's descriptor from a device array. Member tables are ordinary
// dyc_tables whose counters live in one set-owned array, so resizes,
// overflow handling and single-table calls reuse the code above.
// =============================================================================
#include <algorithm>
#include <vector>

struct dyc_set {
    dyc_config cfg;
    int kb = 4, vb = 4, sb = 128, sms = 0, device = 0;
    uint32_t ntables = 0;
    std::vector<dyc_table *> tables;
    Counters *d_tctr = nullptr, *h_tctr = nullptr;  // per-table counters
    Desc *d_desc = nullptr, *h_desc = nullptr;      // per-table descriptors (pinned mirror)
    Counters *d_gctr = nullptr, *h_gctr = nullptr;  // set-wide counters of one call
    unsigned long long *h_actr = nullptr;   // pinned copy of the batch counters (A.ctr)
    unsigned long long *h_hostn = nullptr;  // pinned: the op count of the current batch
    void *abuf = nullptr;
    size_t abytes = 0;
    dyc::ApplyScratch A{};
    void *lbuf = nullptr;
    size_t lbytes = 0;
    void *list_a = nullptr, *list_b = nullptr;
    uint32_t *tid_a = nullptr, *tid_b = nullptr;
    uint64_t list_cap = 0;
    uint32_t *h_tup = nullptr, *h_ter = nullptr;  // pinned copies of A.tup / A.ter
    uint32_t *d_bits_tmp = nullptr;        // dyc_set_apply_each: one table's result bits
    size_t bits_tmp_words = 0;
    // CUDA graphs of the launch sequences (phase A, phase B, both), one entry
    // per buffer set: the kernels read the op count on the device and size
    // their grids by the scratch capacity, so one graph serves any batch size
    struct Graph {
        std::vector<uintptr_t> key;
        // phase A, phase B, both, and the device policy + upsizes + phase B
        cudaGraphExec_t exec[4] = {nullptr, nullptr, nullptr, nullptr};
        bool warm = false;
        uint64_t used = 0;
    };
    std::vector<Graph> graphs;
    uint64_t graph_clock = 0;
    cudaStream_t cap_stream = nullptr;  // capture stream (the caller's may be the legacy one)
    cudaStream_t side = nullptr;        // replays that run beside the main sequence
    cudaEvent_t fork = nullptr, join = nullptr;
    uint32_t blocks_per_sm = 0;  // launch cap of the set kernels (0: as many as fit)
    uint32_t max_evict_all = 0;  // largest member eviction bound
    dyc_op_stats last{};
    // device half of the upsize policy (cfg.device_upsize == 0, auto_resize):
    // one upsize target per member, allocated ahead (h_spare, its device copy
    // d_spare refreshed at every round), the moves k_set_policy lists, which
    // members it upsized, and the buffers they replaced (freed at the next call)
    bool spares = false;
    dyc::Spare *d_spare = nullptr, *h_spare = nullptr;
    dyc::ResizeJob *d_jobs = nullptr;
    dyc::SetPolicyOut *d_pout = nullptr, *h_pout = nullptr;
    uint8_t *d_grew = nullptr, *h_grew = nullptr;
    std::vector<std::pair<void *, uint64_t>> free_later;  // (block, bytes)
    uint64_t free_later_bytes = 0;
    // replaced subtables kept for reuse as later spares, by size, up to
    // spare_cache_cap bytes: a stream-ordered allocation or free costs the
    // host ~1.7 us when it next synchronises, and a round upsizes hundreds
    // of members
    std::multimap<uint64_t, void *> spare_cache;
    uint64_t spare_cache_bytes = 0, spare_cache_cap = 0;
    // the batch of the current dyc_set_apply (phase B resolves its keys with
    // one op there; a captured graph is keyed by these pointers)
    struct Batch {
        const uint32_t *off = nullptr;
        const uint8_t *ops = nullptr;
        const void *keys = nullptr, *vals = nullptr;
        void *out = nullptr;
        uint32_t *bits = nullptr;
    } cur;
};

namespace {

constexpr size_t kSetGraphs = 4;  // cached buffer sets (a server uses one per staging slot)

void set_drop_graph(dyc_set::Graph &g) {
    for (auto &x : g.exec)
        if (x) {
            cudaGraphExecDestroy(x);
            x = nullptr;
        }
    g.warm = false;
}

void set_drop_graphs(dyc_set *s) {
    for (auto &g : s->graphs) set_drop_graph(g);
    s->graphs.clear();
}

// The cache entry for this buffer set (least recently used one replaced).
dyc_set::Graph *set_graph_for(dyc_set *s, std::vector<uintptr_t> &&key) {
    ++s->graph_clock;
    for (auto &g : s->graphs)
        if (g.key == key) {
            g.used = s->graph_clock;
            return &g;
        }
    if (s->graphs.size() < kSetGraphs) {
        s->graphs.emplace_back();
    } else {
        auto lru = std::min_element(s->graphs.begin(), s->graphs.end(),
                                    [](const dyc_set::Graph &a, const dyc_set::Graph &b) {
                                        return a.used < b.used;
                                    });
        set_drop_graph(*lru);
        std::swap(*lru, s->graphs.back());
    }
    dyc_set::Graph &g = s->graphs.back();
    g.key = std::move(key);
    g.used = s->graph_clock;
    return &g;
}

dyc_status set_push_descs(dyc_set *s, cudaStream_t st) {
    for (uint32_t t = 0; t < s->ntables; ++t) s->h_desc[t] = s->tables[t]->D;
    CK(cudaMemcpyAsync(s->d_desc, s->h_desc, sizeof(Desc) * s->ntables, cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));  // the pinned mirror is rewritten by the next push
    return DYC_OK;
}

// Push the descriptors again if any member changed since the last push.
dyc_status set_refresh_descs(dyc_set *s, cudaStream_t st) {
    for (uint32_t t = 0; t < s->ntables; ++t)
        if (memcmp(&s->h_desc[t], &s->tables[t]->D, sizeof(Desc)) != 0) return set_push_descs(s, st);
    return DYC_OK;
}

// Scratch for batches of up to n ops over the set (grow only).
dyc_status set_ensure_scratch(dyc_set *s, uint64_t n) {
    const uint64_t ops = n < 128 ? 128 : n;
    if (s->abuf && s->A.cap_ops >= ops) return DYC_OK;
    set_drop_graphs(s);
    TRY(carve_apply(s->kb, s->vb, ops, 2 * ops, s->ntables, &s->abuf, &s->abytes, &s->A));
    s->A.single_pass = 1u;  // keys with one op in a batch: k_set_unique in phase B
    const size_t slot = s->kb == 4 ? 8 : 16;
    const size_t lb = ((ops * slot + 255) & ~(size_t)255) * 2 + ((ops * 4 + 255) & ~(size_t)255) * 2;
    if (s->lbuf) {
        CK(cudaDeviceSynchronize());
        CK(cudaFree(s->lbuf));
        s->lbuf = nullptr;
    }
    CK(dyc::lib_malloc(&s->lbuf, lb));
    s->lbytes = lb;
    char *p = (char *)s->lbuf;
    const size_t ls = (ops * slot + 255) & ~(size_t)255, lt = (ops * 4 + 255) & ~(size_t)255;
    s->list_a = p;
    s->list_b = p + ls;
    s->tid_a = (uint32_t *)(p + 2 * ls);
    s->tid_b = (uint32_t *)(p + 2 * ls + lt);
    s->list_cap = ops;
    return DYC_OK;
}

#define SET_KB_CALL(s, fn, ...) ((s)->kb == 4 ? Ops<4>::fn(__VA_ARGS__) : Ops<8>::fn(__VA_ARGS__))

// Phase A: group, scatter, pre-batch find, replay; counters to the host.
// Every kernel reads the op count from d_off[ntables] on the device; n (the
// scratch capacity under a graph) only sizes the grids.
dyc_status set_phase_a(dyc_set *s, const uint32_t *d_off, const uint8_t *ops, const void *keys,
                       const void *vals, void *out, uint32_t *bits, uint64_t n, bool new_counts,
                       cudaStream_t st) {
    const dyc::ApplyScratch &A = s->A;
    const LaunchCtx L{s->sms, st, (int)s->blocks_per_sm, s->side, s->fork, s->join};
    const uint32_t vb = (uint32_t)s->vb;
    const uint32_t *d_n = d_off + s->ntables;
    // the op count the host's offsets declare, which bounds the device's
    // (a pinned word: a captured graph copies its current value)
    CK(cudaMemcpyAsync(&A.ctr[dyc::kCtrHostN], s->h_hostn, sizeof(unsigned long long),
                       cudaMemcpyHostToDevice, st));
    // also zeroes phase B's counters (nothing between the phases uses them)
    cudaError_t e = SET_KB_CALL(s, set_group, L, A, d_off, keys, n, bits, s->d_gctr);
    if (e == cudaSuccess)
        e = SET_KB_CALL(s, set_find, L, s->d_desc, s->ntables, s->sb, A.dkey, A.dtid,
                        &A.ctr[dyc::kCtrDistinct], n, A.pre_val, vb, A.pre_hit,
                        &A.ctr[dyc::kCtrBad], s->tables[0]->D.l2_keep != 0u);
    if (e == cudaSuccess)
        e = SET_KB_CALL(s, apply_scatter, L, A, n, d_n, ops, vals, vb, out, bits);
    if (e == cudaSuccess)
        e = SET_KB_CALL(s, apply_replay, L, A, ops, vals, vb, out, bits, n, n, d_n);
    if (e != cudaSuccess) return fail(DYC_ECUDA, "set phase A kernels: %s", cudaGetErrorString(e));
    if (new_counts)  // each table's upserts, for the upsize decision
    {
        CK(cudaMemcpyAsync(s->h_tup, A.tup, (size_t)s->ntables * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(s->h_ter, A.ter, (size_t)s->ntables * 4, cudaMemcpyDeviceToHost, st));
    }
    return DYC_OK;
}

// Phase B: erase list, upsert list, eviction walks; counters to the host.
// hold: a device word that, when nonzero, makes the pass do nothing (the
// device policy found a member the host must upsize further first).
dyc_status set_phase_b(dyc_set *s, uint64_t n, cudaStream_t st, const uint32_t *hold = nullptr) {
    const dyc::ApplyScratch &A = s->A;
    const LaunchCtx L{s->sms, st, (int)s->blocks_per_sm};
    cudaError_t e = cudaSuccess;
    if (A.single_pass)  // keys with one op in the batch, after the policy's upsizes
        e = SET_KB_CALL(s, set_unique, L, A, s->cur.off, s->d_desc, s->ntables, s->d_tctr, s->sb,
                        s->cur.ops, s->cur.keys, s->cur.vals, (uint32_t)s->vb, s->cur.out,
                        s->cur.bits, n, s->list_a, s->tid_a, s->list_cap, s->d_gctr, hold,
                        s->tables[0]->D.l2_keep != 0u);
    if (e == cudaSuccess)
        e = SET_KB_CALL(s, set_mutate, L, s->d_desc, s->ntables, s->d_tctr, s->sb, A.er_key,
                        A.er_tid, &A.ctr[dyc::kCtrEr], A.up_key, A.up_val, (uint32_t)s->vb,
                        A.up_tid, &A.ctr[dyc::kCtrUp], n, s->list_a, s->tid_a, s->list_cap,
                        s->d_gctr, &A.ctr[dyc::kCtrBad], hold, s->tables[0]->D.l2_keep != 0u);
    if (e == cudaSuccess)
        e = SET_KB_CALL(s, set_walk, L, s->d_desc, s->ntables, s->d_tctr, s->sb, s->list_a,
                        s->tid_a, &s->d_gctr->pending, s->list_b, s->tid_b,
                        &s->d_gctr->overflow, s->list_cap, s->max_evict_all, s->d_gctr,
                        s->list_cap, &A.ctr[dyc::kCtrBad]);
    if (e != cudaSuccess) return fail(DYC_ECUDA, "set phase B kernels: %s", cudaGetErrorString(e));
    CK(cudaMemcpyAsync(s->h_actr, A.ctr, dyc::kCtrSlots * sizeof(unsigned long long),
                       cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(s->h_gctr, s->d_gctr, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(s->h_tctr, s->d_tctr, sizeof(Counters) * s->ntables,
                       cudaMemcpyDeviceToHost, st));
    return DYC_OK;
}

// ---- device half of the upsize policy ----------------------------------------
// Replaced subtables and spares that no longer fit, from the previous call
// (no kernel of this call reads them): kept in the spare cache while it has
// room, else freed (stream-ordered).
dyc_status set_release_later(dyc_set *s, cudaStream_t st) {
    for (const auto &b : s->free_later) {
        if (s->spare_cache_bytes + b.second <= s->spare_cache_cap) {
            s->spare_cache.emplace(b.second, b.first);
            s->spare_cache_bytes += b.second;
        } else {
            CK(cudaFreeAsync(b.first, st));
        }
    }
    s->free_later.clear();
    s->free_later_bytes = 0;
    return DYC_OK;
}

// A block of at least `bytes` (and at most a quarter more) from the spare
// cache, or null.
void *set_cached_block(dyc_set *s, uint64_t bytes) {
    auto it = s->spare_cache.lower_bound(bytes);
    if (it == s->spare_cache.end() || it->first - bytes > bytes / 4) return nullptr;
    void *p = it->second;
    s->spare_cache_bytes -= it->first;
    s->spare_cache.erase(it);
    return p;
}

// Give every member a spare that fits its next upsize (subtable pick_up with
// its current bucket count, doubled). Issued while phase A runs on the
// device; allocations are stream-ordered on st. A member whose spare cannot
// be allocated has none this round: the device policy hands it to the host.
void set_fill_spares(dyc_set *s, cudaStream_t st) {
    for (uint32_t t = 0; t < s->ntables; ++t) {
        const dyc_table *m = s->tables[t];
        const uint32_t ti = pick_up(m->D.nb, m->D.d), onb = m->D.nb[ti];
        dyc::Spare &sp = s->h_spare[t];
        if (sp.new_sub && sp.ti == ti && sp.old_nb == onb) continue;
        if (sp.new_sub) {
            s->free_later.emplace_back(sp.new_sub, 2ull * sp.old_nb * m->sb);
            s->free_later_bytes += 2ull * sp.old_nb * m->sb;
        }
        sp = dyc::Spare{nullptr, 0u, 0u};
        if (onb == 0 || (uint64_t)onb * 2 > 0xFFFFFFFFull) continue;
        const uint64_t need = 2ull * onb * m->sb;
        void *p = set_cached_block(s, need);
        if (!p && pool_alloc(s->device, &p, need, st) != cudaSuccess) {
            (void)cudaGetLastError();
            continue;
        }
        sp = dyc::Spare{p, ti, onb};
    }
}

// Spare targets to the device, the policy, the listed upsizes, phase B
// (held back when the host must finish the policy), and what the policy
// did back to the host. One capturable sequence.
dyc_status set_policy_and_b(dyc_set *s, uint64_t n, cudaStream_t st) {
    const LaunchCtx L{s->sms, st, (int)s->blocks_per_sm};
    CK(cudaMemcpyAsync(s->d_spare, s->h_spare, sizeof(dyc::Spare) * s->ntables,
                       cudaMemcpyHostToDevice, st));
    cudaError_t e = SET_KB_CALL(s, set_policy, L, s->d_desc, s->ntables, s->d_tctr, s->A.tup,
                                s->A.ter, s->d_spare, s->cfg.upper_load,
                                (uint32_t)s->tables[0]->slots, s->sb, s->d_jobs, s->d_grew,
                                s->d_pout);
    if (e == cudaSuccess)
        e = SET_KB_CALL(s, resize_up_list, L, s->sb, s->d_jobs, s->d_pout, s->ntables);
    if (e != cudaSuccess) return fail(DYC_ECUDA, "set upsize policy: %s", cudaGetErrorString(e));
    TRY(set_phase_b(s, n, st, &s->d_pout->host));
    CK(cudaMemcpyAsync(s->h_pout, s->d_pout, sizeof(dyc::SetPolicyOut), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(s->h_grew, s->d_grew, s->ntables, cudaMemcpyDeviceToHost, st));
    return DYC_OK;
}

// The members the device upsized: their host descriptors follow the device
// ones (the spare became subtable ti), the old subtable is freed at the next
// call, and grew[t] is set as for a host upsize of the policy.
void set_take_device_upsizes(dyc_set *s, std::vector<uint8_t> &grew) {
    for (uint32_t t = 0; t < s->ntables; ++t) {
        if (!s->h_grew[t]) continue;
        dyc_table *m = s->tables[t];
        dyc::Spare &sp = s->h_spare[t];
        const uint32_t ti = sp.ti, nnb = 2u * sp.old_nb;
        s->free_later.emplace_back(m->D.sub[ti], (uint64_t)sp.old_nb * m->sb);
        s->free_later_bytes += (uint64_t)sp.old_nb * m->sb;
        m->D.sub[ti] = sp.new_sub;
        m->D.nb[ti] = nnb;
        m->D.magic[ti] = dyc::fastmod_magic(nnb);
        m->capacity += (uint64_t)sp.old_nb * m->slots;
        refresh_l2(m);
        m->last.resizes_up++;
        sp = dyc::Spare{nullptr, 0u, 0u};
        s->h_desc[t] = m->D;  // the device descriptor is already this one
        if (grew.empty()) grew.assign(s->ntables, 0);
        grew[t] = 1;
    }
}

// Run a launch sequence issue(stream) directly on st, or through its
// captured graph in entry g (captured on the second call with the same
// buffers, after one direct run has warmed the launch-configuration caches).
// Capture runs on the set's own stream, since the legacy default stream
// cannot be captured; the graph is then launched on st.
template <class F>
dyc_status set_run(dyc_set *s, dyc_set::Graph *g, int which, cudaStream_t st, F &&issue) {
    if (!g || !g->warm) return issue(st);
    if (!g->exec[which]) {
        if (!s->cap_stream) CK(cudaStreamCreateWithFlags(&s->cap_stream, cudaStreamNonBlocking));
        const cudaStream_t cs = s->cap_stream;
        CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        dyc_status r = issue(cs);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(cs, &graph);
        if (r != DYC_OK) {
            if (graph) cudaGraphDestroy(graph);
            return r;
        }
        if (e != cudaSuccess) return fail(DYC_ECUDA, "stream capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&g->exec[which], graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(DYC_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
    }
    CK(cudaGraphLaunch(g->exec[which], st));
    return DYC_OK;
}

// Entries whose eviction walks reached the bound: place them per table after
// an upsize of that table (never dropped).
// Tables with grew[t] set were upsized by the policy after the batch: their
// entries are placed without the extra upsize an overflow otherwise takes.
dyc_status set_overflow(dyc_set *s, uint64_t cnt, const std::vector<uint8_t> &grew,
                        cudaStream_t st) {
    const size_t slot = s->kb == 4 ? 8 : 16;
    std::vector<unsigned char> ent(cnt * slot);
    std::vector<uint32_t> tid(cnt);
    CK(cudaMemcpyAsync(ent.data(), s->list_b, cnt * slot, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(tid.data(), s->tid_b, cnt * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::vector<std::vector<uint64_t>> per(s->ntables);
    for (uint64_t i = 0; i < cnt; ++i) {
        if (tid[i] >= s->ntables)
            return fail(DYC_ECUDA, "overflow entry %llu names table %u of %u",
                        (unsigned long long)i, tid[i], s->ntables);
        per[tid[i]].push_back(i);
    }
    for (uint32_t t = 0; t < s->ntables; ++t) {
        if (per[t].empty()) continue;
        dyc_table *m = s->tables[t];
        const uint64_t c = per[t].size();
        std::vector<unsigned char> hk(c * s->kb), hv(c * s->vb);
        for (uint64_t j = 0; j < c; ++j) {
            const unsigned char *e = ent.data() + per[t][j] * slot;
            // a 4-byte-key slot is key | value << 32; an 8-byte-key slot is {key, value}
            memcpy(hk.data() + j * s->kb, e, s->kb);
            memcpy(hv.data() + j * s->vb, e + (s->kb == 4 ? 4 : 8), s->vb);
        }
        // an upsize or scratch the pool cannot serve: this table's entries and
        // those of the tables after it are held by their tables (not dropped)
        auto hold_rest = [&](uint32_t from, dyc_status why) -> dyc_status {
            const std::string msg = g_err;
            uint64_t held = 0;
            for (uint32_t u = from; u < s->ntables; ++u) {
                dyc_table *mu = s->tables[u];
                for (uint64_t i : per[u]) {
                    const unsigned char *e = ent.data() + i * slot;
                    mu->held.insert(mu->held.end(), e, e + slot);
                }
                mu->held_n += per[u].size();
                held += per[u].size();
            }
            return fail(why, "%s; %llu entries held by their tables for the next call",
                        msg.c_str(), (unsigned long long)held);
        };
        dyc_status r = ensure_io(m, c * (s->kb + s->vb) + 256);
        if (r == DYC_OK) r = ensure_scratch(m, c);
        if (r == DYC_OK && (grew.empty() || !grew[t])) r = resize_up_impl(m, st);
        for (int guard = 0; r == DYC_OK && guard < 64 &&
                            (double)(m->size + c) > m->cfg.upper_load * (double)m->capacity;
             ++guard)
            r = resize_up_impl(m, st);
        if (r != DYC_OK) return hold_rest(t, r);
        char *dk = (char *)m->d_io, *dv = dk + ((c * s->kb + 255) & ~(uint64_t)255);
        CK(cudaMemcpyAsync(dk, hk.data(), c * s->kb, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(dv, hv.data(), c * s->vb, cudaMemcpyHostToDevice, st));
        // a failure inside holds this table's unplaced entries (drain)
        r = insert_chunk(m, dk, dv, c, DYC_FLAG_UNIQUE | DYC_FLAG_NEW_KEYS, st);
        if (r != DYC_OK) return hold_rest(t + 1, r);
        CK(cudaStreamSynchronize(st));  // hk / hv and the io buffer are reused
        s->last.resizes_up += m->last.resizes_up;
        m->last = dyc_op_stats{};
    }
    return DYC_OK;
}

__global__ void k_bits_merge(uint32_t *__restrict__ dst, uint64_t dst_bit,
                             const uint32_t *__restrict__ src, uint64_t m) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride)
        if ((src[i >> 5] >> (i & 31)) & 1u) {
            const uint64_t b = dst_bit + i;
            atomicOr(&dst[b >> 5], 1u << (b & 31));
        }
}

bool set_args_ok(const dyc_set *s, const uint32_t *d_off, const uint32_t *h_off,
                 const uint8_t *ops, const void *keys, const void *vals, uint64_t *n_out) {
    if (!s || !d_off || !h_off) return (fail(DYC_EINVAL, "null set or offsets"), false);
    if (h_off[0] != 0) return (fail(DYC_EINVAL, "offsets must start at 0"), false);
    for (uint32_t t = 0; t < s->ntables; ++t)
        if (h_off[t + 1] < h_off[t]) return (fail(DYC_EINVAL, "offsets must not decrease"), false);
    *n_out = h_off[s->ntables];
    if (*n_out && (!ops || !keys || !vals))
        return (fail(DYC_EINVAL, "null op, key or value array"), false);
    return true;
}

}  // namespace

extern "C" {

dyc_status dyc_set_create(const dyc_config *cfg, uint32_t ntables, const uint64_t *sizes,
                          const uint32_t *num_subtables, dyc_set **out) {
    if (!cfg || !out || !sizes || ntables == 0) return fail(DYC_EINVAL, "null argument or no tables");
    *out = nullptr;
    char why[128];
    if (!valid_config(cfg, why, sizeof(why))) return fail(DYC_EINVAL, "%s", why);
    dyc_set *s = new (std::nothrow) dyc_set();
    if (!s) return fail(DYC_ENOMEM, "host allocation");
    s->cfg = *cfg;
    s->kb = (int)cfg->key_bytes;
    s->vb = (int)cfg->value_bytes;
    s->sb = (int)cfg->bucket_bytes;
    s->device = cfg->device;
    s->ntables = ntables;
    auto undo = [&](dyc_status r) {
        dyc_set_destroy(s);
        return r;
    };
    cudaError_t e = cudaSetDevice(s->device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
    if (e == cudaSuccess) e = dyc::lib_malloc(&s->d_tctr, sizeof(Counters) * ntables);
    if (e == cudaSuccess) e = cudaMemset(s->d_tctr, 0, sizeof(Counters) * ntables);
    if (e == cudaSuccess) e = dyc::lib_malloc_host(&s->h_tctr, sizeof(Counters) * ntables);
    if (e == cudaSuccess) e = dyc::lib_malloc(&s->d_desc, sizeof(Desc) * ntables);
    if (e == cudaSuccess) e = dyc::lib_malloc_host(&s->h_desc, sizeof(Desc) * ntables);
    if (e == cudaSuccess) e = dyc::lib_malloc(&s->d_gctr, sizeof(Counters));
    if (e == cudaSuccess) e = dyc::lib_malloc_host(&s->h_gctr, sizeof(Counters));
    if (e == cudaSuccess)
        e = dyc::lib_malloc_host(&s->h_actr, sizeof(unsigned long long) * dyc::kCtrSlots);
    if (e == cudaSuccess) e = dyc::lib_malloc_host(&s->h_hostn, sizeof(unsigned long long));
    if (e == cudaSuccess) e = dyc::lib_malloc_host(&s->h_tup, sizeof(uint32_t) * ntables);
    if (e == cudaSuccess) e = dyc::lib_malloc_host(&s->h_ter, sizeof(uint32_t) * ntables);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->join, cudaEventDisableTiming);
    s->spares = cfg->auto_resize && cfg->device_upsize == 0u;
    if (s->spares) {
        if (e == cudaSuccess) e = dyc::lib_malloc(&s->d_spare, sizeof(dyc::Spare) * ntables);
        if (e == cudaSuccess) e = dyc::lib_malloc_host(&s->h_spare, sizeof(dyc::Spare) * ntables);
        if (e == cudaSuccess) e = dyc::lib_malloc(&s->d_jobs, sizeof(dyc::ResizeJob) * ntables);
        if (e == cudaSuccess) e = dyc::lib_malloc(&s->d_pout, sizeof(dyc::SetPolicyOut));
        if (e == cudaSuccess) e = dyc::lib_malloc_host(&s->h_pout, sizeof(dyc::SetPolicyOut));
        if (e == cudaSuccess) e = dyc::lib_malloc(&s->d_grew, ntables);
        if (e == cudaSuccess) e = dyc::lib_malloc_host(&s->h_grew, ntables);
        if (e == cudaSuccess) {
            memset(s->h_spare, 0, sizeof(dyc::Spare) * ntables);
            memset(s->h_pout, 0, sizeof(dyc::SetPolicyOut));
            memset(s->h_grew, 0, ntables);
        }
    }
    if (e != cudaSuccess) return undo(fail(DYC_ENOMEM, "set setup: %s", cudaGetErrorString(e)));
    memset(s->h_tctr, 0, sizeof(Counters) * ntables);
    s->tables.assign(ntables, nullptr);
    for (uint32_t t = 0; t < ntables; ++t) {
        dyc_config c = *cfg;
        c.initial_size = sizes[t];
        if (num_subtables) c.num_subtables = num_subtables[t];
        dyc_status r = create_impl(&c, s->d_tctr + t, s->h_tctr + t, false, &s->tables[t]);
        if (r != DYC_OK) return undo(r);
    }
    if (s->spares) {  // the spare cache keeps up to a quarter of the members' bytes
        uint64_t bytes = 0;
        for (const dyc_table *m : s->tables)
            for (uint32_t k = 0; k < m->D.d; ++k) bytes += (uint64_t)m->D.nb[k] * m->sb;
        s->spare_cache_cap = bytes / 4;
    }
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return undo(fail(DYC_ECUDA, "set setup: %s", cudaGetErrorString(e)));
    s->max_evict_all = cfg->max_evictions;
    dyc_status r = set_push_descs(s, 0);
    if (r != DYC_OK) return undo(r);
    *out = s;
    return DYC_OK;
}

dyc_status dyc_set_destroy(dyc_set *s) {
    if (!s) return DYC_OK;
    cudaSetDevice(s->device);
    cudaDeviceSynchronize();
    set_drop_graphs(s);
    if (s->cap_stream) cudaStreamDestroy(s->cap_stream);
    if (s->side) cudaStreamDestroy(s->side);
    if (s->fork) cudaEventDestroy(s->fork);
    if (s->join) cudaEventDestroy(s->join);
    for (dyc_table *t : s->tables)
        if (t) dyc_destroy(t);
    if (s->h_spare)
        for (uint32_t t = 0; t < s->ntables; ++t)
            if (s->h_spare[t].new_sub) cudaFree(s->h_spare[t].new_sub);
    for (const auto &b : s->free_later) cudaFree(b.first);
    for (const auto &b : s->spare_cache) cudaFree(b.second);
    if (s->d_spare) cudaFree(s->d_spare);
    if (s->h_spare) cudaFreeHost(s->h_spare);
    if (s->d_jobs) cudaFree(s->d_jobs);
    if (s->d_pout) cudaFree(s->d_pout);
    if (s->h_pout) cudaFreeHost(s->h_pout);
    if (s->d_grew) cudaFree(s->d_grew);
    if (s->h_grew) cudaFreeHost(s->h_grew);
    if (s->d_tctr) cudaFree(s->d_tctr);
    if (s->h_tctr) cudaFreeHost(s->h_tctr);
    if (s->d_desc) cudaFree(s->d_desc);
    if (s->h_desc) cudaFreeHost(s->h_desc);
    if (s->d_gctr) cudaFree(s->d_gctr);
    if (s->h_gctr) cudaFreeHost(s->h_gctr);
    if (s->h_actr) cudaFreeHost(s->h_actr);
    if (s->h_hostn) cudaFreeHost(s->h_hostn);
    if (s->h_tup) cudaFreeHost(s->h_tup);
    if (s->h_ter) cudaFreeHost(s->h_ter);
    if (s->abuf) cudaFree(s->abuf);
    if (s->lbuf) cudaFree(s->lbuf);
    if (s->d_bits_tmp) cudaFree(s->d_bits_tmp);
    delete s;
    return DYC_OK;
}

dyc_status dyc_set_configure(dyc_set *s, uint32_t blocks_per_sm, const uint32_t *max_evictions) {
    if (!s) return fail(DYC_EINVAL, "null set");
    if (blocks_per_sm > 64) return fail(DYC_EINVAL, "blocks_per_sm must be 0..64");
    if (max_evictions)
        for (uint32_t t = 0; t < s->ntables; ++t)
            if (max_evictions[t] < 1 || max_evictions[t] > 100000)
                return fail(DYC_EINVAL, "max_evictions[%u] must be 1..100000", t);
    set_drop_graphs(s);
    s->blocks_per_sm = blocks_per_sm;
    if (max_evictions) {
        s->max_evict_all = 0;
        for (uint32_t t = 0; t < s->ntables; ++t) {
            s->tables[t]->cfg.max_evictions = max_evictions[t];
            s->tables[t]->D.max_evict = max_evictions[t];
            s->max_evict_all = std::max(s->max_evict_all, max_evictions[t]);
        }
        TRY(set_push_descs(s, 0));
    }
    return DYC_OK;
}

dyc_status dyc_set_table(dyc_set *s, uint32_t i, dyc_table **out) {
    if (!s || !out || i >= s->ntables) return fail(DYC_EINVAL, "bad set or table index");
    *out = s->tables[i];
    return DYC_OK;
}

dyc_status dyc_set_sizes(dyc_set *s, uint64_t *h_sizes, uint64_t *h_capacities) {
    if (!s) return fail(DYC_EINVAL, "null set");
    for (uint32_t t = 0; t < s->ntables; ++t) {
        if (h_sizes) h_sizes[t] = s->tables[t]->size;
        if (h_capacities) h_capacities[t] = s->tables[t]->capacity;
    }
    return DYC_OK;
}

dyc_status dyc_set_spare_bytes(dyc_set *s, uint64_t *bytes) {
    if (!s || !bytes) return fail(DYC_EINVAL, "null argument");
    uint64_t b = s->free_later_bytes + s->spare_cache_bytes;
    if (s->h_spare)
        for (uint32_t t = 0; t < s->ntables; ++t)
            b += 2ull * s->h_spare[t].old_nb * (s->h_spare[t].new_sub ? (uint64_t)s->sb : 0ull);
    *bytes = b;
    return DYC_OK;
}

dyc_status dyc_set_spare_cache(dyc_set *s, uint64_t max_bytes) {
    if (!s) return fail(DYC_EINVAL, "null set");
    {
        int cur = -1;
        CK(cudaGetDevice(&cur));
        if (cur != s->device) CK(cudaSetDevice(s->device));
    }
    s->spare_cache_cap = max_bytes;
    while (s->spare_cache_bytes > max_bytes && !s->spare_cache.empty()) {
        auto it = std::prev(s->spare_cache.end());  // largest first
        CK(cudaFreeAsync(it->second, 0));
        s->spare_cache_bytes -= it->first;
        s->spare_cache.erase(it);
    }
    return DYC_OK;
}

dyc_status dyc_set_last_stats(dyc_set *s, dyc_op_stats *out) {
    if (!s || !out) return fail(DYC_EINVAL, "null argument");
    *out = s->last;
    return DYC_OK;
}

dyc_status dyc_set_apply(dyc_set *s, const uint32_t *d_offsets, const uint32_t *h_offsets,
                         const uint8_t *d_ops, const void *d_keys, const void *d_vals,
                         void *d_vals_out, uint32_t *d_bits_out, uint32_t flags, void *stream) {
    uint64_t n = 0;
    if (!set_args_ok(s, d_offsets, h_offsets, d_ops, d_keys, d_vals, &n)) return DYC_EINVAL;
    if (n == 0) return DYC_OK;
    // cells are indexed by 32 bits and a batch uses twice its ops of them
    if (n >= 0x80000000ull) return fail(DYC_EINVAL, "a set batch takes fewer than 2^31 ops");
    cudaStream_t st = (cudaStream_t)stream;
    {
        int cur = -1;
        CK(cudaGetDevice(&cur));
        if (cur != s->device) CK(cudaSetDevice(s->device));
    }
    s->last = dyc_op_stats{};
    for (dyc_table *m : s->tables) m->last = dyc_op_stats{};
    // entries a failed call left held by a member go back into it first
    for (dyc_table *m : s->tables)
        if (m->held_n) TRY(settle_held(m, st));
    // single-table calls on members since the last set call may have resized
    // them: the kernels must see the current subtables
    TRY(set_refresh_descs(s, st));
    TRY(set_ensure_scratch(s, n));
    *s->h_hostn = n;  // read by the copy at the start of phase A (the last call has synced)
    s->cur = dyc_set::Batch{d_offsets, d_ops, d_keys, d_vals, d_vals_out, d_bits_out};
    dyc_set::Graph *gr = nullptr;
    if (flags & DYC_FLAG_GRAPH)
        gr = set_graph_for(s, {(uintptr_t)d_offsets, (uintptr_t)d_ops, (uintptr_t)d_keys,
                              (uintptr_t)d_vals, (uintptr_t)d_vals_out, (uintptr_t)d_bits_out,
                              // the sequence differs with the resize policy (count copies)
                              (uintptr_t)(flags & DYC_FLAG_NO_RESIZE)});
    // under a graph the grids are sized by the scratch capacity, not by n
    const uint64_t ng = gr ? s->A.cap_ops : n;
    const bool resize = s->cfg.auto_resize && !(flags & DYC_FLAG_NO_RESIZE);
    // The upsize policy (hash_insert_batch, api.cpp:359-369, per table): while
    // size + the batch's inserts > upper bound x capacity, upsize, where the
    // inserts are the table's upserts after the batch is reduced per key and
    // the size is the one after the table's erases (as in dyc_apply), both
    // known on the device after phase A. Where even a batch of nothing but
    // new keys keeps every table within deferred_fill() of its slots, the
    // batch runs both phases back to back and the policy is applied after it
    // with the same sizes and counts, so capacities end as if it had run
    // before the inserts (entries a fuller table could not place go through
    // the overflow path). Otherwise the host reads the counts between the
    // phases and upsizes first. With upsize targets kept ahead (spares), the
    // policy runs on the device between the phases instead (k_set_policy),
    // with no host read unless a member needs a second upsize in the batch.
    bool deferred = true;
    if (resize && !s->spares)
        for (uint32_t t = 0; t < s->ntables && deferred; ++t) {
            const dyc_table *m = s->tables[t];
            const uint64_t cnt = h_offsets[t + 1] - h_offsets[t];
            deferred = (double)(m->size + cnt) <= deferred_fill(m) * (double)m->capacity;
        }
    bool moved = false;
    std::vector<uint8_t> grew;
    // The policy's upsizes go out in waves of at most one per table, each
    // wave one launch for all its tables (a round of many small tables
    // upsizes hundreds of them).
    auto upsize_policy = [&]() -> dyc_status {
        auto over = [&](uint32_t t) {
            const dyc_table *m = s->tables[t];
            // the size the inserts meet: the table's erases go first, as in dyc_apply
            const double base = (double)m->size - (double)s->h_ter[t];
            return s->h_tup[t] &&
                   base + (double)s->h_tup[t] > m->cfg.upper_load * (double)m->capacity;
        };
        std::vector<uint32_t> todo;
        for (uint32_t t = 0; t < s->ntables; ++t)
            if (over(t)) todo.push_back(t);
        std::vector<dyc::ResizeJob> jobs;
        std::vector<void *> olds;
        for (int wave = 0; !todo.empty() && wave < 64; ++wave) {
            jobs.clear();
            olds.clear();
            for (uint32_t t : todo) {
                dyc::ResizeJob j;
                void *old = nullptr;
                TRY(resize_up_prepare(s->tables[t], st, &j, &old));
                jobs.push_back(j);
                olds.push_back(old);
                if (grew.empty()) grew.assign(s->ntables, 0);
                grew[t] = 1;
            }
            moved = true;
            TRY(resize_up_flush(s->kb, s->sb, s->sms, st, jobs, olds));
            std::vector<uint32_t> next;
            for (uint32_t t : todo)
                if (over(t)) next.push_back(t);
            todo.swap(next);
        }
        return DYC_OK;
    };
    if (resize && s->spares) {
        // Phase A, then (while it runs) last round's replaced buffers freed and
        // spares made to fit; then the device policy, its upsizes and phase B
        // in one sequence. The host reads the counts between the phases only
        // when a member needs more than its device upsize.
        TRY(set_run(s, gr, 0, st, [&](cudaStream_t cs) {
            return set_phase_a(s, d_offsets, d_ops, d_keys, d_vals, d_vals_out, d_bits_out, ng,
                               true, cs);
        }));
        TRY(set_release_later(s, st));
        set_fill_spares(s, st);
        TRY(set_run(s, gr, 3, st, [&](cudaStream_t cs) { return set_policy_and_b(s, ng, cs); }));
        CK(cudaStreamSynchronize(st));
        set_take_device_upsizes(s, grew);
        if (s->h_pout->host) {
            s->last.split_phases = 1;
            TRY(upsize_policy());
            TRY(set_push_descs(s, st));
            CK(cudaMemsetAsync(&s->d_pout->host, 0, sizeof(uint32_t), st));
            TRY(set_run(s, gr, 1, st, [&](cudaStream_t cs) { return set_phase_b(s, ng, cs); }));
            CK(cudaStreamSynchronize(st));
        }
    } else if (deferred) {
        TRY(set_run(s, gr, 2, st, [&](cudaStream_t cs) {
            TRY(set_phase_a(s, d_offsets, d_ops, d_keys, d_vals, d_vals_out, d_bits_out, ng,
                            resize, cs));
            return set_phase_b(s, ng, cs);
        }));
        CK(cudaStreamSynchronize(st));
        if (resize) TRY(upsize_policy());  // m->size is still the size before the batch
    } else {
        s->last.split_phases = 1;
        TRY(set_run(s, gr, 0, st, [&](cudaStream_t cs) {
            return set_phase_a(s, d_offsets, d_ops, d_keys, d_vals, d_vals_out, d_bits_out, ng,
                               true, cs);
        }));
        CK(cudaStreamSynchronize(st));
        TRY(upsize_policy());
        if (moved) TRY(set_push_descs(s, st));
        TRY(set_run(s, gr, 1, st, [&](cudaStream_t cs) { return set_phase_b(s, ng, cs); }));
        CK(cudaStreamSynchronize(st));
    }
    if (gr) gr->warm = true;
    // Device offsets that disagree with h_offsets: the kernels clamped them
    // and the batch ran; the bookkeeping below still follows the device's
    // counters, and the call reports the disagreement at the end.
    const unsigned long long bad_offsets = s->h_actr[dyc::kCtrBadOffsets];
    if (s->h_actr[dyc::kCtrBad])
        return fail(DYC_ECUDA, "set batch: %llu device counts or ids out of range",
                    s->h_actr[dyc::kCtrBad]);
    const Counters g = *s->h_gctr;
    if (g.spill) return fail(DYC_EOVERFLOW, "internal list overflow (%llu entries)", g.spill);
    for (uint32_t t = 0; t < s->ntables; ++t) s->tables[t]->size = s->h_tctr[t].size;
    s->last.inserted = g.inserted;
    s->last.updated = g.updated;
    s->last.erased = g.erased;
    s->last.evict_steps = g.evict_steps;
    s->last.overflowed = g.overflow;
    for (dyc_table *m : s->tables) {
        s->last.resizes_up += m->last.resizes_up;
        m->last = dyc_op_stats{};
    }
    if (g.overflow) {
        TRY(set_overflow(s, g.overflow, grew, st));
        moved = true;
    }
    // downsize after the batch (hash_delete_batch, api.cpp:494-505, per table)
    if (s->cfg.auto_resize && !(flags & DYC_FLAG_NO_RESIZE)) {
        for (dyc_table *m : s->tables) {
            if ((double)m->size < m->cfg.lower_load * (double)m->capacity &&
                m->capacity > m->cfg.min_downsize_capacity) {
                dyc_status r = resize_down_impl(m, st);
                if (r != DYC_OK && r != DYC_EINVAL) return r;
                moved = true;
                s->last.resizes_down += m->last.resizes_down;
                s->last.resizes_up += m->last.resizes_up;
                m->last = dyc_op_stats{};
            }
        }
    }
    if (moved) TRY(set_push_descs(s, st));
    if (bad_offsets)
        return fail(DYC_EINVAL, "device offsets disagree with h_offsets (%llu reports)",
                    bad_offsets);
    return DYC_OK;
}

dyc_status dyc_set_apply_each(dyc_set *s, const uint32_t *d_offsets, const uint32_t *h_offsets,
                              const uint8_t *d_ops, const void *d_keys, const void *d_vals,
                              void *d_vals_out, uint32_t *d_bits_out, uint32_t flags,
                              void *stream) {
    uint64_t n = 0;
    if (!set_args_ok(s, d_offsets, h_offsets, d_ops, d_keys, d_vals, &n)) return DYC_EINVAL;
    if (n == 0) return DYC_OK;
    cudaStream_t st = (cudaStream_t)stream;
    s->last = dyc_op_stats{};
    uint64_t maxm = 0;
    for (uint32_t t = 0; t < s->ntables; ++t)
        maxm = std::max<uint64_t>(maxm, h_offsets[t + 1] - h_offsets[t]);
    if (d_bits_out) {
        const size_t words = (size_t)(maxm / 32 + 1);
        if (s->bits_tmp_words < words) {
            if (s->d_bits_tmp) CK(cudaFree(s->d_bits_tmp));
            s->d_bits_tmp = nullptr;
            CK(dyc::lib_malloc(&s->d_bits_tmp, words * 4));
            s->bits_tmp_words = words;
        }
        CK(cudaMemsetAsync(d_bits_out, 0, (size_t)((n + 31) / 32) * 4, st));
    }
    for (uint32_t t = 0; t < s->ntables; ++t) {
        const uint64_t o = h_offsets[t], m = h_offsets[t + 1] - o;
        if (!m) continue;
        dyc_table *tb = s->tables[t];
        TRY(dyc_apply(tb, d_ops + o, (const char *)d_keys + o * s->kb,
                      (const char *)d_vals + o * s->vb,
                      m, d_vals_out ? (char *)d_vals_out + o * s->vb : nullptr,
                      d_bits_out ? s->d_bits_tmp : nullptr, flags, st));
        if (d_bits_out) {
            k_bits_merge<<<(unsigned)std::min<uint64_t>((m + 255) / 256, 1024), 256, 0, st>>>(
                d_bits_out, o, s->d_bits_tmp, m);
            CK(cudaGetLastError());
        }
        const dyc_op_stats &l = tb->last;
        s->last.inserted += l.inserted;
        s->last.updated += l.updated;
        s->last.erased += l.erased;
        s->last.evict_steps += l.evict_steps;
        s->last.overflowed += l.overflowed;
        s->last.resizes_up += l.resizes_up;
        s->last.resizes_down += l.resizes_down;
    }
    CK(cudaStreamSynchronize(st));
    return set_push_descs(s, st);
}

}  // extern "C"

// =============================================================================
// Snapshot / restore (include/dycuckoo.h dyc_snapshot*, dyc_restore).
// =============================================================================
static_assert(sizeof(dyc_snapshot_header) == 256, "snapshot header is 256 bytes");

namespace {

constexpr uint64_t kSnapGold = 0x9E3779B97F4A7C15ull;

__device__ __forceinline__ uint64_t snap_mix(uint64_t x) {
    x += kSnapGold;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// sum of snap_mix(w[i] ^ (base + i) * gold) into *sum (mod 2^64, so the
// order of the additions does not matter)
__global__ void __launch_bounds__(256) k_snapshot_sum(const uint64_t *__restrict__ w, uint64_t n,
                                                      uint64_t base,
                                                      unsigned long long *__restrict__ sum) {
    uint64_t acc = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        acc += snap_mix(w[i] ^ ((base + i) * kSnapGold));
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(sum, (unsigned long long)acc);
}

// Checksum of the table's subtables, in subtable order, on `s`.
dyc_status table_checksum(dyc_table *t, cudaStream_t s, uint64_t *out) {
    unsigned long long *d = &t->d_ctr->pad[1];
    CK(cudaMemsetAsync(d, 0, sizeof(unsigned long long), s));
    uint64_t base = 0;
    for (uint32_t i = 0; i < t->D.d; ++i) {
        const uint64_t words = (uint64_t)t->D.nb[i] * t->sb / 8;
        const unsigned blocks = (unsigned)std::min<uint64_t>((words + 255) / 256, (uint64_t)t->sms * 8);
        k_snapshot_sum<<<blocks, 256, 0, s>>>((const uint64_t *)t->D.sub[i], words, base, d);
        CK(cudaGetLastError());
        base += words;
    }
    unsigned long long h = 0;
    CK(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    *out = h;
    return DYC_OK;
}

uint64_t snapshot_payload(const dyc_table *t) {
    uint64_t p = 0;
    for (uint32_t i = 0; i < t->D.d; ++i) p += (uint64_t)t->D.nb[i] * t->sb;
    return p;
}

}  // namespace

extern "C" {

dyc_status dyc_snapshot_bytes(dyc_table *t, uint64_t *bytes) {
    if (!t || !bytes) return fail(DYC_EINVAL, "null argument");
    if (t->held_n) {  // held entries are placed first: the layout may grow
        TRY(set_device(t));
        TRY(settle_held(t, 0));
    }
    *bytes = sizeof(dyc_snapshot_header) + snapshot_payload(t);
    return DYC_OK;
}

dyc_status dyc_snapshot(dyc_table *t, void *h_buf, uint64_t buf_bytes, void *stream) {
    if (!t || !h_buf) return fail(DYC_EINVAL, "null argument");
    if (t->held_n) {  // placed first (may upsize: the size check below then sees it)
        TRY(set_device(t));
        TRY(settle_held(t, (cudaStream_t)stream));
    }
    const uint64_t payload = snapshot_payload(t);
    if (buf_bytes < sizeof(dyc_snapshot_header) + payload)
        return fail(DYC_EINVAL, "snapshot buffer of %llu bytes, need %llu",
                    (unsigned long long)buf_bytes,
                    (unsigned long long)(sizeof(dyc_snapshot_header) + payload));
    TRY(set_device(t));
    cudaStream_t s = (cudaStream_t)stream;
    dyc_snapshot_header h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, "DYCSNAP1", 8);
    h.version = 2;
    h.header_bytes = sizeof(h);
    h.key_bytes = t->cfg.key_bytes;
    h.value_bytes = t->cfg.value_bytes;
    h.bucket_bytes = t->cfg.bucket_bytes;
    h.num_subtables = t->D.d;
    h.max_evictions = t->cfg.max_evictions;
    h.auto_resize = t->cfg.auto_resize;
    h.size = t->size;
    h.capacity = t->capacity;
    h.upper_load = t->cfg.upper_load;
    h.lower_load = t->cfg.lower_load;
    h.min_downsize_capacity = t->cfg.min_downsize_capacity;
    h.initial_size = t->cfg.initial_size;
    for (uint32_t i = 0; i < t->D.d; ++i) h.nbuckets[i] = t->D.nb[i];
    h.payload_bytes = payload;
    TRY(table_checksum(t, s, &h.checksum));
    char *dst = (char *)h_buf + sizeof(h);
    for (uint32_t i = 0; i < t->D.d; ++i) {
        const uint64_t b = (uint64_t)t->D.nb[i] * t->sb;
        CK(cudaMemcpyAsync(dst, t->D.sub[i], b, cudaMemcpyDeviceToHost, s));
        dst += b;
    }
    CK(cudaStreamSynchronize(s));
    memcpy(h_buf, &h, sizeof(h));
    return DYC_OK;
}

dyc_status dyc_restore(const void *h_buf, uint64_t buf_bytes, int32_t device, dyc_table **out) {
    if (!h_buf || !out) return fail(DYC_EINVAL, "null argument");
    *out = nullptr;
    dyc_snapshot_header h;
    if (buf_bytes < sizeof(h)) return fail(DYC_EINVAL, "snapshot shorter than its header");
    memcpy(&h, h_buf, sizeof(h));
    if (memcmp(h.magic, "DYCSNAP1", 8) != 0 || h.version != 2 || h.header_bytes != sizeof(h))
        return fail(DYC_EINVAL, "not a version-2 DyCuckoo snapshot");
    dyc_config c;
    dyc_config_default(&c);
    c.key_bytes = h.key_bytes;
    c.value_bytes = h.value_bytes;
    c.bucket_bytes = h.bucket_bytes;
    c.num_subtables = h.num_subtables;
    c.max_evictions = h.max_evictions;
    c.auto_resize = h.auto_resize;
    c.upper_load = h.upper_load;
    c.lower_load = h.lower_load;
    c.min_downsize_capacity = h.min_downsize_capacity;
    c.initial_size = h.initial_size;
    c.device = device;
    char why[128];
    if (!valid_config(&c, why, sizeof(why))) return fail(DYC_EINVAL, "snapshot header: %s", why);
    uint64_t payload = 0, slots = 0;
    const uint64_t per_bucket = c.bucket_bytes / (c.key_bytes == 4 ? 8 : 16) -
                                (c.bucket_bytes == 128 ? 1 : 0);
    for (uint32_t i = 0; i < c.num_subtables; ++i) {
        if (h.nbuckets[i] == 0) return fail(DYC_EINVAL, "snapshot header: empty subtable %u", i);
        payload += (uint64_t)h.nbuckets[i] * c.bucket_bytes;
        slots += (uint64_t)h.nbuckets[i] * per_bucket;
    }
    if (payload != h.payload_bytes || slots != h.capacity || h.size > slots)
        return fail(DYC_EINVAL, "snapshot header: inconsistent sizes");
    if (buf_bytes < sizeof(h) + payload) return fail(DYC_EINVAL, "snapshot payload is truncated");
    dyc_table *t = nullptr;
    TRY(create_impl(&c, nullptr, nullptr, true, &t, h.nbuckets));
    auto undo = [&](dyc_status r) {
        dyc_destroy(t);
        return r;
    };
    const char *src = (const char *)h_buf + sizeof(h);
    for (uint32_t i = 0; i < t->D.d; ++i) {
        const uint64_t b = (uint64_t)t->D.nb[i] * t->sb;
        cudaError_t e = cudaMemcpy(t->D.sub[i], src, b, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return undo(fail(DYC_ECUDA, "restore copy: %s", cudaGetErrorString(e)));
        src += b;
    }
    uint64_t sum = 0;
    dyc_status r = table_checksum(t, 0, &sum);
    if (r != DYC_OK) return undo(r);
    if (sum != h.checksum) return undo(fail(DYC_EINVAL, "snapshot checksum mismatch"));
    t->size = h.size;
    cudaError_t e = cudaMemcpy(&t->d_ctr->size, &h.size, sizeof(h.size), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return undo(fail(DYC_ECUDA, "restore size: %s", cudaGetErrorString(e)));
    *out = t;
    return DYC_OK;
}

}  // extern "C"

// =============================================================================
// Wide-value tables (include/dycuckoo.h dyc_wide_*): an ordinary table maps
// keys to 32-bit handles, values live in a device heap of fixed-size rows.
// =============================================================================
#include "dyc_wide.cuh"

using dyc::WideAlloc;

struct dyc_wide {
    dyc_table *t = nullptr;  // key -> handle
    uint32_t vbytes = 0, words = 0;
    uint32_t *heap = nullptr, *stack = nullptr;
    WideAlloc *d_alloc = nullptr, *h_alloc = nullptr;
    uint64_t cap = 0, bump = 0, free_top = 0;  // host mirror of the allocator
    void *scr = nullptr;
    size_t scr_bytes = 0;
    uint64_t scr_n = 0;
    uint32_t *pre_h = nullptr, *bits = nullptr, *new_h = nullptr;
    void *new_keys = nullptr;
    unsigned long long *cnt = nullptr;    // [0] new keys, [1] updates (device)
    unsigned long long *h_cnt = nullptr;  // pinned copy
    uint32_t *h_cap = nullptr;            // pinned staging of the heap size
    dyc_op_stats last{};
};

namespace {

dyc_status wide_ensure_scratch(dyc_wide *w, uint64_t n) {
    if (w->scr && w->scr_n >= n) return DYC_OK;
    const uint64_t m = std::max<uint64_t>(n, 1024);
    auto al = [](uint64_t x) { return (x + 255) & ~(uint64_t)255; };
    const uint64_t need = al(m * 4) * 2 + al((m / 32 + 1) * 4) + al(m * w->t->kb) + 256;
    if (w->scr) {
        CK(cudaDeviceSynchronize());
        CK(cudaFree(w->scr));
        w->scr = nullptr;
    }
    CK(dyc::lib_malloc(&w->scr, need));
    char *p = (char *)w->scr;
    w->pre_h = (uint32_t *)p;
    p += al(m * 4);
    w->new_h = (uint32_t *)p;
    p += al(m * 4);
    w->bits = (uint32_t *)p;
    p += al((m / 32 + 1) * 4);
    w->new_keys = p;
    p += al(m * w->t->kb);
    w->cnt = (unsigned long long *)p;
    w->scr_bytes = need;
    w->scr_n = m;
    return DYC_OK;
}

// Room for n more handles: grow heap and free stack (stream-ordered).
dyc_status wide_ensure_heap(dyc_wide *w, uint64_t n, cudaStream_t s) {
    const uint64_t avail = w->cap - w->bump + w->free_top;
    if (avail >= n) return DYC_OK;
    uint64_t nc = std::max<uint64_t>(w->cap * 2, w->cap + (n - avail));
    if (nc > 0xFFFFFFFFull) nc = 0xFFFFFFFFull;
    if (nc - w->bump + w->free_top < n) return fail(DYC_ENOMEM, "wide table: more than 2^32 values");
    uint32_t *heap = nullptr, *stack = nullptr;
    CK(pool_alloc(w->t->device, (void **)&heap, nc * w->vbytes, s));
    CK(pool_alloc(w->t->device, (void **)&stack, nc * 4, s));
    if (w->heap) {
        if (w->bump)
            CK(cudaMemcpyAsync(heap, w->heap, w->bump * w->vbytes, cudaMemcpyDeviceToDevice, s));
        if (w->free_top)
            CK(cudaMemcpyAsync(stack, w->stack, w->free_top * 4, cudaMemcpyDeviceToDevice, s));
        CK(cudaFreeAsync(w->heap, s));
        CK(cudaFreeAsync(w->stack, s));
    }
    w->heap = heap;
    w->stack = stack;
    w->cap = nc;
    *w->h_cap = (uint32_t)nc;
    CK(cudaMemcpyAsync(&w->d_alloc->cap, w->h_cap, 4, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));  // the pinned staging word is reused by the next growth
    return DYC_OK;
}

dyc_status wide_read_alloc(dyc_wide *w, cudaStream_t s) {
    CK(cudaMemcpyAsync(w->h_alloc, w->d_alloc, sizeof(WideAlloc), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    w->bump = w->h_alloc->bump;
    w->free_top = w->h_alloc->free_top;
    return DYC_OK;
}

unsigned wide_grid(dyc_wide *w, uint64_t n) {
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, (uint64_t)w->t->sms * 8));
}

}  // namespace

extern "C" {

dyc_status dyc_wide_create(const dyc_config *cfg, uint32_t value_bytes, dyc_wide **out) {
    if (!cfg || !out) return fail(DYC_EINVAL, "null argument");
    *out = nullptr;
    if (value_bytes == 0 || value_bytes % 4 || value_bytes > 65536)
        return fail(DYC_EINVAL, "wide values are 4..65536 bytes, a multiple of 4");
    dyc_config c = *cfg;
    c.value_bytes = 4;  // the table stores handles
    dyc_wide *w = new (std::nothrow) dyc_wide();
    if (!w) return fail(DYC_ENOMEM, "host allocation");
    w->vbytes = value_bytes;
    w->words = value_bytes / 4;
    dyc_status r = create_impl(&c, nullptr, nullptr, true, &w->t);
    if (r != DYC_OK) {
        delete w;
        return r;
    }
    cudaError_t e = dyc::lib_malloc(&w->d_alloc, sizeof(WideAlloc));
    if (e == cudaSuccess) e = cudaMemset(w->d_alloc, 0, sizeof(WideAlloc));
    if (e == cudaSuccess) e = dyc::lib_malloc_host(&w->h_alloc, sizeof(WideAlloc));
    if (e == cudaSuccess) e = dyc::lib_malloc_host(&w->h_cnt, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = dyc::lib_malloc_host(&w->h_cap, sizeof(uint32_t));
    if (e != cudaSuccess) {
        dyc_wide_destroy(w);
        return fail(DYC_ENOMEM, "wide table setup: %s", cudaGetErrorString(e));
    }
    r = wide_ensure_heap(w, std::max<uint64_t>(1024, std::min<uint64_t>(cfg->initial_size, 1ull << 30)), 0);
    if (r != DYC_OK) {
        dyc_wide_destroy(w);
        return r;
    }
    *out = w;
    return DYC_OK;
}

dyc_status dyc_wide_destroy(dyc_wide *w) {
    if (!w) return DYC_OK;
    if (w->t) {
        cudaSetDevice(w->t->device);
        cudaDeviceSynchronize();
    }
    if (w->heap) cudaFree(w->heap);
    if (w->stack) cudaFree(w->stack);
    if (w->d_alloc) cudaFree(w->d_alloc);
    if (w->h_alloc) cudaFreeHost(w->h_alloc);
    if (w->h_cnt) cudaFreeHost(w->h_cnt);
    if (w->h_cap) cudaFreeHost(w->h_cap);
    if (w->scr) cudaFree(w->scr);
    if (w->t) dyc_destroy(w->t);
    delete w;
    return DYC_OK;
}

dyc_status dyc_wide_table(dyc_wide *w, dyc_table **out) {
    if (!w || !out) return fail(DYC_EINVAL, "null argument");
    *out = w->t;
    return DYC_OK;
}

dyc_status dyc_wide_last_stats(dyc_wide *w, dyc_op_stats *out) {
    if (!w || !out) return fail(DYC_EINVAL, "null argument");
    *out = w->last;
    return DYC_OK;
}

dyc_status dyc_wide_insert(dyc_wide *w, const void *d_keys, const void *d_vals, uint64_t n,
                           uint32_t flags, void *stream) {
    if (!w) return fail(DYC_EINVAL, "null table");
    if (n == 0) return DYC_OK;
    if (!d_keys || !d_vals) return fail(DYC_EINVAL, "null key or value array");
    dyc_table *t = w->t;
    TRY(set_device(t));
    cudaStream_t s = (cudaStream_t)stream;
    w->last = dyc_op_stats{};
    if (t->held_n) TRY(settle_held(t, s));
    if (t->held_n) TRY(settle_held(t, s));  // (key, handle) slots a failed call held
    const uint64_t chunk = t->chunk;
    const uint64_t m0 = std::min(n, chunk);
    TRY(ensure_scratch(t, m0));
    TRY(wide_ensure_scratch(w, m0));
    for (uint64_t off = 0; off < n; off += chunk) {
        const uint64_t m = std::min(chunk, n - off);
        const char *k = (const char *)d_keys + off * t->kb;
        const uint32_t *v = (const uint32_t *)((const char *)d_vals + off * w->vbytes);
        // current handles of the chunk's keys
        cudaError_t e = KB_CALL(t, find, ctx(t, s), t->D, t->sb, k, w->pre_h, 4u, w->bits, m);
        if (e != cudaSuccess) return fail(DYC_ECUDA, "wide find: %s", cudaGetErrorString(e));
        const bool use_dedup = !(flags & DYC_FLAG_UNIQUE) && m > 1;
        const Scratch S = chunk_scratch(t, m);
        if (use_dedup) {  // clears the chunk's cells first
            e = KB_CALL(t, dedup, ctx(t, s), S, k, m, dyc::kKeepLast);
            if (e != cudaSuccess) return fail(DYC_ECUDA, "dedup kernel: %s", cudaGetErrorString(e));
        }
        TRY(wide_ensure_heap(w, m, s));
        CK(cudaMemsetAsync(w->cnt, 0, 2 * sizeof(unsigned long long), s));
        const unsigned grid = wide_grid(w, m);
        if (t->kb == 4)
            dyc::k_wide_stage<4><<<grid, 256, 0, s>>>(S, use_dedup ? 1 : 0, k, v, w->words, m,
                                                      w->pre_h, w->bits, w->heap, w->stack,
                                                      w->d_alloc, w->new_keys, w->new_h, w->cnt,
                                                      w->cnt + 1);
        else
            dyc::k_wide_stage<8><<<grid, 256, 0, s>>>(S, use_dedup ? 1 : 0, k, v, w->words, m,
                                                      w->pre_h, w->bits, w->heap, w->stack,
                                                      w->d_alloc, w->new_keys, w->new_h, w->cnt,
                                                      w->cnt + 1);
        dyc::k_wide_commit<<<1, 1, 0, s>>>(w->d_alloc);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(w->h_cnt, w->cnt, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        TRY(wide_read_alloc(w, s));
        const uint64_t fresh = w->h_cnt[0];
        w->last.updated += w->h_cnt[1];
        if (fresh) {
            if (t->cfg.auto_resize && !(flags & DYC_FLAG_NO_RESIZE)) {
                int guard = 0;
                while ((double)(t->size + fresh) > t->cfg.upper_load * (double)t->capacity &&
                       guard++ < 64)
                    TRY(resize_up_impl(t, s));
            }
            t->last = dyc_op_stats{};
            TRY(insert_chunk(t, w->new_keys, w->new_h, fresh, DYC_FLAG_UNIQUE | DYC_FLAG_NEW_KEYS, s));
            w->last.inserted += t->last.inserted;
            w->last.evict_steps += t->last.evict_steps;
            w->last.overflowed += t->last.overflowed;
            w->last.resizes_up += t->last.resizes_up;
        }
    }
    return DYC_OK;
}

dyc_status dyc_wide_find(dyc_wide *w, const void *d_keys, void *d_vals_out, uint32_t *d_hit_bits,
                         uint64_t n, void *stream) {
    if (!w) return fail(DYC_EINVAL, "null table");
    if (n == 0) return DYC_OK;
    if (!d_keys || !d_vals_out) return fail(DYC_EINVAL, "null key or value array");
    dyc_table *t = w->t;
    TRY(set_device(t));
    cudaStream_t s = (cudaStream_t)stream;
    if (t->held_n) TRY(settle_held(t, s));
    const uint64_t chunk = t->chunk;
    TRY(wide_ensure_scratch(w, std::min(n, chunk)));
    for (uint64_t off = 0; off < n; off += chunk) {
        const uint64_t m = std::min(chunk, n - off);
        uint32_t *bits = d_hit_bits ? d_hit_bits + off / 32 : w->bits;
        cudaError_t e = KB_CALL(t, find, ctx(t, s), t->D, t->sb, (const char *)d_keys + off * t->kb,
                                w->pre_h, 4u, bits, m);
        if (e != cudaSuccess) return fail(DYC_ECUDA, "wide find: %s", cudaGetErrorString(e));
        dyc::k_wide_gather<<<wide_grid(w, m), 256, 0, s>>>(
            w->pre_h, bits, m, w->heap, w->words,
            (uint32_t *)((char *)d_vals_out + off * w->vbytes));
        CK(cudaGetLastError());
    }
    return DYC_OK;
}

dyc_status dyc_wide_erase(dyc_wide *w, const void *d_keys, uint64_t n, void *d_vals_out,
                          uint32_t *d_erased_bits, uint64_t *h_erased_count, uint32_t flags,
                          void *stream) {
    if (!w) return fail(DYC_EINVAL, "null table");
    if (h_erased_count) *h_erased_count = 0;
    if (n == 0) return DYC_OK;
    if (!d_keys) return fail(DYC_EINVAL, "null key array");
    dyc_table *t = w->t;
    TRY(set_device(t));
    cudaStream_t s = (cudaStream_t)stream;
    w->last = dyc_op_stats{};
    const uint64_t chunk = t->chunk;
    TRY(wide_ensure_scratch(w, std::min(n, chunk)));
    uint64_t total = 0;
    for (uint64_t off = 0; off < n; off += chunk) {
        const uint64_t m = std::min(chunk, n - off);
        const char *k = (const char *)d_keys + off * t->kb;
        // handles before the erase
        cudaError_t e = KB_CALL(t, find, ctx(t, s), t->D, t->sb, k, w->pre_h, 4u, w->bits, m);
        if (e != cudaSuccess) return fail(DYC_ECUDA, "wide find: %s", cudaGetErrorString(e));
        uint32_t *eb = d_erased_bits ? d_erased_bits + off / 32 : w->bits;
        uint64_t cnt = 0;
        // no downsize inside: the erased bits and handles are read below
        TRY(dyc_erase(t, k, m, eb, &cnt, flags | DYC_FLAG_NO_RESIZE, s));
        total += cnt;
        dyc::k_wide_free<<<wide_grid(w, m), 256, 0, s>>>(
            w->pre_h, eb, m, w->heap, w->words,
            d_vals_out ? (uint32_t *)((char *)d_vals_out + off * w->vbytes) : nullptr, w->stack,
            w->d_alloc);
        dyc::k_wide_commit_free<<<1, 1, 0, s>>>(w->d_alloc);
        CK(cudaGetLastError());
        TRY(wide_read_alloc(w, s));
    }
    w->last.erased = total;
    if (h_erased_count) *h_erased_count = total;
    // downsize after the batch (api.cpp:494-505); handles move with their keys
    if (t->cfg.auto_resize && !(flags & DYC_FLAG_NO_RESIZE) &&
        (double)t->size < t->cfg.lower_load * (double)t->capacity &&
        t->capacity > t->cfg.min_downsize_capacity) {
        t->last = dyc_op_stats{};
        dyc_status st = resize_down_impl(t, s);
        if (st != DYC_OK && st != DYC_EINVAL) return st;
        w->last.resizes_down += t->last.resizes_down;
        w->last.resizes_up += t->last.resizes_up;
    }
    return DYC_OK;
}

dyc_status dyc_wide_export(dyc_wide *w, void *d_keys_out, void *d_vals_out, uint64_t capacity,
                           uint64_t *n_out, void *stream) {
    if (!w) return fail(DYC_EINVAL, "null table");
    dyc_table *t = w->t;
    cudaStream_t s = (cudaStream_t)stream;
    TRY(set_device(t));
    TRY(wide_ensure_scratch(w, std::max<uint64_t>(capacity, 1)));
    uint64_t got = 0;
    TRY(dyc_export(t, d_keys_out, w->pre_h, capacity, &got, stream));
    if (n_out) *n_out = got;
    const uint64_t m = std::min(got, capacity);
    if (m && d_vals_out) {
        dyc::k_wide_gather<<<wide_grid(w, m), 256, 0, s>>>(w->pre_h, nullptr, m, w->heap, w->words,
                                                           (uint32_t *)d_vals_out);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(s));
    }
    return DYC_OK;
}

}  // extern "C"
