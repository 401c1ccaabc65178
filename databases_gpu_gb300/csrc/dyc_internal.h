// dyc_internal.h -- shared between the kernels and the host side of the
// C ABI: the device-side table descriptor, the per-table counters and the
// kernel launchers.
#pragma once

#include <atomic>
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace dyc {

// Every device and pinned-host allocation the library makes goes through
// these (counted for dyc_debug_alloc_count).
extern std::atomic<unsigned long long> g_lib_allocs;
template <class T> cudaError_t lib_malloc(T **p, size_t bytes) {
    g_lib_allocs.fetch_add(1, std::memory_order_relaxed);
    return cudaMalloc((void **)p, bytes);
}
template <class T> cudaError_t lib_malloc_host(T **p, size_t bytes) {
    g_lib_allocs.fetch_add(1, std::memory_order_relaxed);
    return cudaMallocHost((void **)p, bytes);
}

// The reference's modulus before the bucket modulo, written as in
// GPU/dyhash/dy_hash.h:24 (294967291, not the prime 4294967291).
constexpr uint32_t kPrime = 294967291u;
constexpr int kMaxSub = 6;
// Polls of a bounded device wait (mbarrier try_wait): far beyond any copy's
// completion; a wait that runs out records a timeout instead of hanging.
constexpr uint32_t kWaitTries = 1u << 22;

// Table descriptor passed by value to every kernel (the reference keeps one
// in __constant__ memory, cuckoo.cu:16, which limits a process to one table).
struct Desc {
    void *sub[kMaxSub];       // subtable base addresses
    uint64_t magic[kMaxSub];  // fastmod reciprocals of nb[]
    uint32_t nb[kMaxSub];     // buckets per subtable
    uint32_t d;               // subtable count
    uint32_t max_evict;       // eviction bound of this table (read by the set kernels)
    uint32_t l2_keep;         // 1: the table fits the L2; its bucket reads ask to stay there
    uint32_t pad;
};

// Per-table device counters (one 128-byte block). `size` persists; the rest
// are per-call and reset before each insert / erase / resize.
struct Counters {
    unsigned long long size;
    unsigned long long inserted, updated, erased, rejected, superseded;
    unsigned long long pending, overflow, evict_steps;
    unsigned long long spill;  // pending entries a list could not hold (must stay 0)
    unsigned long long pad[2];      // scratch words of dyc_export and dyc_snapshot
    unsigned long long timeouts;    // bounded device waits that gave up (must stay 0)
    unsigned long long nins;        // scratch word: insert ops of a dyc_apply batch
    unsigned long long pad2[2];
};
static_assert(sizeof(Counters) == 128, "Counters is one 128-byte block");

enum DedupMode { kKeepLast = 0, kKeepFirst = 1 };

// Scratch lists used by one insert / erase / resize chunk.
struct Scratch {
    void *dedup;            // open-addressing table of (key, op index)
    uint32_t *dedup_idx;    // op index array for 8-byte keys
    uint64_t dedup_cap;     // power of two
    void *list_a;           // pending entries (slots)
    void *list_b;           // overflow entries (slots)
    uint64_t list_cap;      // entries per list
    // one bit per op of the chunk, set for the op its key's dedup cell names
    // (filled from the dedup table after the claims); null: the winner is
    // looked up in the dedup table by each op
    uint32_t *winbits;
    // nonzero once the dedup claims met a key twice; while it stays zero
    // every op of the chunk is its key's only op (no winner bits are needed)
    uint32_t *dupseen;
};

// Dedup tables of at least this many cells get the winners pass (winbits);
// smaller ones fit in the L2 beside the bucket lines, so an op of a chunk
// with repeats looks its winner up in the table instead, and the pass's
// launch is saved.
constexpr uint64_t kWinnersMinCap = 1ull << 22;
__host__ __device__ inline bool winners_pass(const Scratch &S) {
    return S.winbits != nullptr && S.dedup_cap >= kWinnersMinCap;
}

// Scratch of one mixed batch of at most `cap_ops` ops. The multi-table
// fields are null for a single table.
struct ApplyScratch {
    // cap_cells cells: 4-byte keys {key, count} in 8 bytes, 8-byte keys
    // {key, count, pad} in 16; key 0 = free. After compaction the count field
    // holds the cell's distinct-key id.
    void *cells;
    uint32_t *op_cell;         // cell of each op
    uint32_t *op_rank;         // place of each op inside its key's segment
    void *dkey;                // distinct keys
    uint32_t *dcnt;            // per distinct key: ops
    unsigned long long *dseg;  // per distinct key: segment start << 32
    uint32_t *seg;             // op indices grouped by key
    void *pre_val;             // pre-batch value per distinct key
    uint32_t *pre_hit;         // pre-batch hit bits per distinct key
    void *up_key, *up_val;     // upserts to apply
    void *er_key;              // erases to apply
    unsigned long long *ctr;   // see kCtr*
    uint32_t *wseg;            // distinct ids of segments replayed by a warp
    uint32_t *mid;             // distinct ids of segments replayed by a block
    uint32_t *sort_tmp;        // merge scratch of long segments (same offsets as seg)
    uint64_t cap_cells;        // >= 2 * cap_ops
    uint64_t cap_ops;
    // multi-table batches
    uint32_t *dtid;            // table of a distinct key
    uint32_t *up_tid, *er_tid; // table of each upsert / erase
    uint32_t *tup;             // per table: upserts listed (the upsize policy's insert batch)
    uint32_t *ter;             // per table: erases listed (keys present before the batch)
    uint32_t *tcell_off;       // per table: first cell of its region (ntables + 1)
    uint32_t *tidx;            // table of every kTidxStep-th op (cap_ops / kTidxStep + 1)
    uint32_t ntables;
    // one table's batch (null: none): k_apply_group sets *gate once it meets
    // a key twice; compaction and the scatter pass run only when it did.
    unsigned long long *gate;
    // nonzero: keys with a single op in the batch, and key-0 ops, are left
    // to the one-pass kernel (k_apply_unique with op_cell / cells), which
    // runs after the replays. Compaction lists only keys with several ops,
    // so the find of the distinct keys, the scatter, the replays and the
    // mutation see those alone.
    uint32_t single_pass;
    // single_pass batches: bit i set when op i is left to the one-pass
    // kernel (written by the scatter, one word per warp, cap_ops / 32 + 1)
    uint32_t *single;
};

// Cell words after compaction: kIdBit | distinct id. A word without the bit
// in a single_pass batch is a count of 1 (a key compaction left alone).
constexpr uint32_t kIdBit = 0x80000000u;

constexpr uint32_t kTidxStep = 64;  // ops per entry of ApplyScratch::tidx

// ApplyScratch::ctr slots. Every count and id the batch kernels read from
// device memory is checked against the scratch capacity (and table ids
// against the table count) before it indexes anything; a value out of range
// is clamped or its item skipped, and counted in kCtrBad (an internal count
// out of range) or kCtrBadOffsets (the device offsets of a set batch
// disagree with the op count the host declared, kCtrHostN). The host turns
// either count into an error.
enum : int {
    kCtrDistinct = 0,    // distinct keys
    kCtrPlaced = 1,      // ops given a segment slot
    kCtrUp = 2,          // upserts listed
    kCtrEr = 3,          // erases listed
    kCtrMid = 4,         // block segments
    kCtrWarp = 5,        // warp segments
    kCtrBad = 6,         // device-read counts or ids out of range (must stay 0)
    kCtrBadOffsets = 7,  // set batch: offsets[ntables] != kCtrHostN, or an op outside its table
    kCtrHostN = 8,       // set batch: op count from the host's offsets (copied before the kernels)
    kCtrRepeat = 9,      // one table's batch: nonzero once k_apply_group met a key twice
    kCtrSlots = 16
};
constexpr uint32_t kNoId = 0xffffffffu;  // a cell left without a distinct-key id


// Upsizes of many subtables (of different tables) in one launch: job j
// doubles old_sub (old_nb buckets, subtable index t of its table) into
// new_sub; its blocks are [block0, next job's block0). Passed by value as the
// kernel's parameter block, so at most kMaxResizeJobs per launch.
struct ResizeJob {
    const void *old_sub;
    void *new_sub;
    uint64_t magic;  // fastmod reciprocal of 2 * old_nb
    uint32_t old_nb, t, block0;
    uint32_t table;  // member of a table set (jobs the set's upsize policy lists on the device)
};
constexpr uint32_t kMaxResizeJobs = 768;
constexpr uint32_t kResizeChunksPerBlock = 2048;  // 32-byte chunks a block moves
struct ResizeJobs {
    uint32_t n, blocks;
    ResizeJob j[kMaxResizeJobs];
};
static_assert(sizeof(ResizeJobs) <= 32000, "kernel parameter block limit");

// The subtable an upsize doubles (api.cpp:115-122): the first one after a
// subtable twice its size, else subtable 0 (subtables grow in index order).
__host__ __device__ inline uint32_t pick_up_index(const uint32_t *nb, uint32_t d) {
    for (uint32_t i = 0; i + 1 < d; ++i)
        if (nb[i] == 2u * nb[i + 1]) return i + 1;
    return 0;
}

// A table-set member's next upsize target, allocated by the host ahead of
// the round that needs it: new_sub holds 2 * old_nb buckets for subtable ti.
// It fits only while subtable ti is the one pick_up_index names and still
// has old_nb buckets.
struct Spare {
    void *new_sub;  // null: none
    uint32_t ti, old_nb;
};
// What the device half of a set round's upsize policy did: jobs listed for
// k_resize_up_list (tasks of kResizeChunksPerBlock chunks), and whether a
// member needs more than its one device upsize (phase B then waits for the
// host to apply the rest of the policy).
struct SetPolicyOut {
    uint32_t njobs, ntasks, host, pad;
};

// Launch parameters picked once per kernel from the occupancy calculator.
struct LaunchCtx {
    int sms;
    cudaStream_t stream;
    int max_blocks_per_sm = 0;  // 0: as many as fit (else a cap, chosen by a tuner)
    // optional second stream for launches independent of the main sequence:
    // forked after `fork` is recorded on `stream`, joined back through `join`
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};

// Kernel launchers, one set per key width; `sb` = bucket bytes (32/64/128).
// All return cudaGetLastError() of their launches.
template <int KB> struct Ops {
    static cudaError_t find(const LaunchCtx &L, const Desc &D, int sb, const void *keys,
                            void *vals, uint32_t vb, uint32_t *hits, uint64_t n);
    // the batch dedup of a chunk. With the table's own scratch (winbits
    // set) it first clears the chunk's cells, winner bits and repeat flag,
    // and `nzero` 64-bit words at `zero` (the call counters), in one launch;
    // without, the caller has cleared the cells.
    static cudaError_t dedup(const LaunchCtx &L, const Scratch &S, const void *keys, uint64_t n,
                             DedupMode mode, unsigned long long *zero = nullptr,
                             uint32_t nzero = 0);
    // insert: place or update every op; ops whose two buckets are full go to
    // list_a (counted in pending). new_keys = caller promises absent keys.
    static cudaError_t place(const LaunchCtx &L, const Desc &D, int sb, const Scratch &S,
                             bool use_dedup, bool new_keys, const void *keys, const void *vals,
                             uint32_t vb, uint64_t n, Counters *ctr);
    // eviction walks for the entries of `src` (count at *src_count); entries
    // that reach the bound go to `dst` (count at *dst_count). count_new adds
    // successes to ctr->inserted and ctr->size.
    static cudaError_t walk(const LaunchCtx &L, const Desc &D, int sb, const void *src,
                            const unsigned long long *src_count, void *dst,
                            unsigned long long *dst_count, uint64_t dst_cap, uint32_t max_evict,
                            bool count_new, Counters *ctr, uint64_t max_entries);
    static cudaError_t erase(const LaunchCtx &L, const Desc &D, int sb, const Scratch &S,
                             bool use_dedup, const void *keys, uint64_t n, uint32_t *bits,
                             Counters *ctr);
    static cudaError_t resize_up(const LaunchCtx &L, int sb, uint32_t t, const void *old_sub,
                                 uint32_t old_nb, void *new_sub);
    // J.n jobs in one launch of J.blocks blocks (job block ranges filled in)
    static cudaError_t resize_up_many(const LaunchCtx &L, int sb, const ResizeJobs &J);
    // the jobs a set's device policy listed (out->njobs of them, at most
    // max_jobs, out->ntasks tasks), on a grid fixed at launch
    static cudaError_t resize_up_list(const LaunchCtx &L, int sb, const ResizeJob *jobs,
                                      const SetPolicyOut *out, uint32_t max_jobs);
    // device half of a set round's upsize policy (one block): members whose
    // upserts take them above upper x capacity switch to their spare subtable
    // (descriptor rewritten, move listed in jobs, grew[t] = 1)
    static cudaError_t set_policy(const LaunchCtx &L, Desc *descs, uint32_t ntables,
                                  const Counters *tctr, const uint32_t *tup, const uint32_t *ter,
                                  const Spare *spares, double upper, uint32_t slots, int sb,
                                  ResizeJob *jobs, uint8_t *grew, SetPolicyOut *out);
    // halve an even subtable: merged buckets to new_sub, leftovers to list;
    // a tile-copy wait gives up after tile_wait_tries polls (counted in
    // *timeouts; old_sub is only read)
    static cudaError_t resize_down(const LaunchCtx &L, int sb, const void *old_sub,
                                   uint32_t old_nb, void *new_sub, void *list,
                                   unsigned long long *list_count, uint64_t list_cap,
                                   unsigned long long *spill, unsigned long long *timeouts,
                                   uint32_t tile_wait_tries);
    // every live slot of one subtable to list (general rehash)
    static cudaError_t collect(const LaunchCtx &L, int sb, const void *sub, uint32_t nb,
                               void *list, unsigned long long *list_count, uint64_t list_cap,
                               unsigned long long *spill);
    // mixed batches (dyc_apply.cuh). One table: apply_group (group +
    // compact), find of the distinct keys, apply_scatter, apply_replay.
    // Many tables (dyc_set.cuh): set_group replaces apply_group, and
    // set_find / set_mutate / set_walk replace find / erase + place / walk.
    static cudaError_t apply_group(const LaunchCtx &L, const ApplyScratch &A, const void *keys,
                                  uint64_t n);
    // a mixed batch whose keys are all distinct, in one probe pass (ops left
    // without a slot go to S.list_a, counted in ctr->pending). With a single
    // bitmap (a single_pass batch after its grouping and scatter), only the
    // ops whose bit is set, and their hit bits are ORed in; all ops when
    // *gate is 0 (no key repeated, so the scatter did not run).
    static cudaError_t apply_unique(const LaunchCtx &L, const Desc &D, int sb, const Scratch &S,
                                    const uint8_t *ops, const void *keys, const void *vals,
                                    uint32_t vb, void *vals_out, uint32_t *bits_out, uint64_t n,
                                    Counters *ctr, const uint32_t *single = nullptr,
                                    const unsigned long long *gate = nullptr);
    // *count += the INSERT ops among ops[0..n)
    static cudaError_t count_inserts(const LaunchCtx &L, const uint8_t *ops, uint64_t n,
                                     unsigned long long *count);
    // after the find of the distinct keys: single-op keys resolved in op
    // order, the other ops scattered into their keys' segments. n_ptr (many
    // tables): the op count on the device; n then only sizes grids
    static cudaError_t apply_scatter(const LaunchCtx &L, const ApplyScratch &A, uint64_t n,
                                     const uint32_t *n_ptr, const uint8_t *ops, const void *vals,
                                     uint32_t vb, void *vals_out, uint32_t *bits_out);
    static cudaError_t apply_replay(const LaunchCtx &L, const ApplyScratch &A, const uint8_t *ops,
                                   const void *vals, uint32_t vb, void *vals_out,
                                   uint32_t *bits_out, uint64_t n, uint64_t max_distinct,
                                   const uint32_t *n_ptr = nullptr);
    // prep (counters, gctr, result bits, cell regions) + grouping + compaction
    static cudaError_t set_group(const LaunchCtx &L, const ApplyScratch &A, const uint32_t *off,
                                 const void *keys, uint64_t n, uint32_t *bits, Counters *gctr);
    // The set kernels below read their item counts from device memory and
    // clamp them to max_n / max_entries (the capacity of the lists behind
    // them); a table id at or above ntables skips its item. Either event is
    // counted in *bad. hint: the members keep their lines in the L2 (their
    // probes carry L2 eviction-priority hints; plain loads otherwise).
    static cudaError_t set_find(const LaunchCtx &L, const Desc *descs, uint32_t ntables, int sb,
                                const void *keys, const uint32_t *tids,
                                const unsigned long long *n_ptr, uint64_t max_n, void *vals,
                                uint32_t vb, uint32_t *hits, unsigned long long *bad,
                                bool hint = false);
    // erases and upserts of a set batch in one launch (max_n: both lists'
    // bound); nothing when *hold is nonzero (the host finishes the policy first)
    static cudaError_t set_mutate(const LaunchCtx &L, const Desc *descs, uint32_t ntables,
                                  Counters *tctr, int sb, const void *er_keys,
                                  const uint32_t *er_tids, const unsigned long long *ne_ptr,
                                  const void *up_keys, const void *up_vals, uint32_t vb,
                                  const uint32_t *up_tids, const unsigned long long *nu_ptr,
                                  uint64_t max_n, void *list_a, uint32_t *list_a_tid,
                                  uint64_t list_cap, Counters *gctr, unsigned long long *bad,
                                  const uint32_t *hold = nullptr, bool hint = false);
    // the ops of a single_pass set batch whose key has no other op in it
    // (and key-0 ops), one probe each (k_set_unique); max_n bounds the grid,
    // the op count is read on the device; nothing when *hold is nonzero
    static cudaError_t set_unique(const LaunchCtx &L, const ApplyScratch &A, const uint32_t *off,
                                  const Desc *descs, uint32_t ntables, Counters *tctr, int sb,
                                  const uint8_t *ops, const void *keys, const void *vals,
                                  uint32_t vb, void *vals_out, uint32_t *bits_out,
                                  uint64_t max_n, void *list_a, uint32_t *list_a_tid,
                                  uint64_t list_cap, Counters *gctr, const uint32_t *hold,
                                  bool hint);
    static cudaError_t set_walk(const LaunchCtx &L, const Desc *descs, uint32_t ntables,
                                Counters *tctr, int sb, const void *src, const uint32_t *src_tid,
                                const unsigned long long *src_count, void *dst, uint32_t *dst_tid,
                                unsigned long long *dst_count, uint64_t dst_cap,
                                uint32_t max_evict, Counters *gctr, uint64_t max_entries,
                                unsigned long long *bad);
    // set every fingerprint bit of every bucket of a subtable
    static cudaError_t mark_all(const LaunchCtx &L, int sb, void *sub, uint32_t nb);
    static cudaError_t export_all(const LaunchCtx &L, const Desc &D, int sb, void *keys,
                                  void *vals, uint32_t vb, uint64_t cap,
                                  unsigned long long *count);
};

}  // namespace dyc
