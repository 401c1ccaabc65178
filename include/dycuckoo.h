/*
 * dycuckoo.h -- C ABI of the GB300 DyCuckoo dynamic hash table.
 *
 * A DyCuckoo table holds d subtables (2..6, default 4) of fixed-size buckets.
 * A key lives in one of two buckets: the pair of subtables chosen by the
 * reference's "two-layer" pair map, at the bucket given by the reference's
 * per-subtable hash functions. Batches of inserts, finds and erases run as
 * sm_103a kernels; a subtable grows or shrinks by a factor of two on its own
 * (upsize / downsize), driven by load-factor thresholds.
 *
 * Reference: pauline-ly/databases_gpu, GPU/dyhash. Each entry point below
 * names the reference interface it replaces. The reference's surface is the
 * C++ class hashAPI (GPU/dyhash/api.h:9-54) over device-pointer launch
 * wrappers (GPU/dyhash/cuckoo.h:99-114); this header is the C form of both,
 * and include/dycuckoo_hashapi.hpp restores the hashAPI class on top of it.
 *
 * Conventions
 *   - Every function returns a dyc_status; dyc_last_error() holds a message
 *     for the calling thread after a failure (the reference has no return
 *     codes: api.cpp uses checkCudaErrors and gtest EXPECT_* instead).
 *   - `d_` pointers are device pointers, `h_` pointers host pointers.
 *     Keys are uint32 or uint64 (key_bytes), values uint32 or uint64
 *     (value_bytes); arrays are dense.
 *   - `stream` is a cudaStream_t passed as void*. Calls on one table are
 *     ordered on the stream given; a table must not be used from two host
 *     threads at once. Different tables may be used from different threads.
 *   - Key 0 is the empty-slot sentinel (as in the reference): an insert of
 *     key 0 is rejected and counted, a find or erase of key 0 misses.
 *
 * Semantics (fixed by this library; the reference leaves them undefined)
 *   - insert is an upsert. Within one insert batch a repeated key keeps the
 *     value of its last occurrence (batch index order).
 *   - find writes the value (0 on a miss) and one hit bit per key.
 *   - erase removes present keys and reports how many it removed; within one
 *     erase batch only the first occurrence of a repeated key removes it.
 *   - no entry is ever dropped: an eviction chain that reaches its bound
 *     parks its entry, the table upsizes and the entry is placed again.
 *
 * Failures
 *   - A call that fails after it has taken entries out of the table (an
 *     upsize the device cannot serve: DYC_ENOMEM; eviction overflow that
 *     outlasts every upsize round: DYC_EOVERFLOW) keeps the entries it could
 *     not place on the host, "held" by the table, instead of dropping them
 *     (the reference drops them: cuckoo.cu:422-431, :714-722). Held entries
 *     are counted by dyc_size and reported in dyc_op_stats.held; finds do
 *     not see them until they are placed. Every later call on the table
 *     (any insert, find, erase, apply, resize, export or snapshot) places
 *     them first, upsizing as needed, and fails the same way if it still
 *     cannot; dyc_insert with n = 0 places them and nothing else.
 *   - A downsize that cannot allocate, or whose bounded copy waits give up
 *     (DYC_ETIMEOUT), leaves the table as it was.
 */
#ifndef DYCUCKOO_H
#define DYCUCKOO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum dyc_status {
    DYC_OK = 0,
    DYC_ENOMEM = 1,    /* device or pinned-host allocation failed */
    DYC_EINVAL = 2,    /* bad argument or unsupported configuration */
    DYC_EOVERFLOW = 3, /* eviction overflow persisted after repeated upsizes */
    DYC_ETIMEOUT = 4,  /* a bounded device-side wait gave up */
    DYC_ECUDA = 5,     /* a CUDA runtime call failed */
    DYC_ENOTSUP = 6    /* valid request this library does not support */
} dyc_status;

typedef struct dyc_table dyc_table;

/* Table configuration. Reference: compile-time macros of GPU/dyhash/dy_hash.h
 * (TABLE_NUM :32, MAX_ITER :33, ELEM_NUM_P_gpu :34) and test_uilt.h:1-2
 * (Upper_Bound / Lower_Bound), made runtime fields. */
typedef struct dyc_config {
    uint32_t key_bytes;      /* 4 or 8 */
    uint32_t value_bytes;    /* 4 or 8 (4-byte keys take 4-byte values) */
    uint32_t num_subtables;  /* d, 2..6; default 4 */
    uint32_t bucket_bytes;   /* 32, 64 or 128; default 128 (one DRAM line) */
    uint32_t max_evictions;  /* eviction chain bound; default 64 */
    uint32_t auto_resize;    /* 1: apply upper/lower load thresholds */
    uint64_t initial_size;   /* the hashAPI(size) argument: keys to size for */
    double upper_load;       /* upsize when size would exceed this; default 0.8 */
    double lower_load;       /* downsize below this after erase; default 0.5 */
    uint64_t min_downsize_capacity; /* no downsize at or below this capacity */
    int32_t device;          /* CUDA device ordinal; default 0 */
    uint32_t l2_resident;    /* 2: ask the L2 to keep the buckets: probes carry an
                                evict_last L2 cache hint and find streams its keys and
                                results with evict_first. 0 (default) and 1: plain
                                accesses, which measured faster on GB300 (a table of 1.2x
                                the L2: 51.1 against 48.1 G finds/s with the hints; hinted
                                loads of one hot line many warps read at once are 2.5x
                                slower). A table set follows its configuration for all
                                members. No counterpart in the reference. */
    uint32_t device_upsize;  /* table sets (dyc_set_apply with auto_resize): 0 (default)
                                keeps one upsize target allocated ahead for every member,
                                so a round's upsize policy runs on the device between the
                                round's two phases, inside its launch sequence; a member
                                that needs a second upsize in the round hands the rest of
                                the policy to the host. Costs device memory: a spare holds
                                twice the buckets of the member's next subtable to grow
                                (dyc_set_spare_bytes). 1: the host applies the policy
                                between the phases. Results are the same either way. */
    uint32_t reserved[5];
} dyc_config;

/* Per-call flags. */
#define DYC_FLAG_UNIQUE 1u    /* caller promises no key repeats in this batch: inserts and
                                 erases skip the batch dedup, dyc_apply resolves every op in
                                 one probe pass. A batch that repeats a key anyway gets
                                 unspecified results: a new key inserted twice may be
                                 stored twice, and counts may include it twice */
#define DYC_FLAG_NEW_KEYS 2u  /* insert: caller promises no key of the batch is in the table */
#define DYC_FLAG_NO_RESIZE 4u /* skip the load-factor policy for this call */

/* Counters of the last insert / erase / resize call on a table. */
typedef struct dyc_op_stats {
    uint64_t inserted;    /* new keys placed */
    uint64_t updated;     /* existing keys whose value was replaced */
    uint64_t erased;      /* keys removed */
    uint64_t rejected;    /* ops on key 0 */
    uint64_t superseded;  /* repeated keys resolved by the batch-order rule */
    uint64_t evict_steps; /* eviction exchanges performed */
    uint64_t overflowed;  /* chains that reached the bound and were re-placed */
    uint64_t resizes_up;
    uint64_t resizes_down;
    uint64_t split_phases; /* dyc_set_apply: 1 when the host read the batch's new-key
                              counts between its phases (a table could have filled) */
    uint64_t held;         /* entries held outside the table after a failed call (see
                              "Failures" below); the next call on the table places them */
} dyc_op_stats;

/* Defaults: 4-byte keys and values, d = 4, 128-byte buckets, bound 64,
 * thresholds 0.8 / 0.5, downsize guard 4*1M*1.2 slots (api.cpp:496). */
void dyc_config_default(dyc_config *cfg);

/* Replaces hashAPI::hashAPI(size) (GPU/dyhash/api.cpp:26-91): subtables of
 * nextPrime(size / (d * slots)) buckets, rounded up to even (api.cpp:46-56);
 * no __constant__ descriptor, any number of live tables. Subtables and
 * resize buffers come from a stream-ordered allocation pool the library
 * keeps per device (in place of the reference's CNMeM pool), which holds
 * freed memory up to a quarter of the device and returns it when the
 * device's last table is destroyed. */
dyc_status dyc_create(const dyc_config *cfg, dyc_table **out);

/* Replaces hashAPI::~hashAPI (api.cpp:93-109). */
dyc_status dyc_destroy(dyc_table *t);

/* Map `bytes` of device memory into the library pool of `device` now
 * (allocate and free), so that later resizes reuse it instead of mapping
 * new memory, which costs about 3 ms per GB on a GB300. The pool keeps at
 * most a quarter of the device's memory. Call it after creating a table on
 * the device (the pool is emptied when the device's last table goes). */
dyc_status dyc_pool_reserve(int32_t device, uint64_t bytes);

/* Replaces gpu_lp_insert / cuckoo_insert (GPU/dyhash/cuckoo.cu:858-877,
 * :324-432) and the resize-before-insert check of hashAPI::hash_insert_batch
 * (api.cpp:359-369). Returns after the batch is in the table (it reads the
 * overflow counters back). */
dyc_status dyc_insert(dyc_table *t, const void *d_keys, const void *d_vals, uint64_t n,
                      uint32_t flags, void *stream);

/* Replaces gpu_lp_search / cuckoo_search (cuckoo.cu:881-899, :460-520).
 * d_hit_bits_out (optional) receives ceil(n/32) words, bit i%32 of word i/32
 * set when key i was found. Asynchronous on `stream`. */
dyc_status dyc_find(dyc_table *t, const void *d_keys, void *d_vals_out,
                    uint32_t *d_hit_bits_out, uint64_t n, void *stream);

/* Replaces gpu_lp_delete / cuckoo_delete (cuckoo.cu:901-916, :524-587) and the
 * downsize-after-delete check of hash_delete_batch (api.cpp:494-505).
 * d_erased_bits_out (optional) as for find; h_erased_count (optional)
 * receives the number of keys removed. Returns after the erase is complete. */
dyc_status dyc_erase(dyc_table *t, const void *d_keys, uint64_t n,
                     uint32_t *d_erased_bits_out, uint64_t *h_erased_count,
                     uint32_t flags, void *stream);

/* Replaces hashAPI::resize_up + GPU_cuckoo_resize_up (api.cpp:112-141,
 * cuckoo.cu:731-758, kernel :600-627): doubles the subtable the reference
 * would pick. */
dyc_status dyc_resize_up(dyc_table *t, void *stream);

/* Replaces hashAPI::resize_low + GPU_cuckoo_resize_down (api.cpp:143-173,
 * cuckoo.cu:762-788, kernel :638-728): halves the subtable the reference
 * would pick; entries that no longer fit are placed again, never dropped. */
dyc_status dyc_resize_down(dyc_table *t, void *stream);

/* Live key count (hashAPI::num_size, exact here) and slot capacity
 * (hashAPI::table_size). */
dyc_status dyc_size(dyc_table *t, uint64_t *size);
dyc_status dyc_capacity(dyc_table *t, uint64_t *capacity);

/* Buckets per subtable (cuckoo.h:39-51 Lsize >> 4) and the subtable count. */
dyc_status dyc_layout(dyc_table *t, uint32_t *nbuckets_out, uint32_t *num_subtables);

/* Device address and byte size of subtable i (the reference's
 * table.table[i], cuckoo.h:42). Slots are bucket_bytes/slot_bytes per
 * bucket; a 4-byte-key slot is key | value << 32, an 8-byte-key slot is
 * {key, value} (16 bytes). In 128-byte buckets the last slot is a metadata
 * word, not an entry: bit f of its low 64 bits is set once some key k whose
 * first-probe bucket this is, with f = (fold(k) * 0x9E3779B1 mod 2^32) >> 26,
 * was stored in its second bucket (fold(k) = k for 4-byte keys). */
dyc_status dyc_subtable(dyc_table *t, uint32_t i, void **d_ptr, uint64_t *bytes);

/* Every live (key, value) into d_keys_out / d_vals_out (no order), at most
 * `capacity` of them; *n_out = number of live entries. The reference has no
 * export; its debug dump is show_table (cuckoo.cu:795-816). */
dyc_status dyc_export(dyc_table *t, void *d_keys_out, void *d_vals_out, uint64_t capacity,
                      uint64_t *n_out, void *stream);

/* Counters of the last insert / erase / resize call. */
dyc_status dyc_last_stats(dyc_table *t, dyc_op_stats *out);

/* Host-buffer forms: the signatures of hashAPI::hash_insert / hash_search /
 * hash_delete (api.cpp:184-303). They stage through pinned buffers owned by
 * the table and return when the results are in host memory. */
dyc_status dyc_insert_host(dyc_table *t, const void *h_keys, const void *h_vals, uint64_t n,
                           uint32_t flags);
dyc_status dyc_find_host(dyc_table *t, const void *h_keys, void *h_vals_out,
                         uint32_t *h_hit_bits_out, uint64_t n);
dyc_status dyc_erase_host(dyc_table *t, const void *h_keys, uint64_t n,
                          uint32_t *h_erased_bits_out, uint64_t *erased_count);

/* Op codes of dyc_apply. */
#define DYC_OP_FIND 0u
#define DYC_OP_INSERT 1u
#define DYC_OP_ERASE 2u

/* Mixed batch: n ops, op i = (d_ops[i], d_keys[i], d_vals[i]), applied in
 * batch index order. The reference names this kernel family but never
 * shipped it (README.md:9-10, "mixed insert/find/delete kernels ... not
 * uploaded yet"); the semantics are those of the single-op calls, in order:
 *   - FIND   : d_vals_out[i] = value (0 if absent), bit i = present;
 *   - INSERT : upsert of d_vals[i]; d_vals_out[i] = previous value (0 if the
 *              key was absent), bit i = key was present before the op;
 *   - ERASE  : removes the key; d_vals_out[i] = removed value (0 if absent),
 *              bit i = key was present before the op.
 * An op sees the latest earlier op on its key in the batch, else the table
 * as it was before the call. Ops on key 0 miss and change nothing.
 * d_vals is read only for INSERT ops but must hold n values; d_vals_out and
 * d_bits_out (ceil(n/32) words) are optional. Ops other than 0/1/2 are
 * treated as FIND. Inserts may upsize first (projected load above
 * upper_load); the batch may downsize after (load below lower_load), unless
 * DYC_FLAG_NO_RESIZE. Returns after the batch is in the table.
 * DYC_FLAG_UNIQUE (no key repeats in the batch): every op is resolved and
 * applied in one probe pass of its key's buckets. There is no grouping of
 * the batch by key. The results are the same. The upsize policy then
 * counts every INSERT op as a possible new key, as dyc_insert does.
 * Without the flag the batch is grouped by key on the device: keys with
 * one op in the chunk take the same one-pass kernel, and only repeated keys
 * go through the per-key replay (no host round trip in between). */
dyc_status dyc_apply(dyc_table *t, const uint8_t *d_ops, const void *d_keys, const void *d_vals,
                     uint64_t n, void *d_vals_out, uint32_t *d_bits_out, uint32_t flags,
                     void *stream);

/* ---- Wide values -----------------------------------------------------------
 * Tables whose values are value_bytes long (any multiple of 4 up to 65536),
 * the counterpart of the reference's lock-based variant for values wider
 * than a slot (GPU/warp: key[]/value[] buckets, cuckoo.h:15-18, bucket locks
 * cuckoo.cu:95-101, delete returning the value :353-359). Here the cuckoo
 * table maps each key to a 32-bit handle, a row of a device value heap; a
 * batch is deduplicated before it touches the table, so every key has one
 * writer and no lock is needed, and evictions and resizes move the (key,
 * handle) slot, never the value. A find costs one more random access (the
 * heap row). Semantics are those of the plain table: upsert, last insert of
 * a key in a batch wins, first erase removes; erase hands back the removed
 * values. Arrays of values are dense, value_bytes per key. */
typedef struct dyc_wide dyc_wide;

/* cfg as for dyc_create (its value_bytes is ignored: the table holds
 * handles); the heap starts with room for cfg->initial_size values and
 * doubles when needed. */
dyc_status dyc_wide_create(const dyc_config *cfg, uint32_t value_bytes, dyc_wide **out);
dyc_status dyc_wide_destroy(dyc_wide *w);
/* Returns after the batch is in the table. */
dyc_status dyc_wide_insert(dyc_wide *w, const void *d_keys, const void *d_vals, uint64_t n,
                           uint32_t flags, void *stream);
/* Values of hits, zeros for misses; d_hit_bits optional. Asynchronous. */
dyc_status dyc_wide_find(dyc_wide *w, const void *d_keys, void *d_vals_out, uint32_t *d_hit_bits,
                         uint64_t n, void *stream);
/* d_vals_out (optional): the removed value for each op that removed its key,
 * zeros for the others. Returns after the erase is complete. */
dyc_status dyc_wide_erase(dyc_wide *w, const void *d_keys, uint64_t n, void *d_vals_out,
                          uint32_t *d_erased_bits, uint64_t *h_erased_count, uint32_t flags,
                          void *stream);
/* Every live (key, value), at most `capacity`; *n_out = live entries. */
dyc_status dyc_wide_export(dyc_wide *w, void *d_keys_out, void *d_vals_out, uint64_t capacity,
                           uint64_t *n_out, void *stream);
/* The key -> handle table (for its size, capacity and layout). */
dyc_status dyc_wide_table(dyc_wide *w, dyc_table **out);
dyc_status dyc_wide_last_stats(dyc_wide *w, dyc_op_stats *out);

/* ---- Snapshot / restore ----------------------------------------------------
 * A snapshot is a host buffer: this 256-byte header, then every subtable's
 * buckets in subtable order, byte for byte as they are in device memory (the
 * slot layout of dyc_subtable). Restoring gives a table with the same
 * configuration, subtable sizes and slot positions, so it behaves exactly as
 * the snapshotted one. The reference has no checkpoint (it writes only
 * diagnostics, api.cpp:221-242). Little-endian; widths are fixed. */
typedef struct dyc_snapshot_header {
    char magic[8];              /* "DYCSNAP1" */
    uint32_t version;           /* 2 (metadata words hold displacement fingerprints) */
    uint32_t header_bytes;      /* 256 */
    uint32_t key_bytes, value_bytes, bucket_bytes, num_subtables;
    uint32_t max_evictions, auto_resize;
    uint64_t size;              /* live keys */
    uint64_t capacity;          /* entry slots */
    double upper_load, lower_load;
    uint64_t min_downsize_capacity, initial_size;
    uint32_t nbuckets[6];       /* per subtable; unused entries 0 */
    uint64_t payload_bytes;     /* sum of nbuckets[i] * bucket_bytes */
    uint64_t checksum;          /* sum over the payload's 64-bit words w[i] of
                                   splitmix64(w[i] ^ i * 0x9E3779B97F4A7C15), mod 2^64 */
    uint8_t reserved[128];
} dyc_snapshot_header;

/* Bytes dyc_snapshot writes (header + payload). */
dyc_status dyc_snapshot_bytes(dyc_table *t, uint64_t *bytes);

/* Write the table into h_buf (at least dyc_snapshot_bytes). Waits for work
 * queued on `stream`, returns when the buffer is complete. */
dyc_status dyc_snapshot(dyc_table *t, void *h_buf, uint64_t buf_bytes, void *stream);

/* A new table on `device` from a snapshot. DYC_EINVAL (and no table) when
 * the header is malformed (or of another version), the buffer is short or the checksum of the
 * restored subtables does not match. */
dyc_status dyc_restore(const void *h_buf, uint64_t buf_bytes, int32_t device, dyc_table **out);

/* ---- Table sets ----------------------------------------------------------
 * Many independent tables (each a dyc_table with its own size, subtables and
 * resizes) whose mixed batches are served together: one launch sequence per
 * batch for the whole set, each launch a grid-stride pass over a work list
 * that spans every table, instead of one launch sequence per table. The
 * reference serves one table per hashAPI object; this extends it to the
 * many-small-tables case (no reference counterpart).
 *
 * A batch is given as per-table op ranges: the ops of table t are indices
 * [offsets[t], offsets[t+1]) of d_ops / d_keys / d_vals / d_vals_out and
 * bits of d_bits_out, with offsets[0] = 0 and ntables + 1 entries (a device
 * copy, read by the kernels, and a host copy, used to size scratch).
 * Per table the semantics and results are exactly those of dyc_apply on that
 * table with its range; the resize policy runs per table. A batch holds
 * fewer than 2^31 ops. */
typedef struct dyc_set dyc_set;

#define DYC_FLAG_GRAPH 8u /* dyc_set_apply: run the launch sequences as CUDA graphs,
                             captured on the second call with the same arrays
                             and replayed after that, whatever the op count (the
                             kernels read it from the device offsets); up to
                             four array sets are kept */

/* ntables tables sharing cfg's key/value width, bucket size, eviction bound
 * and thresholds; table t is sized for sizes[t] keys (the hashAPI(size)
 * argument) and has num_subtables[t] subtables (NULL: cfg->num_subtables). */
dyc_status dyc_set_create(const dyc_config *cfg, uint32_t ntables, const uint64_t *sizes,
                          const uint32_t *num_subtables, dyc_set **out);
dyc_status dyc_set_destroy(dyc_set *s);

/* Launch and table parameters, typically chosen by a tuner per table-size
 * class (databases_gpu_gb300/tune.py): blocks_per_sm caps the resident
 * blocks per SM of the set's launches (0: as many as fit); max_evictions
 * (NULL: unchanged) gives every member its own eviction bound. */
dyc_status dyc_set_configure(dyc_set *s, uint32_t blocks_per_sm, const uint32_t *max_evictions);

/* Member table i. Single-table calls may be made on it between set calls;
 * it is destroyed with the set. */
dyc_status dyc_set_table(dyc_set *s, uint32_t i, dyc_table **out);

/* Live keys and slot capacity of every member (host arrays of ntables). */
dyc_status dyc_set_sizes(dyc_set *s, uint64_t *h_sizes, uint64_t *h_capacities);

/* Device bytes the set holds beside its members' subtables: the upsize
 * targets of dyc_config.device_upsize (0 when it is 1 or auto_resize is off)
 * and the subtables they replaced. At the next dyc_set_apply a replaced
 * subtable is either freed or kept to serve as a later upsize target
 * (dyc_set_spare_cache). */
dyc_status dyc_set_spare_bytes(dyc_set *s, uint64_t *bytes);

/* Bound on the replaced subtables a set keeps for reuse as upsize targets
 * (default: a quarter of the members' bytes at creation; 0 keeps none).
 * A kept block serves a later target of at most a quarter fewer bytes, so
 * a round's upsizes make no allocation or free on a hit. Blocks above a
 * lowered bound are freed at once (stream-ordered on the legacy stream).
 * The request server lowers it to an eighth of its HBM headroom. */
dyc_status dyc_set_spare_cache(dyc_set *s, uint64_t max_bytes);

/* Mixed batch over the set (see above). Returns when the batch is in the
 * tables. flags: DYC_FLAG_NO_RESIZE, DYC_FLAG_GRAPH. d_offsets must hold
 * the same values as h_offsets: the kernels read the op count and the
 * tables' ranges from d_offsets, clamp them to what h_offsets declared, and
 * the call returns DYC_EINVAL after the batch when they disagree (or are
 * out of order); the ops then went to the tables d_offsets named. A count
 * or id the kernels read from device memory out of range (which no valid
 * call produces) returns DYC_ECUDA. */
dyc_status dyc_set_apply(dyc_set *s, const uint32_t *d_offsets, const uint32_t *h_offsets,
                         const uint8_t *d_ops, const void *d_keys, const void *d_vals,
                         void *d_vals_out, uint32_t *d_bits_out, uint32_t flags, void *stream);

/* The same batch as one dyc_apply per table, one table after another: the
 * per-table launch path, for comparison. Same results. */
dyc_status dyc_set_apply_each(dyc_set *s, const uint32_t *d_offsets, const uint32_t *h_offsets,
                              const uint8_t *d_ops, const void *d_keys, const void *d_vals,
                              void *d_vals_out, uint32_t *d_bits_out, uint32_t flags,
                              void *stream);

/* Counters of the last dyc_set_apply / dyc_set_apply_each, summed over the
 * tables. */
dyc_status dyc_set_last_stats(dyc_set *s, dyc_op_stats *out);

/* ---- Request server --------------------------------------------------------
 * A serving loop over a table set with one table per tenant (no reference
 * counterpart: the reference is a library called in batches). Requests --
 * mixed op batches in host memory for one tenant -- are submitted from any
 * thread and return a ticket at once. A pipeline of three threads runs
 * continuous batching: while the device executes one step, the next step is
 * assembled from every request that has arrived and is admitted (tenants'
 * ops grouped, copied host->device), and the previous step's results go back
 * device->host and to their requests. Requests of one tenant take effect in
 * submission order, ops of a request in index order, so each request's
 * results are those it gets when run alone after the earlier requests of its
 * tenant. Admission is first-in first-out against a cap on the device bytes
 * of tables, scratch and staging, counting each request's possible growth
 * with resize headroom; a request that cannot fit even on an idle server is
 * rejected with DYC_ENOMEM. */
typedef struct dyc_server dyc_server;

typedef struct dyc_server_config {
    uint64_t hbm_cap_bytes; /* admission cap in device bytes (0: none) */
    uint64_t max_step_ops;  /* most ops in one step (default 1 << 22); also the
                               largest request */
    uint32_t coalesce;      /* 1 (default): continuous batching over the set;
                               0: one request per step through dyc_apply on its
                               tenant's table (the per-request path) */
    uint32_t pad0;
    uint64_t pool_reserve_bytes; /* dyc_pool_reserve at creation, so tenant growth
                                    does not map memory inside steps; default
                                    DYC_POOL_RESERVE_AUTO: twice the tables' bytes
                                    at creation, within hbm_cap_bytes; 0: none */
    uint32_t reserved[4];
} dyc_server_config;

#define DYC_POOL_RESERVE_AUTO (~(uint64_t)0)

typedef struct dyc_server_stats {
    uint64_t requests;      /* completed (including rejected) */
    uint64_t ops;           /* ops of completed requests */
    uint64_t steps;         /* device steps run */
    uint64_t deferred;      /* requests that waited for memory at least once */
    uint64_t rejected;      /* requests that could never be admitted */
    uint64_t max_step_ops;  /* largest step */
    uint64_t device_bytes;  /* tables + scratch + staging, after the last step */
    double busy_seconds;    /* time the executor spent in device steps */
    uint64_t resizes_up;    /* table upsizes inside steps */
    uint64_t resizes_down;  /* table downsizes inside steps */
    double resize_step_seconds; /* executor time of the steps that resized a table */
    double assemble_seconds;    /* assembler time from taking requests to queuing the step */
    double exec_idle_seconds;   /* executor time waiting for an assembled step */
    uint64_t upload_late_steps; /* steps whose upload was still running when picked up */
    uint64_t split_steps;       /* steps with split_phases set */
} dyc_server_stats;

void dyc_server_config_default(dyc_server_config *c);

/* Tenant tables as dyc_set_create(table_cfg, ntenants, sizes, NULL). */
dyc_status dyc_server_create(const dyc_config *table_cfg, uint32_t ntenants,
                             const uint64_t *sizes, const dyc_server_config *cfg,
                             dyc_server **out);

/* Runs every submitted request, then stops the threads and frees everything. */
dyc_status dyc_server_destroy(dyc_server *s);

/* Queue a request; the host arrays must stay valid (and outputs unread)
 * until dyc_server_wait reports it done. h_vals_out (n values) and
 * h_bits_out (ceil(n/32) words) are optional; results as dyc_apply. */
dyc_status dyc_server_submit(dyc_server *s, uint32_t tenant, const uint8_t *h_ops,
                             const void *h_keys, const void *h_vals, uint64_t n,
                             void *h_vals_out, uint32_t *h_bits_out, uint64_t *ticket);

/* Wait for a request (timeout_ms < 0: no limit). DYC_OK when it completed,
 * with its own status in *req_status and submit-to-done time in
 * *latency_ns; DYC_ETIMEOUT when the limit passed first (wait again later).
 * A ticket can be waited for until it has been reported complete once. */
dyc_status dyc_server_wait(dyc_server *s, uint64_t ticket, int64_t timeout_ms,
                           dyc_status *req_status, uint64_t *latency_ns);

dyc_status dyc_server_stats_get(dyc_server *s, dyc_server_stats *out);

/* The tenant tables. Use them only while no request is queued or running. */
dyc_status dyc_server_set(dyc_server *s, dyc_set **out);

/* Erase that allocates nothing. It has no counterpart in the reference.
 *
 * For callers that must not allocate device memory while they run: a host
 * engine whose own allocator owns every byte of HBM (a buffer pool sized to
 * the device, or an admission budget that counts each allocation), or a
 * latency-bound request path that cannot take the device-wide
 * synchronisation cudaMalloc/cudaFree may cause. dyc_erase takes its
 * batch-dedup table from scratch the table allocates on demand; this form
 * takes it from one fixed device array compiled into the library instead
 * (6 MiB, held on every device that loads the library until the process
 * exits), and it never downsizes (a downsize allocates).
 *
 *   - at most 262144 keys per call; a larger n returns DYC_EINVAL and does
 *     nothing;
 *   - the first call on a device looks up the array's device address (a
 *     one-time set-up per device); make that first call before any stream
 *     capture;
 *   - every call shares the one array and clears what it needs first, so
 *     calls that overlap on the GPU (on different streams or host threads,
 *     for any tables) race and must be serialised by the caller;
 *   - results, erased bits, count and flags are as for dyc_erase, with
 *     DYC_FLAG_NO_RESIZE always in effect. */
dyc_status dyc_erase_noalloc(dyc_table *t, const void *d_keys, uint64_t n,
                             uint32_t *d_erased_bits_out, uint64_t *h_erased_count,
                             uint32_t flags, void *stream);

const char *dyc_status_string(dyc_status s);
const char *dyc_last_error(void);

/* Failure injection for tests of the error paths above (no counterpart in
 * the reference, which has no error paths). Process-wide, for tests only.
 *   DYC_INJECT_RESET: clear every injection.
 *   DYC_INJECT_POOL_ALLOC: the n-th allocation from the library pool from
 *     now on (subtables of resizes, downsize lists) fails as if the device
 *     were out of memory; n = 0 clears.
 *   DYC_INJECT_CHUNK_OPS: tables created from now on split inserts and
 *     erases into chunks of n ops (a multiple of 32, at most 2^22; 0 = the
 *     default 2^22), so that small tests reach the paths of many chunks.
 *   DYC_INJECT_WAIT_TRIES: the downsize kernel's bounded waits on its tile
 *     copies give up after n polls (n = 0: at the first poll); the wait for
 *     copies still in flight before a block exits keeps its full bound. */
#define DYC_INJECT_RESET 0u
#define DYC_INJECT_POOL_ALLOC 1u
#define DYC_INJECT_WAIT_TRIES 2u
#define DYC_INJECT_CHUNK_OPS 3u
dyc_status dyc_debug_inject(uint32_t kind, uint64_t n);

/* Number of device and pinned-host allocations the library has made in this
 * process (cudaMalloc, cudaMallocHost, allocations from its pool), for
 * tests that a call allocates nothing. No counterpart in the reference. */
dyc_status dyc_debug_alloc_count(uint64_t *count);

#ifdef __cplusplus
}
#endif
#endif /* DYCUCKOO_H */
