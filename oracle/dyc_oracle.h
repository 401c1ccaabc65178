/*
 * dyc_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * The oracle: a CPU restatement of the DyCuckoo hot path of the reference
 * (pauline-ly/databases_gpu, GPU/dyhash). It is the checker for the CUDA
 * library and the timed CPU baseline. Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU legs may load it; the product library never links it.
 *
 * Two independent models live here:
 *   orc_ck_*  -- the reference's cuckoo table as the reference builds it
 *                (d subtables, B-slot buckets of packed key<<32|value words,
 *                the reference's hash functions, pair choice, eviction rule,
 *                resize kernels and sizing), run sequentially or on host threads.
 *   orc_map_* -- the key->value semantics every implementation must produce
 *                (upsert, batch-order duplicate rule, erase counts).
 */
#ifndef DYC_ORACLE_H
#define DYC_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---- MT19937 (Matsumoto & Nishimura 2002); the reference's tests seed it
 *      with 10327 (GPU/dyhash/Main_backup_0910.cpp:180). ---- */
typedef struct { uint32_t mt[624]; int mti; } orc_mt;
void     orc_mt_seed(orc_mt *st, uint32_t seed);
uint32_t orc_mt_u32(orc_mt *st);
uint32_t orc_mt_u31(orc_mt *st);
double   orc_mt_real1(orc_mt *st);
void     orc_mt_fill_u32(orc_mt *st, uint32_t *out, uint64_t n);

/* ---- key generators (GPU/dyhash/random_numbers.cpp) ---- */
void orc_shuffle(orc_mt *st, uint32_t n, uint32_t *a);
int  orc_gen_unique_ref(orc_mt *st, uint32_t *out, uint32_t n, uint32_t max_number);
void orc_gen_queries(orc_mt *st, uint32_t size, float failure_rate, uint32_t *pool,
                     uint32_t *queries);
int  orc_gen_unique_full(orc_mt *st, uint32_t *out, uint32_t n);

/* ---- hash functions and pair choice (GPU/dyhash/cuckoo.cu:27-213) ---- */
#define ORC_PRIME 294967291u
uint32_t orc_hash1(uint32_t k);
uint32_t orc_hash2(uint32_t k);
uint32_t orc_hash3(uint32_t k);
uint32_t orc_hash4(uint32_t k);
uint32_t orc_hash5(uint32_t k);
uint32_t orc_fold64(uint64_t k);
uint32_t orc_bucket_of(uint32_t hkey, uint32_t t, uint32_t nbuckets);
uint32_t orc_choose_hash(uint32_t hkey, uint32_t d);
uint32_t orc_pos1(uint32_t pair, uint32_t d);
uint32_t orc_pos2(uint32_t pair, uint32_t d);
void     orc_hash_batch(const uint32_t *keys, uint64_t n, uint32_t d,
                        const uint32_t *nbuckets, uint32_t *t1, uint32_t *b1,
                        uint32_t *t2, uint32_t *b2);

/* ---- sizing (GPU/dyhash/api.cpp:4-22, :46-56) ---- */
int      orc_is_prime(int32_t num);
uint32_t orc_next_prime(uint32_t n);
uint32_t orc_subtable_buckets(uint64_t size, uint32_t d, uint32_t slots);
int      orc_pick_up_nb(const uint32_t *nbuckets, uint32_t d);   /* api.cpp:115-122 */
int      orc_pick_down_nb(const uint32_t *nbuckets, uint32_t d); /* api.cpp:147-153 */

/* ---- reference cuckoo table (u32 key / u32 value, packed key<<32|value) ---- */
typedef struct orc_ck orc_ck;
orc_ck  *orc_ck_new(uint64_t size, uint32_t d, uint32_t slots, uint32_t max_evict);
void     orc_ck_free(orc_ck *t);
uint64_t orc_ck_insert(orc_ck *t, const uint32_t *k, const uint32_t *v, uint64_t n,
                       int32_t *evict_counts);
uint64_t orc_ck_insert_mt(orc_ck *t, const uint32_t *k, const uint32_t *v, uint64_t n,
                          int threads);
void     orc_ck_find(const orc_ck *t, const uint32_t *k, uint32_t *out, uint64_t n,
                     int threads);
void     orc_ck_erase(orc_ck *t, const uint32_t *k, uint64_t n);
int      orc_ck_resize_up(orc_ck *t);
int      orc_ck_resize_down(orc_ck *t);
int      orc_ck_pick_up(const orc_ck *t);
int      orc_ck_pick_down(const orc_ck *t);
uint64_t orc_ck_capacity(const orc_ck *t);
uint64_t orc_ck_count(const orc_ck *t);
uint64_t orc_ck_dropped(const orc_ck *t);
void     orc_ck_layout(const orc_ck *t, uint32_t *nbuckets_out);
uint64_t orc_ck_export(const orc_ck *t, uint32_t *k, uint32_t *v);
const uint64_t *orc_ck_subtable(const orc_ck *t, uint32_t i);

/* ---- semantic map (u64 keys and values; key 0 is never stored) ----
 * op codes for orc_map_apply: 0 = find, 1 = insert (upsert), 2 = erase.
 * Per op, out_v/out_hit = the key's value / presence just before the op
 * (the value found, replaced or removed; 0 and no hit when absent).        */
typedef struct orc_map orc_map;
orc_map *orc_map_new(uint64_t cap_hint);
void     orc_map_free(orc_map *m);
uint64_t orc_map_size(const orc_map *m);
void     orc_map_apply(orc_map *m, const uint8_t *ops, const uint64_t *k, const uint64_t *v,
                       uint64_t n, uint64_t *out_v, uint8_t *out_hit);
uint64_t orc_map_export(const orc_map *m, uint64_t *k, uint64_t *v);

#ifdef __cplusplus
}
#endif
#endif
