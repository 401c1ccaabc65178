/*
 * dyc_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle; see dyc_oracle.h).
 *
 * A plain-C restatement of the reference's DyCuckoo hot path, written from its
 * behaviour. Every function names the reference lines it follows. Nothing in
 * the product library (databases_gpu_gb300/csrc) includes or links this file.
 */
#include "dyc_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ======================================================================
 * MT19937, the published generator of Matsumoto & Nishimura (2002 init).
 * Reference copy: GPU/dyhash/mt19937ar.cpp:57-145 (init_genrand,
 * genrand_int32, genrand_int31, genrand_real1).
 * ====================================================================== */
#define MT_N 624
#define MT_M 397

void orc_mt_seed(orc_mt *st, uint32_t seed) {
    st->mt[0] = seed;
    for (int i = 1; i < MT_N; ++i) {
        uint32_t prev = st->mt[i - 1];
        st->mt[i] = 1812433253u * (prev ^ (prev >> 30)) + (uint32_t)i;
    }
    st->mti = MT_N;
}

static void mt_refill(orc_mt *st) {
    static const uint32_t mag[2] = {0u, 0x9908b0dfu};
    uint32_t *mt = st->mt;
    int kk;
    for (kk = 0; kk < MT_N - MT_M; ++kk) {
        uint32_t y = (mt[kk] & 0x80000000u) | (mt[kk + 1] & 0x7fffffffu);
        mt[kk] = mt[kk + MT_M] ^ (y >> 1) ^ mag[y & 1u];
    }
    for (; kk < MT_N - 1; ++kk) {
        uint32_t y = (mt[kk] & 0x80000000u) | (mt[kk + 1] & 0x7fffffffu);
        mt[kk] = mt[kk + (MT_M - MT_N)] ^ (y >> 1) ^ mag[y & 1u];
    }
    uint32_t y = (mt[MT_N - 1] & 0x80000000u) | (mt[0] & 0x7fffffffu);
    mt[MT_N - 1] = mt[MT_M - 1] ^ (y >> 1) ^ mag[y & 1u];
    st->mti = 0;
}

uint32_t orc_mt_u32(orc_mt *st) {
    if (st->mti >= MT_N) mt_refill(st);
    uint32_t y = st->mt[st->mti++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

uint32_t orc_mt_u31(orc_mt *st) { return orc_mt_u32(st) >> 1; }

double orc_mt_real1(orc_mt *st) { return orc_mt_u32(st) * (1.0 / 4294967295.0); }

void orc_mt_fill_u32(orc_mt *st, uint32_t *out, uint64_t n) {
    for (uint64_t i = 0; i < n; ++i) out[i] = orc_mt_u32(st);
}

/* ======================================================================
 * Key generators. GPU/dyhash/random_numbers.cpp:16-24 (Shuffle),
 * :26-77 (GenerateUniqueRandomNumbers), :96-117 (GenerateQueries).
 * ====================================================================== */
static int cmp_u32(const void *a, const void *b) {
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return (x > y) - (x < y);
}

void orc_shuffle(orc_mt *st, uint32_t n, uint32_t *a) {
    /* Fisher-Yates with a modulo draw, random_numbers.cpp:19-23 */
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t left = n - i;
        uint32_t j = i + (orc_mt_u32(st) % left);
        uint32_t t = a[i];
        a[i] = a[j];
        a[j] = t;
    }
}

/* Draw with `draw`, sort, mark repeats with `filler`, re-sort, redraw the tail
 * until n distinct values exist, then shuffle (random_numbers.cpp:34-73).
 * `full` selects 32-bit draws with 0 and 0xffffffff rejected (the key space
 * [1, 2^32-2] used by the u32 workloads) instead of the reference's 31-bit
 * draws. */
static int gen_unique(orc_mt *st, uint32_t *out, uint32_t n, uint32_t filler, int full) {
    uint32_t total = (uint32_t)(n * 1.1);
    if (total < n) total = n;
    uint32_t *tmp = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(total ? total : 1));
    if (!tmp) return 0;
    uint32_t uniq = 0;
    while (uniq < n) {
        for (uint32_t i = uniq; i < total; ++i) {
            uint32_t x;
            if (full) {
                do { x = orc_mt_u32(st); } while (x == 0u || x == 0xffffffffu);
            } else {
                do { x = orc_mt_u31(st); } while (x > filler);
            }
            tmp[i] = x;
        }
        qsort(tmp, total, sizeof(uint32_t), cmp_u32);
        uniq = 1;
        for (uint32_t i = 1; i < total; ++i) {
            if (tmp[i - 1] == tmp[i]) tmp[i - 1] = filler;
            else ++uniq;
        }
        qsort(tmp, total, sizeof(uint32_t), cmp_u32);
    }
    orc_shuffle(st, uniq, tmp);
    memcpy(out, tmp, sizeof(uint32_t) * (size_t)n);
    free(tmp);
    return 1;
}

int orc_gen_unique_ref(orc_mt *st, uint32_t *out, uint32_t n, uint32_t max_number) {
    return gen_unique(st, out, n, max_number, 0);
}

int orc_gen_unique_full(orc_mt *st, uint32_t *out, uint32_t n) {
    return gen_unique(st, out, n, 0xffffffffu, 1);
}

void orc_gen_queries(orc_mt *st, uint32_t size, float failure_rate, uint32_t *pool,
                     uint32_t *queries) {
    /* random_numbers.cpp:100-116: hits from pool[0,size), misses from
     * pool[size,2size), then one shuffle of the query array. */
    uint32_t nfail = (uint32_t)(failure_rate * size);
    uint32_t ngood = size - nfail;
    if (ngood) {
        orc_shuffle(st, size, pool);
        memcpy(queries, pool, sizeof(uint32_t) * ngood);
    }
    if (nfail) {
        orc_shuffle(st, size, pool + size);
        memcpy(queries + ngood, pool + size, sizeof(uint32_t) * nfail);
    }
    orc_shuffle(st, size, queries);
}

/* ======================================================================
 * Hash functions: GPU/dyhash/cuckoo.cu:27-64 (get_hash1..4), :110-120
 * (get_hash5), :76-90 (hash_function), :190-213 (choose_hash/pos1/pos2 for
 * four subtables), GPU/dyhash/diff_hash_num_pos_fun.cpp:14-188 (pair maps
 * for 2, 3, 5 and 6 subtables).
 * ====================================================================== */
uint32_t orc_hash1(uint32_t k) {
    k = ~k + (k << 15);
    k = k ^ (k >> 12);
    k = k + (k << 2);
    k = k ^ (k >> 4);
    k = k * 2057u;
    k = k ^ (k >> 16);
    return k;
}

uint32_t orc_hash2(uint32_t a) {
    a = (a + 0x7ed55d16u) + (a << 12);
    a = (a ^ 0xc761c23cu) ^ (a >> 19);
    a = (a + 0x165667b1u) + (a << 5);
    a = (a + 0xd3a2646cu) ^ (a << 9);
    a = (a + 0xfd7046c5u) + (a << 3);
    a = (a ^ 0xb55a4f09u) ^ (a >> 16);
    return a;
}

uint32_t orc_hash3(uint32_t s) { return ((s ^ 59064253u) + 72355969u) % ORC_PRIME; }

uint32_t orc_hash4(uint32_t a) {
    a = (a ^ 61u) ^ (a >> 16);
    a = a + (a << 3);
    a = a ^ (a >> 4);
    a = a * 0x27d4eb2du;
    a = a ^ (a >> 15);
    return a;
}

uint32_t orc_hash5(uint32_t a) {
    a -= (a << 6);
    a ^= (a >> 17);
    a -= (a << 9);
    a ^= (a << 4);
    a -= (a << 3);
    a ^= (a << 10);
    a ^= (a >> 15);
    return a;
}

/* 64-bit keys are folded to the 32-bit hash input; equality always uses all
 * 64 bits. The reference has no 64-bit key path; this fold is this
 * project's specification. */
uint32_t orc_fold64(uint64_t k) {
    uint32_t lo = (uint32_t)k, hi = (uint32_t)(k >> 32);
    return lo ^ hi ^ (0x9e3779b9u * hi);
}

uint32_t orc_bucket_of(uint32_t hk, uint32_t t, uint32_t nb) {
    uint32_t h;
    switch (t & 3u) {
    case 0: h = orc_hash1(hk); break;
    case 1: h = orc_hash2(hk); break;
    case 2: h = orc_hash3(hk); break;
    default: h = orc_hash4(hk); break;
    }
    return h % ORC_PRIME % nb;
}

uint32_t orc_choose_hash(uint32_t hk, uint32_t d) {
    switch (d) {
    case 2: return hk & 1u;
    case 3: return orc_hash5(hk) % 3u;
    case 5: return orc_hash5(hk) % 10u;
    case 6: return orc_hash5(hk) % 15u;
    default: return orc_hash5(hk) % 6u;
    }
}

uint32_t orc_pos1(uint32_t p, uint32_t d) {
    switch (d) {
    case 2: return p;
    case 3: return (p & 1u) ? 1u : 0u;
    case 5:
        if (p == 9u) return 3u;
        if (p & 1u) return 0u;
        if (p & 2u) return 2u;
        return 1u;
    case 6:
        if (p <= 4u) return 0u;
        if (p <= 8u) return 1u;
        if (p <= 11u) return 2u;
        if (p <= 13u) return 3u;
        return 4u;
    default:
        if (p & 1u) return 0u;
        if (p & 2u) return 2u;
        return 1u;
    }
}

uint32_t orc_pos2(uint32_t p, uint32_t d) {
    switch (d) {
    case 2: return p ^ 1u;
    case 3: return (p & 1u) ? 2u : (p >> 1) + 1u;
    case 5:
        if (p == 9u) return 4u;
        if (p & 1u) return (p >> 1) + 1u;
        if (p & 2u) return (p >> 2) + 3u;
        return (p >> 2) + 2u;
    case 6:
        if (p <= 4u) return p + 1u;
        if (p <= 8u) return p - 3u;
        if (p <= 11u) return p - 6u;
        if (p <= 13u) return p - 8u;
        return 5u;
    default:
        if (p & 1u) return (p >> 1) + 1u;
        if (p & 2u) return 3u;
        return (p >> 2) + 2u;
    }
}

void orc_hash_batch(const uint32_t *keys, uint64_t n, uint32_t d, const uint32_t *nb,
                    uint32_t *t1, uint32_t *b1, uint32_t *t2, uint32_t *b2) {
    for (uint64_t i = 0; i < n; ++i) {
        uint32_t p = orc_choose_hash(keys[i], d);
        uint32_t a = orc_pos1(p, d), b = orc_pos2(p, d);
        t1[i] = a;
        t2[i] = b;
        b1[i] = orc_bucket_of(keys[i], a, nb[a]);
        b2[i] = orc_bucket_of(keys[i], b, nb[b]);
    }
}

/* ======================================================================
 * Sizing: GPU/dyhash/api.cpp:4-11 (isPrime, which also calls 1 prime),
 * :13-22 (nextPrime), :47-54 (buckets per subtable, rounded up to even).
 * ====================================================================== */
int orc_is_prime(int32_t num) {
    if (num == 2 || num == 3) return 1;
    if (num % 6 != 1 && num % 6 != 5) return 0;
    for (int32_t i = 5; (int64_t)i * i <= num; i += 6)
        if (num % i == 0 || num % (i + 2) == 0) return 0;
    return 1;
}

uint32_t orc_next_prime(uint32_t n) {
    while (!orc_is_prime((int32_t)n)) ++n;
    return n;
}

uint32_t orc_subtable_buckets(uint64_t size, uint32_t d, uint32_t slots) {
    uint32_t s = (uint32_t)(size / ((uint64_t)d * slots));
    s = orc_next_prime(s);
    return (s & 1u) ? s + 1u : s;
}

/* ======================================================================
 * The reference cuckoo table. Slots are packed key<<32|value words
 * (GPU/dyhash/cuckoo.h:13-16); a bucket is `slots` consecutive words
 * (cuckoo.h:30-34, 16 in the reference); subtable t has nb[t] buckets
 * (cuckoo.h:39-51, Lsize = nb*slots).
 * ====================================================================== */
#define ORC_MAXD 6
struct orc_ck {
    uint32_t d, B, max_evict;
    uint32_t nb[ORC_MAXD];
    uint64_t *sub[ORC_MAXD];
    uint64_t capacity; /* hashAPI::table_size */
    uint64_t dropped;  /* entries lost at the end of an eviction chain */
};

static inline uint32_t ek(uint64_t e) { return (uint32_t)(e >> 32); }

/* makeEntry(k, v) with the reference's `int v` (cuckoo.cu:337-345,
 * cuckoo.h:14): a value >= 2^31 sign-extends and lowers the key part by 1. */
static inline uint64_t make_entry_ref(uint32_t k, uint32_t v) {
    return ((uint64_t)k << 32) + (uint64_t)(int64_t)(int32_t)v;
}

static inline uint32_t other_of(uint32_t p, uint32_t pre, uint32_t d) {
    /* get_pos, cuckoo.cu:310-312 */
    return (pre == orc_pos1(p, d)) ? orc_pos2(p, d) : orc_pos1(p, d);
}

orc_ck *orc_ck_new(uint64_t size, uint32_t d, uint32_t slots, uint32_t max_evict) {
    if (d < 2 || d > ORC_MAXD || slots == 0 || slots > 32 || (slots & (slots - 1))) return NULL;
    orc_ck *t = (orc_ck *)calloc(1, sizeof(orc_ck));
    if (!t) return NULL;
    t->d = d;
    t->B = slots;
    t->max_evict = max_evict;
    uint32_t nb = orc_subtable_buckets(size, d, slots);
    for (uint32_t i = 0; i < d; ++i) {
        t->nb[i] = nb;
        t->sub[i] = (uint64_t *)calloc((size_t)nb * slots, sizeof(uint64_t));
        if (!t->sub[i]) { orc_ck_free(t); return NULL; }
        t->capacity += (uint64_t)nb * slots;
    }
    return t;
}

void orc_ck_free(orc_ck *t) {
    if (!t) return;
    for (uint32_t i = 0; i < ORC_MAXD; ++i) free(t->sub[i]);
    free(t);
}

/* One eviction chain: warp_insert, cuckoo.cu:365-432. The 16-lane group
 * becomes a scan over the bucket's slots in lane order:
 *   empty slot (key 0) -> first one; else a resident whose pair id
 *   choose_hash(resident) differs from the current table id (the reference
 *   compares a pair id with a table id, :398-400; with two subtables every
 *   slot qualifies, diff_hash_num_pos_fun.cpp:3-6); else slot evict_num%B.
 * The exchanged-out word continues in the other table of its pair. After
 * max_evict exchanges the carried entry is dropped (:422-431). */
static int ck_chain(orc_ck *t, uint64_t entry, uint32_t pre, int32_t *count, int atomic) {
    const uint32_t d = t->d, B = t->B;
    for (uint32_t e = 0; e < t->max_evict; ++e) {
        uint32_t key = ek(entry);
        uint32_t tn = other_of(orc_choose_hash(key, d), pre, d);
        uint64_t *b = t->sub[tn] + (uint64_t)orc_bucket_of(key, tn, t->nb[tn]) * B;
        uint32_t mask = 0;
        for (uint32_t i = 0; i < B; ++i) {
            uint64_t s = atomic ? __atomic_load_n(&b[i], __ATOMIC_RELAXED) : b[i];
            if (ek(s) == 0) mask |= 1u << i;
        }
        if (!mask) {
            for (uint32_t i = 0; i < B; ++i) {
                uint64_t s = atomic ? __atomic_load_n(&b[i], __ATOMIC_RELAXED) : b[i];
                if (d == 2 || orc_choose_hash(ek(s), d) != tn) mask |= 1u << i;
            }
        }
        uint32_t c = mask ? (uint32_t)__builtin_ctz(mask) : (e & (B - 1));
        uint64_t old;
        if (atomic) {
            old = __atomic_exchange_n(&b[c], entry, __ATOMIC_RELAXED);
        } else {
            old = b[c];
            b[c] = entry;
        }
        if (count) ++*count;
        entry = old;
        if (entry == 0) return 1;
        pre = tn;
    }
    return 0;
}

static uint32_t first_pre(uint32_t k, uint32_t d) {
    /* cuckoo.cu:336-341: odd keys start in the second table of their pair */
    uint32_t pre = 100u;
    if (k & 1u) pre = other_of(orc_choose_hash(k, d), 100u, d);
    return pre;
}

uint64_t orc_ck_insert(orc_ck *t, const uint32_t *k, const uint32_t *v, uint64_t n,
                       int32_t *evict_counts) {
    /* cuckoo_insert, cuckoo.cu:324-355: no existence check; a repeated key
     * takes a second slot. */
    uint64_t fails = 0;
    for (uint64_t i = 0; i < n; ++i) {
        int32_t c = 0;
        if (!ck_chain(t, make_entry_ref(k[i], v[i]), first_pre(k[i], t->d), &c, 0)) ++fails;
        if (evict_counts) evict_counts[i] = c;
    }
    t->dropped += fails;
    return fails;
}

typedef struct {
    orc_ck *t;
    const uint32_t *k, *v, *q;
    uint32_t *out;
    uint64_t lo, hi, fails;
} ck_job;

static void *ck_insert_worker(void *arg) {
    ck_job *j = (ck_job *)arg;
    for (uint64_t i = j->lo; i < j->hi; ++i)
        if (!ck_chain(j->t, make_entry_ref(j->k[i], j->v[i]), first_pre(j->k[i], j->t->d), NULL, 1))
            ++j->fails;
    return NULL;
}

/* The same lock-free exchange chain run by host threads (one op per thread
 * at a time, like one 16-lane group per op on the GPU). */
uint64_t orc_ck_insert_mt(orc_ck *t, const uint32_t *k, const uint32_t *v, uint64_t n,
                          int threads) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t th[256];
    ck_job jobs[256];
    for (int i = 0; i < threads; ++i) {
        jobs[i].t = t;
        jobs[i].k = k;
        jobs[i].v = v;
        jobs[i].lo = n * (uint64_t)i / threads;
        jobs[i].hi = n * (uint64_t)(i + 1) / threads;
        jobs[i].fails = 0;
        pthread_create(&th[i], NULL, ck_insert_worker, &jobs[i]);
    }
    uint64_t fails = 0;
    for (int i = 0; i < threads; ++i) {
        pthread_join(th[i], NULL);
        fails += jobs[i].fails;
    }
    t->dropped += fails;
    return fails;
}

/* cuckoo_search, cuckoo.cu:460-520: probe pos1, then pos2; the first slot
 * whose key matches gives the value; a miss yields 0 (the host API
 * pre-zeroes the answer buffer, api.cpp:275). */
static inline uint32_t ck_find_one(const orc_ck *t, uint32_t k) {
    const uint32_t d = t->d, B = t->B;
    uint32_t p = orc_choose_hash(k, d);
    uint32_t tn = orc_pos1(p, d);
    const uint64_t *b = t->sub[tn] + (uint64_t)orc_bucket_of(k, tn, t->nb[tn]) * B;
    for (uint32_t i = 0; i < B; ++i)
        if (ek(b[i]) == k) return (uint32_t)b[i];
    tn = orc_pos2(p, d);
    b = t->sub[tn] + (uint64_t)orc_bucket_of(k, tn, t->nb[tn]) * B;
    for (uint32_t i = 0; i < B; ++i)
        if (ek(b[i]) == k) return (uint32_t)b[i];
    return 0;
}

static void *ck_find_worker(void *arg) {
    ck_job *j = (ck_job *)arg;
    for (uint64_t i = j->lo; i < j->hi; ++i) j->out[i] = ck_find_one(j->t, j->q[i]);
    return NULL;
}

void orc_ck_find(const orc_ck *t, const uint32_t *k, uint32_t *out, uint64_t n, int threads) {
    if (threads <= 1) {
        for (uint64_t i = 0; i < n; ++i) out[i] = ck_find_one(t, k[i]);
        return;
    }
    if (threads > 256) threads = 256;
    pthread_t th[256];
    ck_job jobs[256];
    for (int i = 0; i < threads; ++i) {
        jobs[i].t = (orc_ck *)t;
        jobs[i].q = k;
        jobs[i].out = out;
        jobs[i].lo = n * (uint64_t)i / threads;
        jobs[i].hi = n * (uint64_t)(i + 1) / threads;
        pthread_create(&th[i], NULL, ck_find_worker, &jobs[i]);
    }
    for (int i = 0; i < threads; ++i) pthread_join(th[i], NULL);
}

/* cuckoo_delete, cuckoo.cu:524-587: key 0 is skipped; every matching slot of
 * the pos1 bucket is cleared, and pos2 is only tried if pos1 had none. */
void orc_ck_erase(orc_ck *t, const uint32_t *k, uint64_t n) {
    const uint32_t d = t->d, B = t->B;
    for (uint64_t q = 0; q < n; ++q) {
        uint32_t key = k[q];
        if (key == 0) continue;
        uint32_t p = orc_choose_hash(key, d);
        uint32_t tabs[2] = {orc_pos1(p, d), orc_pos2(p, d)};
        for (int r = 0; r < 2; ++r) {
            uint32_t tn = tabs[r];
            uint64_t *b = t->sub[tn] + (uint64_t)orc_bucket_of(key, tn, t->nb[tn]) * B;
            int hit = 0;
            for (uint32_t i = 0; i < B; ++i)
                if (ek(b[i]) == key) { b[i] = 0; hit = 1; }
            if (hit) break;
        }
    }
}

/* hashAPI::resize_up target choice, api.cpp:115-122: the first subtable that
 * is half the size of its predecessor, else subtable 0. */
int orc_pick_up_nb(const uint32_t *nb, uint32_t d) {
    for (uint32_t i = 0; i + 1 < d; ++i)
        if (nb[i] == 2u * nb[i + 1]) return (int)i + 1;
    return 0;
}

/* hashAPI::resize_low target choice, api.cpp:147-153: the last subtable of
 * the larger group, else the last subtable. */
int orc_pick_down_nb(const uint32_t *nb, uint32_t d) {
    for (uint32_t i = 0; i + 1 < d; ++i)
        if (nb[i] > nb[i + 1]) return (int)i;
    return (int)d - 1;
}

int orc_ck_pick_up(const orc_ck *t) { return orc_pick_up_nb(t->nb, t->d); }
int orc_ck_pick_down(const orc_ck *t) { return orc_pick_down_nb(t->nb, t->d); }

/* Upsize: cuckoo_resize_up, cuckoo.cu:600-627, with the wrapper's size
 * doubling (:737-743) and the capacity update (api.cpp:129). Each word keeps
 * its slot index in the new bucket hash % 2nb, which is b or b+nb. */
int orc_ck_resize_up(orc_ck *t) {
    int ti = orc_ck_pick_up(t);
    const uint32_t B = t->B, nb = t->nb[ti], nnb = 2u * nb;
    uint64_t *nw = (uint64_t *)calloc((size_t)nnb * B, sizeof(uint64_t));
    if (!nw) return -1;
    const uint64_t *old = t->sub[ti];
    for (uint64_t b = 0; b < nb; ++b)
        for (uint32_t i = 0; i < B; ++i) {
            uint64_t e = old[b * B + i];
            if (e) nw[(uint64_t)orc_bucket_of(ek(e), (uint32_t)ti, nnb) * B + i] = e;
        }
    free(t->sub[ti]);
    t->sub[ti] = nw;
    t->nb[ti] = nnb;
    t->capacity += (uint64_t)nb * B;
    return ti;
}

/* Downsize: cuckoo_resize_down, cuckoo.cu:638-728, and the wrapper
 * (:762-788, api.cpp:143-173). New bucket j takes old[j][i], or when that is
 * empty old[j+nb'][B-1-i]; words of old[j+nb'] not taken are re-inserted with
 * the eviction chain starting from the resized table's pair partner. The
 * reference runs merges and re-inserts of different buckets concurrently
 * (a re-insert can land in a bucket not merged yet); this restatement merges
 * every bucket first and then re-inserts in bucket and slot order. */
int orc_ck_resize_down(orc_ck *t) {
    int ti = orc_ck_pick_down(t);
    const uint32_t B = t->B, nb = t->nb[ti], nnb = (nb + 1u) / 2u;
    uint64_t *nw = (uint64_t *)calloc((size_t)nnb * B, sizeof(uint64_t));
    uint64_t *resid = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)nnb * B + 1));
    if (!nw || !resid) { free(nw); free(resid); return -1; }
    const uint64_t *old = t->sub[ti];
    uint64_t nres = 0;
    for (uint64_t j = 0; j < nnb; ++j) {
        const uint64_t *b1 = old + j * B;
        const uint64_t *b2 = (j + nnb < nb) ? old + (j + nnb) * B : NULL;
        for (uint32_t i = 0; i < B; ++i) {
            uint64_t cross = b2 ? b2[B - 1 - i] : 0;
            uint64_t e = b1[i] ? b1[i] : cross;
            nw[j * B + i] = e;
            if (e != cross && cross != 0) resid[nres++] = cross;
        }
    }
    free(t->sub[ti]);
    t->sub[ti] = nw;
    t->nb[ti] = nnb;
    t->capacity -= (uint64_t)nnb * B;
    for (uint64_t r = 0; r < nres; ++r)
        if (!ck_chain(t, resid[r], (uint32_t)ti, NULL, 0)) ++t->dropped;
    free(resid);
    return ti;
}

uint64_t orc_ck_capacity(const orc_ck *t) { return t->capacity; }
uint64_t orc_ck_dropped(const orc_ck *t) { return t->dropped; }

void orc_ck_layout(const orc_ck *t, uint32_t *nb_out) {
    for (uint32_t i = 0; i < t->d; ++i) nb_out[i] = t->nb[i];
}

const uint64_t *orc_ck_subtable(const orc_ck *t, uint32_t i) {
    return i < t->d ? t->sub[i] : NULL;
}

uint64_t orc_ck_count(const orc_ck *t) {
    uint64_t c = 0;
    for (uint32_t s = 0; s < t->d; ++s)
        for (uint64_t i = 0; i < (uint64_t)t->nb[s] * t->B; ++i) c += t->sub[s][i] != 0;
    return c;
}

uint64_t orc_ck_export(const orc_ck *t, uint32_t *k, uint32_t *v) {
    uint64_t c = 0;
    for (uint32_t s = 0; s < t->d; ++s)
        for (uint64_t i = 0; i < (uint64_t)t->nb[s] * t->B; ++i) {
            uint64_t e = t->sub[s][i];
            if (!e) continue;
            k[c] = ek(e);
            v[c] = (uint32_t)e;
            ++c;
        }
    return c;
}

/* ======================================================================
 * Semantic map: what every implementation must return. Open addressing
 * with linear probing and backward-shift deletion; key 0 marks a free cell.
 *   insert = upsert; ops of one batch apply in index order (so a repeated
 *   insert key keeps the last value, and a find sees the latest earlier
 *   insert/erase of its key in the batch); erase reports whether the key
 *   was present and returns its value. Key 0 is the empty sentinel: an
 *   insert of it is rejected, a find or erase of it misses.
 * ====================================================================== */
struct orc_map {
    uint64_t *k, *v;
    uint64_t mask, n;
};

static inline uint64_t mix64(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

orc_map *orc_map_new(uint64_t hint) {
    orc_map *m = (orc_map *)calloc(1, sizeof(orc_map));
    if (!m) return NULL;
    uint64_t cap = 16;
    while (cap < 2 * hint) cap <<= 1;
    m->k = (uint64_t *)calloc(cap, sizeof(uint64_t));
    m->v = (uint64_t *)calloc(cap, sizeof(uint64_t));
    if (!m->k || !m->v) { orc_map_free(m); return NULL; }
    m->mask = cap - 1;
    return m;
}

void orc_map_free(orc_map *m) {
    if (!m) return;
    free(m->k);
    free(m->v);
    free(m);
}

uint64_t orc_map_size(const orc_map *m) { return m->n; }

static int map_grow(orc_map *m) {
    uint64_t oc = m->mask + 1, nc = oc * 2;
    uint64_t *ok = m->k, *ov = m->v;
    uint64_t *nk = (uint64_t *)calloc(nc, sizeof(uint64_t));
    uint64_t *nv = (uint64_t *)calloc(nc, sizeof(uint64_t));
    if (!nk || !nv) { free(nk); free(nv); return 0; }
    for (uint64_t i = 0; i < oc; ++i) {
        if (!ok[i]) continue;
        uint64_t h = mix64(ok[i]) & (nc - 1);
        while (nk[h]) h = (h + 1) & (nc - 1);
        nk[h] = ok[i];
        nv[h] = ov[i];
    }
    free(ok);
    free(ov);
    m->k = nk;
    m->v = nv;
    m->mask = nc - 1;
    return 1;
}

static inline uint64_t map_slot(const orc_map *m, uint64_t key, int *found) {
    uint64_t h = mix64(key) & m->mask;
    while (m->k[h]) {
        if (m->k[h] == key) { *found = 1; return h; }
        h = (h + 1) & m->mask;
    }
    *found = 0;
    return h;
}

static void map_remove_at(orc_map *m, uint64_t h) {
    uint64_t i = h;
    for (;;) {
        uint64_t j = (i + 1) & m->mask;
        for (;;) {
            if (!m->k[j]) { m->k[i] = 0; m->v[i] = 0; m->n--; return; }
            uint64_t home = mix64(m->k[j]) & m->mask;
            /* move j back to i unless home lies cyclically in (i, j] */
            int keep = (i <= j) ? (i < home && home <= j) : (i < home || home <= j);
            if (!keep) break;
            j = (j + 1) & m->mask;
        }
        m->k[i] = m->k[j];
        m->v[i] = m->v[j];
        i = j;
    }
}

void orc_map_apply(orc_map *m, const uint8_t *ops, const uint64_t *k, const uint64_t *v,
                   uint64_t n, uint64_t *out_v, uint8_t *out_hit) {
    for (uint64_t i = 0; i < n; ++i) {
        uint64_t key = k[i];
        int found = 0;
        uint64_t h = key ? map_slot(m, key, &found) : 0;
        uint64_t rv = 0;
        uint8_t hit = 0;
        switch (ops[i]) {
        case 1: /* insert */
            if (!key) break;
            if (found) { /* the previous value comes back, as for erase */
                rv = m->v[h];
                m->v[h] = v[i];
                hit = 1;
            } else {
                if ((m->n + 1) * 2 > m->mask + 1) {
                    map_grow(m);
                    h = map_slot(m, key, &found);
                }
                m->k[h] = key;
                m->v[h] = v[i];
                m->n++;
            }
            break;
        case 2: /* erase */
            if (key && found) {
                rv = m->v[h];
                hit = 1;
                map_remove_at(m, h);
            }
            break;
        default: /* find */
            if (key && found) {
                rv = m->v[h];
                hit = 1;
            }
            break;
        }
        if (out_v) out_v[i] = rv;
        if (out_hit) out_hit[i] = hit;
    }
}

uint64_t orc_map_export(const orc_map *m, uint64_t *k, uint64_t *v) {
    uint64_t c = 0;
    for (uint64_t i = 0; i <= m->mask; ++i)
        if (m->k[i]) {
            k[c] = m->k[i];
            v[c] = m->v[i];
            ++c;
        }
    return c;
}
