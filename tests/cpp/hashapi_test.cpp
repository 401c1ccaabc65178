// hashapi_test.cpp -- the reference's gtest cases for hashAPI
// (GPU/dyhash/Main_backup_0910.cpp:208-411, GPU/warp/Main.cpp:530-611),
// written against include/dycuckoo_hashapi.hpp, with exact checks where the
// reference tolerates 2% mismatches (Main_backup_0910.cpp:25).
//
// Keys come from the oracle's restatement of the reference generator
// (MT19937 seeded 10327, GenerateUniqueRandomNumbers); the oracle is linked
// only as the input generator. Build and run: tests/test_cpp_hashapi.py.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <unordered_map>
#include <vector>

#include "dycuckoo_hashapi.hpp"

extern "C" {
#include "dyc_oracle.h"
}

using dycuckoo::hashAPI;
using dycuckoo::TYPE;

static int g_failed = 0;
static orc_mt g_mt;

#define EXPECT(cond, ...)                                     \
    do {                                                      \
        if (!(cond)) {                                        \
            std::printf("  expectation failed: " __VA_ARGS__); \
            std::printf("\n");                                \
            ok = false;                                       \
        }                                                     \
    } while (0)

static size_t mismatches(const TYPE *got, const TYPE *exp, size_t n) {
    size_t bad = 0;
    for (size_t i = 0; i < n; ++i) bad += got[i] != exp[i];
    return bad;
}

// HastTest.SizeTEST (Main_backup_0910.cpp:33-153, :208-217)
static bool size_test(TYPE size) {
    bool ok = true;
    std::vector<TYPE> key(2 * (size_t)size), value(2 * (size_t)size), chck(size, 0);
    orc_gen_unique_ref(&g_mt, key.data(), 2 * size, 0xfffffffeu);
    for (TYPE i = 0; i < 2 * size; ++i) value[i] = 3 * i + 3 + 1;
    hashAPI h((TYPE)(size * 1.1));
    h.hash_insert(key.data(), value.data(), size);
    h.hash_search(key.data(), chck.data(), size);
    EXPECT(mismatches(chck.data(), value.data(), size) == 0, "size %u: lookups differ", size);
    EXPECT(h.num_size() == size, "size %u: num_size %llu", size, (unsigned long long)h.num_size());
    // keys of the second half were never inserted
    std::vector<TYPE> miss(size, 1);
    h.hash_search(key.data() + size, miss.data(), size);
    EXPECT(std::count(miss.begin(), miss.end(), 0u) == (long)size, "size %u: false hits", size);
    return ok;
}

// HashBoundaryTest.InsertsameKeyValue (Main_backup_0910.cpp:236-275). The
// reference expects 2 for absent keys, the miss marker of its older lock
// variant; a miss here is 0, as in dyhash's hash_search (api.cpp:275).
static bool same_key_test() {
    bool ok = true;
    const int N = 100;
    std::vector<TYPE> key(N, 11), value(N, 9), search(N), chck(N, 0);
    for (int i = 0; i < N; ++i) search[i] = i;
    hashAPI h5(N);
    h5.hash_insert(key.data(), value.data(), N);
    h5.hash_search(search.data(), chck.data(), N);
    for (int i = 1; i < N; ++i) EXPECT(chck[i] == (i == 11 ? 9u : 0u), "key %d -> %u", i, chck[i]);
    h5.hash_search(key.data(), chck.data(), N);
    for (int i = 0; i < N; ++i) EXPECT(chck[i] == 9u, "repeat %d -> %u", i, chck[i]);
    EXPECT(h5.num_size() == 1, "one live key, got %llu", (unsigned long long)h5.num_size());
    return ok;
}

// HashBoundaryTest.RandTestKV (Main_backup_0910.cpp:278-313): keys may
// repeat; the last value of a repeated key wins.
static bool rand_kv_test() {
    bool ok = true;
    const int N = 100;
    std::vector<TYPE> key(N), value(N), chck(N, 0);
    uint32_t s = 12345;
    std::unordered_map<TYPE, TYPE> last;
    for (int i = 0; i < N; ++i) {
        s = s * 1103515245u + 12345u;
        key[i] = (s >> 8) % 1000000u + 1u;
        value[i] = i;
        last[key[i]] = value[i];
    }
    hashAPI h(N);
    h.hash_insert(key.data(), value.data(), N);
    h.hash_search(key.data(), chck.data(), N);
    for (int i = 0; i < N; ++i) EXPECT(chck[i] == last[key[i]], "key %u -> %u", key[i], chck[i]);
    return ok;
}

// HashResizeTest.RandTestWithUpDown (Main_backup_0910.cpp:321-411)
static bool resize_test(TYPE size) {
    bool ok = true;
    std::vector<TYPE> key(2 * (size_t)size), value(2 * (size_t)size), chck(size, 0);
    orc_gen_unique_ref(&g_mt, key.data(), 2 * size, 0xfffffffeu);
    for (TYPE i = 0; i < 2 * size; ++i) value[i] = 3 * i + 3 + 1;
    hashAPI h(size * 2);
    h.hash_insert(key.data(), value.data(), size);
    h.hash_search(key.data(), chck.data(), size);
    EXPECT(mismatches(chck.data(), value.data(), size) == 0, "before resize");
    for (int r = 0; r < 2; ++r) {
        h.resize_low();
        std::fill(chck.begin(), chck.end(), 0);
        h.hash_search(key.data(), chck.data(), size);
        EXPECT(mismatches(chck.data(), value.data(), size) == 0, "after resize_low %d", r);
    }
    for (int r = 0; r < 3; ++r) {
        h.resize_up();
        std::fill(chck.begin(), chck.end(), 0);
        h.hash_search(key.data(), chck.data(), size);
        EXPECT(mismatches(chck.data(), value.data(), size) == 0, "after resize_up %d", r);
    }
    EXPECT(h.num_size() == size, "num_size %llu", (unsigned long long)h.num_size());
    return ok;
}

// HashnewApiTest.test1 (GPU/warp/Main.cpp:530-611): the batch pool API,
// inserts and searches, then deletes, with the load-factor policy on.
static bool batch_api_test() {
    bool ok = true;
    const int nb = 40;
    const TYPE total = (TYPE)nb * dycuckoo::BATCH_SIZE;
    std::vector<TYPE> key(total), value(total), chck(total, 0);
    orc_gen_unique_ref(&g_mt, key.data(), total, 0xfffffffeu);
    for (TYPE i = 0; i < total; ++i) value[i] = i + 1;
    hashAPI h(dycuckoo::BATCH_SIZE);
    h.set_data_to_gpu(key.data(), value.data(), total);
    for (int i = 0; i < nb; ++i) {
        h.hash_insert_batch();
        h.hash_search_batch();
        EXPECT(h.num_size() <= dycuckoo::kUpperBound * h.table_size() + 1, "load above 0.8");
    }
    EXPECT(h.num_size() == total, "num_size %llu", (unsigned long long)h.num_size());
    h.hash_search(key.data(), chck.data(), total);
    EXPECT(mismatches(chck.data(), value.data(), total) == 0, "lookups after batch inserts");
    const uint64_t grown = h.table_size();
    for (int i = 0; i < nb; ++i) h.hash_delete_batch();
    EXPECT(h.num_size() == 0, "num_size after deletes %llu", (unsigned long long)h.num_size());
    EXPECT(h.table_size() < grown, "no downsize happened");
    std::fill(chck.begin(), chck.end(), 7);
    h.hash_search(key.data(), chck.data(), total);
    EXPECT(std::count(chck.begin(), chck.end(), 0u) == (long)total, "keys left after deletes");
    return ok;
}

static void run(const char *name, bool (*fn)()) {
    std::printf("[ RUN      ] %s\n", name);
    bool ok = false;
    try {
        ok = fn();
    } catch (const std::exception &e) {
        std::printf("  exception: %s\n", e.what());
    }
    std::printf(ok ? "[       OK ] %s\n" : "[  FAILED  ] %s\n", name);
    if (!ok) ++g_failed;
}

int main() {
    orc_mt_seed(&g_mt, 10327u);
    static const TYPE sizes[] = {100, 200, 1024, 2048, 4096, 1 << 12, 1 << 16, 1 << 20, 1 << 22};
    for (TYPE s : sizes) {
        char name[64];
        std::snprintf(name, sizeof(name), "HastTest.SizeTEST/%u", s);
        std::printf("[ RUN      ] %s\n", name);
        bool ok = false;
        try {
            ok = size_test(s);
        } catch (const std::exception &e) {
            std::printf("  exception: %s\n", e.what());
        }
        std::printf(ok ? "[       OK ] %s\n" : "[  FAILED  ] %s\n", name);
        if (!ok) ++g_failed;
    }
    run("HashBoundaryTest.InsertsameKeyValue", same_key_test);
    run("HashBoundaryTest.RandTestKV", rand_kv_test);
    run("HashResizeTest.RandTestWithUpDown", [] { return resize_test(1000000); });
    run("HashnewApiTest.test1", batch_api_test);
    std::printf(g_failed ? "%d test(s) FAILED\n" : "ALL PASSED\n", g_failed);
    return g_failed ? 1 : 0;
}
