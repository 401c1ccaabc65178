// dyc_serve_load.cpp -- open-loop load generator for the request server
// (not part of libdycuckoo.so; built and run by `python bench.py`).
//
// Tenant tables: u64 keys / u32 values, initial sizes log-uniform in
// [2^lo, 2^hi] keys, preloaded with keys splitmix64(j + 1), j < size.
// Requests arrive as a Poisson process at `rate` per second; each picks a
// tenant by Zipf(s) rank, a size log-uniform in [2^bmin, 2^bmax] ops and a
// slice of a pre-generated op pool (70% find on j < 2^17, 20% insert on
// j < 2^25, 10% erase on j < 2^17). The generator submits each request at its
// arrival time (or as soon as it can when behind) and a second thread waits
// for completions. Latency = completion - scheduled arrival. Prints one JSON
// line.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "dycuckoo.h"

namespace {

using Clock = std::chrono::steady_clock;

uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

uint64_t key_of(uint64_t j) {
    const uint64_t k = splitmix64(j + 1);
    return k ? k : 1;  // never 0 (splitmix64 is a bijection; at most one j maps to 0)
}

double arg(int argc, char **argv, const char *name, double def) {
    for (int i = 1; i + 1 < argc; ++i)
        if (!strcmp(argv[i], name)) return atof(argv[i + 1]);
    return def;
}

}  // namespace

int main(int argc, char **argv) {
    const int tenants = (int)arg(argc, argv, "--tenants", 64);
    const int lo = (int)arg(argc, argv, "--log2-size-min", 16);
    const int hi = (int)arg(argc, argv, "--log2-size-max", 24);
    const double rate = arg(argc, argv, "--rate", 2e5);
    const double seconds = arg(argc, argv, "--seconds", 0.25);
    const int bmin = (int)arg(argc, argv, "--log2-batch-min", 5);
    const int bmax = (int)arg(argc, argv, "--log2-batch-max", 16);
    const double zipf_s = arg(argc, argv, "--zipf", 0.9);
    const double cap_gb = arg(argc, argv, "--cap-gb", 120);
    const int coalesce = (int)arg(argc, argv, "--coalesce", 1);
    const uint64_t max_step = (uint64_t)arg(argc, argv, "--max-step-ops", 1 << 22);
    const int pool_log2 = (int)arg(argc, argv, "--pool-log2", 24);
    const uint64_t seed = (uint64_t)arg(argc, argv, "--seed", 10327);
    const int device_upsize = (int)arg(argc, argv, "--device-upsize", 0);
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> U(0.0, 1.0);

    // ---- tenants
    std::vector<uint64_t> sizes(tenants);
    for (auto &s : sizes) s = (uint64_t)std::llround(std::pow(2.0, lo + U(rng) * (hi - lo)));
    dyc_config cfg;
    dyc_config_default(&cfg);
    cfg.key_bytes = 8;
    cfg.value_bytes = 4;
    cfg.device_upsize = (uint32_t)device_upsize;
    dyc_server_config scfg;
    dyc_server_config_default(&scfg);
    scfg.hbm_cap_bytes = (uint64_t)(cap_gb * 1e9);
    scfg.coalesce = (uint32_t)coalesce;
    scfg.max_step_ops = max_step;
    dyc_server *srv = nullptr;
    const auto tc0 = Clock::now();
    if (dyc_server_create(&cfg, tenants, sizes.data(), &scfg, &srv) != DYC_OK) {
        fprintf(stderr, "dyc_server_create: %s\n", dyc_last_error());
        return 1;
    }
    dyc_set *set = nullptr;
    dyc_server_set(srv, &set);
    uint64_t total_keys = 0;
    {
        const uint64_t mx = *std::max_element(sizes.begin(), sizes.end());
        std::vector<uint64_t> k(mx);
        std::vector<uint32_t> v(mx);
        for (int t = 0; t < tenants; ++t) {
            for (uint64_t j = 0; j < sizes[t]; ++j) {
                k[j] = key_of(j);
                v[j] = (uint32_t)j;
            }
            dyc_table *m = nullptr;
            dyc_set_table(set, t, &m);
            if (dyc_insert_host(m, k.data(), v.data(), sizes[t],
                                DYC_FLAG_UNIQUE | DYC_FLAG_NEW_KEYS) != DYC_OK) {
                fprintf(stderr, "preload: %s\n", dyc_last_error());
                return 1;
            }
            total_keys += sizes[t];
        }
    }
    const double setup_s = std::chrono::duration<double>(Clock::now() - tc0).count();

    // ---- op pool
    const uint64_t P = 1ull << pool_log2;
    std::vector<uint8_t> pops(P);
    std::vector<uint64_t> pkeys(P);
    std::vector<uint32_t> pvals(P);
    for (uint64_t i = 0; i < P; ++i) {
        const double u = U(rng);
        const uint8_t op = u < 0.7 ? DYC_OP_FIND : (u < 0.9 ? DYC_OP_INSERT : DYC_OP_ERASE);
        const uint64_t range = op == DYC_OP_INSERT ? (1ull << 25) : (1ull << 17);
        pops[i] = op;
        pkeys[i] = key_of(rng() % range);
        pvals[i] = (uint32_t)rng();
    }

    // ---- schedule
    std::vector<double> zcdf(tenants);
    double acc = 0;
    for (int r = 0; r < tenants; ++r) zcdf[r] = (acc += 1.0 / std::pow(r + 1.0, zipf_s));
    for (auto &c : zcdf) c /= acc;
    const uint64_t N = (uint64_t)std::max(1.0, rate * seconds);
    std::vector<double> at(N);
    std::vector<uint32_t> ten(N);
    std::vector<uint64_t> len(N), off(N), out_off(N);
    std::exponential_distribution<double> gap(rate);
    double t = 0;
    uint64_t total_ops = 0;
    for (uint64_t i = 0; i < N; ++i) {
        t += gap(rng);
        at[i] = t;
        ten[i] = (uint32_t)(std::lower_bound(zcdf.begin(), zcdf.end(), U(rng)) - zcdf.begin());
        if (ten[i] >= (uint32_t)tenants) ten[i] = tenants - 1;
        len[i] = (uint64_t)std::llround(std::pow(2.0, bmin + U(rng) * (bmax - bmin)));
        off[i] = rng() % (P - len[i]);
        out_off[i] = total_ops;
        total_ops += len[i];
    }
    std::vector<uint32_t> outv(total_ops);
    std::vector<uint32_t> outb(total_ops / 32 + N + 1);
    memset(outv.data(), 0, outv.size() * 4);
    memset(outb.data(), 0, outb.size() * 4);
    std::vector<uint64_t> bits_off(N);
    {
        uint64_t b = 0;
        for (uint64_t i = 0; i < N; ++i) {
            bits_off[i] = b;
            b += (len[i] + 31) / 32;
        }
    }

    // ---- run
    std::vector<uint64_t> ticket(N);
    std::vector<double> late(N), lat(N);
    std::atomic<uint64_t> published{0};
    std::atomic<int> failures{0};
    const auto t0 = Clock::now() + std::chrono::milliseconds(20);
    std::thread waiter([&] {
        for (uint64_t i = 0; i < N; ++i) {
            while (published.load(std::memory_order_acquire) <= i) std::this_thread::yield();
            dyc_status st = DYC_OK;
            uint64_t ns = 0;
            if (dyc_server_wait(srv, ticket[i], -1, &st, &ns) != DYC_OK || st != DYC_OK)
                failures++;
            lat[i] = late[i] + ns * 1e-9;
        }
    });
    for (uint64_t i = 0; i < N; ++i) {
        const auto due = t0 + std::chrono::duration_cast<Clock::duration>(
                                  std::chrono::duration<double>(at[i]));
        std::this_thread::sleep_until(due);
        const auto now = Clock::now();
        late[i] = std::chrono::duration<double>(now - due).count();
        if (dyc_server_submit(srv, ten[i], pops.data() + off[i], pkeys.data() + off[i],
                              pvals.data() + off[i], len[i], outv.data() + out_off[i],
                              outb.data() + bits_off[i], &ticket[i]) != DYC_OK) {
            fprintf(stderr, "submit: %s\n", dyc_last_error());
            return 1;
        }
        published.store(i + 1, std::memory_order_release);
    }
    waiter.join();
    const double wall = std::chrono::duration<double>(Clock::now() - t0).count();
    dyc_server_stats st;
    dyc_server_stats_get(srv, &st);
    double last_done = 0;
    for (uint64_t i = 0; i < N; ++i) last_done = std::max(last_done, at[i] + lat[i]);
    std::vector<double> sl = lat;
    std::sort(sl.begin(), sl.end());
    auto pct = [&](double p) { return sl[std::min<uint64_t>(N - 1, (uint64_t)(p * N))] * 1e3; };
    double late_max = *std::max_element(late.begin(), late.end());
    printf("{\"requests\": %llu, \"ops\": %llu, \"rate_per_s\": %.0f, \"arrival_span_s\": %.4f, "
           "\"offered_mops\": %.1f, \"sustained_mops\": %.1f, \"p50_ms\": %.3f, \"p99_ms\": %.3f, "
           "\"max_ms\": %.3f, \"submit_late_max_ms\": %.3f, \"steps\": %llu, "
           "\"max_step_ops\": %llu, \"deferred\": %llu, \"rejected\": %llu, \"failures\": %d, "
           "\"executor_busy_frac\": %.3f, \"device_bytes\": %llu, \"tenants\": %d, "
           "\"keys_preloaded\": %llu, \"setup_s\": %.2f, \"coalesce\": %d, \"wall_s\": %.3f, "
           "\"resizes_up\": %llu, \"resizes_down\": %llu, \"resize_step_busy_frac\": %.3f, "
           "\"assemble_frac\": %.3f, \"exec_idle_frac\": %.3f, \"upload_late_steps\": %llu, "
           "\"split_steps\": %llu}\n",
           (unsigned long long)N, (unsigned long long)total_ops, rate, at[N - 1],
           total_ops / at[N - 1] / 1e6, total_ops / last_done / 1e6, pct(0.5), pct(0.99),
           sl[N - 1] * 1e3, late_max * 1e3, (unsigned long long)st.steps,
           (unsigned long long)st.max_step_ops, (unsigned long long)st.deferred,
           (unsigned long long)st.rejected, failures.load(), st.busy_seconds / last_done,
           (unsigned long long)st.device_bytes, tenants, (unsigned long long)total_keys, setup_s,
           coalesce, wall, (unsigned long long)st.resizes_up, (unsigned long long)st.resizes_down,
           st.busy_seconds > 0 ? st.resize_step_seconds / st.busy_seconds : 0.0,
           st.assemble_seconds / last_done, st.exec_idle_seconds / last_done,
           (unsigned long long)st.upload_late_steps, (unsigned long long)st.split_steps);
    dyc_server_destroy(srv);
    return failures.load() ? 2 : 0;
}
