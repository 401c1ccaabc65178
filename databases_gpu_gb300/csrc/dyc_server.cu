// dyc_server.cu -- the request server of include/dycuckoo.h (dyc_server_*):
// continuous batching of tenants' mixed-op requests over a table set.
//
// Pipeline (three threads, three staging slots of pinned host + device
// buffers, two copy streams):
//   assembler : takes admitted requests first-in first-out into a free slot
//               (up to max_step_ops), groups them by tenant keeping
//               submission order, copies their ops into pinned staging and
//               issues the host->device copies (upload stream)
//   executor  : runs the slot's step on the device (dyc_set_apply, or
//               dyc_apply per request without coalescing) once its upload is
//               done
//   completer : copies the step's results device->host (download stream),
//               hands every request its values and bits, frees the slot
// so one step's uploads and the previous step's downloads overlap the
// current step's kernels. Only this file's public calls touch the set.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <functional>

#include <cuda_runtime.h>

#include "dycuckoo.h"
#include "dyc_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

// Fixed pool of helper threads for the staging copies: run(n, f) calls f(i)
// for i in [0, n) on the helpers and the caller, and returns when all are done.
class CopyPool {
  public:
    explicit CopyPool(int helpers) {
        for (int i = 0; i < helpers; ++i) th_.emplace_back([this] { loop(); });
    }
    ~CopyPool() {
        {
            std::lock_guard<std::mutex> g(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &t : th_) t.join();
    }
    void run(uint64_t n, const std::function<void(uint64_t)> &f) {
        if (n == 0) return;
        {
            std::lock_guard<std::mutex> g(mu_);
            job_ = &f;
            n_ = n;
            next_ = 0;
            left_ = n;
            ++gen_;
        }
        cv_.notify_all();
        work();
        std::unique_lock<std::mutex> lk(mu_);
        done_.wait(lk, [&] { return left_ == 0; });
        job_ = nullptr;
    }

  private:
    void work() {
        for (;;) {
            uint64_t i;
            const std::function<void(uint64_t)> *f;
            {
                std::lock_guard<std::mutex> g(mu_);
                if (!job_ || next_ >= n_) return;
                i = next_++;
                f = job_;
            }
            (*f)(i);
            std::lock_guard<std::mutex> g(mu_);
            if (--left_ == 0) done_.notify_all();
        }
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return stop_ || (gen_ != seen && job_ && next_ < n_); });
                if (stop_) return;
                seen = gen_;
            }
            work();
        }
    }
    std::vector<std::thread> th_;
    std::mutex mu_;
    std::condition_variable cv_, done_;
    const std::function<void(uint64_t)> *job_ = nullptr;
    uint64_t n_ = 0, next_ = 0, left_ = 0, gen_ = 0;
    bool stop_ = false;
};

// Helper threads per copying stage (assembler, completer). Seven per stage
// oversubscribed the 16 host cores the server shares with its clients: at
// 1.72 G ops/s offered, request p50 ranged 0.9-5.9 ms and a client's own
// submissions ran up to 8 ms late; with three, p50 0.63-0.93 ms, clients at
// most 1.5 ms late, the same sustained rate.
constexpr int kCopyHelpers = 3;

struct Req {
    uint64_t ticket;
    uint32_t tenant;
    const uint8_t *ops;
    const void *keys;
    const void *vals;
    uint64_t n;
    void *out;
    uint32_t *bits;
    uint64_t growth;  // admission estimate, bytes
    Clock::time_point t_submit, t_done;
    dyc_status status = DYC_OK;
    bool done = false;
    bool deferred = false;
    uint64_t pos = 0;  // first op in its step's batch
};

struct Slot {
    uint8_t *h_ops = nullptr, *d_ops = nullptr;
    char *h_keys = nullptr, *h_vals = nullptr, *h_out = nullptr;
    char *d_keys = nullptr, *d_vals = nullptr, *d_out = nullptr;
    uint32_t *h_bits = nullptr, *d_bits = nullptr;
    uint32_t *h_off = nullptr, *d_off = nullptr;
    cudaEvent_t up = nullptr, down = nullptr;
    std::vector<Req *> reqs;
    uint64_t n = 0;
    dyc_status status = DYC_OK;
};

constexpr int kSlots = 3;

}  // namespace

struct dyc_server {
    dyc_server_config scfg;
    dyc_config tcfg;
    uint32_t ntenants = 0;
    int kb = 4, vb = 4, device = 0;
    size_t slot_bytes = 8;
    dyc_set *set = nullptr;
    std::vector<dyc_table *> members;
    Slot slot[kSlots];
    cudaStream_t up = nullptr, down = nullptr, exec = nullptr;

    std::mutex mu;
    std::condition_variable cv;  // every state change below
    std::deque<Req *> queue;
    std::unordered_map<uint64_t, Req *> live;
    std::deque<int> free_slots, to_exec, to_complete;
    uint64_t next_ticket = 1;
    bool stop = false, asm_done = false, exec_done = false;
    int in_flight = 0;        // slots between assembler and completer
    uint64_t completions = 0; // slots the completer has finished

    uint64_t fixed_bytes = 0, table_bytes = 0, pending_growth = 0;
    dyc_server_stats st{};
    CopyPool asm_pool{kCopyHelpers}, comp_pool{kCopyHelpers};
    std::thread t_asm, t_exec, t_comp;
};

namespace {

// Bits [pos, pos+n) of src into dst[0..ceil(n/32)).
void extract_bits(const uint32_t *src, uint64_t pos, uint64_t n, uint32_t *dst) {
    const uint64_t words = (n + 31) / 32;
    const uint64_t w0 = pos >> 5, sh = pos & 31;
    for (uint64_t j = 0; j < words; ++j) {
        uint64_t v = src[w0 + j] >> sh;
        if (sh && w0 + j + 1 <= (pos + n - 1) >> 5) v |= (uint64_t)src[w0 + j + 1] << (32 - sh);
        uint32_t x = (uint32_t)v;
        const uint64_t left = n - 32 * j;
        if (left < 32) x &= (1u << left) - 1u;
        dst[j] = x;
    }
}

uint64_t table_device_bytes(dyc_server *s) {
    std::vector<uint64_t> cap(s->ntenants);
    dyc_set_sizes(s->set, nullptr, cap.data());
    uint64_t slots = 0;
    for (uint64_t c : cap) slots += c;
    const uint64_t sb = s->tcfg.bucket_bytes;
    const uint64_t per_bucket = sb / s->slot_bytes - (sb == 128 ? 1 : 0);
    uint64_t spare = 0;  // upsize targets kept ahead by the set
    dyc_set_spare_bytes(s->set, &spare);
    return slots / per_bucket * sb + spare;
}

void finish_slot_error(dyc_server *s, Slot &sl, dyc_status err) {
    for (Req *r : sl.reqs) r->status = err;
}

void assembler(dyc_server *s) {
    cudaSetDevice(s->device);
    const uint64_t cap = s->scfg.hbm_cap_bytes;
    for (;;) {
        std::unique_lock<std::mutex> lk(s->mu);
        s->cv.wait(lk, [&] { return (s->stop && s->queue.empty()) ||
                                    (!s->queue.empty() && !s->free_slots.empty()); });
        if (s->queue.empty()) break;  // stop requested and drained
        // admission, first-in first-out
        std::vector<Req *> take;
        uint64_t n = 0;
        const uint64_t room = s->scfg.coalesce ? s->scfg.max_step_ops : 0;
        while (!s->queue.empty()) {
            Req *r = s->queue.front();
            if (!take.empty() && (n + r->n > room)) break;
            if (cap && s->fixed_bytes + s->table_bytes + s->pending_growth + r->growth > cap) {
                if (take.empty() && s->in_flight == 0) {
                    // nothing else holds memory: it can never be admitted
                    s->queue.pop_front();
                    r->status = DYC_ENOMEM;
                    r->done = true;
                    r->t_done = Clock::now();
                    s->st.rejected++;
                    s->st.requests++;
                    continue;
                }
                if (!r->deferred) {
                    r->deferred = true;
                    s->st.deferred++;
                }
                break;  // wait for running steps to free memory
            }
            s->queue.pop_front();
            s->pending_growth += r->growth;
            take.push_back(r);
            n += r->n;
            if (!s->scfg.coalesce) break;  // one request per step
        }
        if (take.empty()) {
            s->cv.notify_all();  // rejections
            // deferred: wait until a running step finishes and frees memory
            const uint64_t seen = s->completions;
            s->cv.wait(lk, [&] { return s->in_flight == 0 || s->completions != seen; });
            continue;
        }
        const int b = s->free_slots.front();
        s->free_slots.pop_front();
        s->in_flight++;
        lk.unlock();
        const auto ta = Clock::now();

        Slot &sl = s->slot[b];
        sl.reqs = take;
        sl.n = n;
        sl.status = DYC_OK;
        // group by tenant, submission order inside a tenant
        std::vector<uint64_t> cnt(s->ntenants + 1, 0);
        for (Req *r : take) cnt[r->tenant + 1] += r->n;
        for (uint32_t t = 0; t < s->ntenants; ++t) cnt[t + 1] += cnt[t];
        for (uint32_t t = 0; t <= s->ntenants; ++t) sl.h_off[t] = (uint32_t)cnt[t];
        for (Req *r : take) {
            r->pos = s->scfg.coalesce ? cnt[r->tenant] : 0;
            if (s->scfg.coalesce) cnt[r->tenant] += r->n;
        }
        s->asm_pool.run(take.size(), [&](uint64_t i) {
            const Req *r = take[i];
            memcpy(sl.h_ops + r->pos, r->ops, r->n);
            memcpy(sl.h_keys + r->pos * s->kb, r->keys, r->n * s->kb);
            memcpy(sl.h_vals + r->pos * s->vb, r->vals, r->n * s->vb);
        });
        cudaError_t e = cudaMemcpyAsync(sl.d_ops, sl.h_ops, n, cudaMemcpyHostToDevice, s->up);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(sl.d_keys, sl.h_keys, n * s->kb, cudaMemcpyHostToDevice, s->up);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(sl.d_vals, sl.h_vals, n * s->vb, cudaMemcpyHostToDevice, s->up);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(sl.d_off, sl.h_off, (s->ntenants + 1) * sizeof(uint32_t),
                                cudaMemcpyHostToDevice, s->up);
        if (e == cudaSuccess) e = cudaEventRecord(sl.up, s->up);
        if (e != cudaSuccess) sl.status = DYC_ECUDA;
        const double asm_s = std::chrono::duration<double>(Clock::now() - ta).count();
        lk.lock();
        s->st.assemble_seconds += asm_s;
        s->to_exec.push_back(b);
        s->cv.notify_all();
    }
    std::lock_guard<std::mutex> g(s->mu);
    s->asm_done = true;
    s->cv.notify_all();
}

void executor(dyc_server *s) {
    cudaSetDevice(s->device);
    for (;;) {
        int b;
        const auto tw = Clock::now();
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv.wait(lk, [&] { return !s->to_exec.empty() || s->asm_done; });
            if (s->to_exec.empty()) break;
            b = s->to_exec.front();
            s->to_exec.pop_front();
        }
        Slot &sl = s->slot[b];
        const auto t0 = Clock::now();
        const double idle = std::chrono::duration<double>(t0 - tw).count();
        const bool late = cudaEventQuery(sl.up) == cudaErrorNotReady;
        dyc_status r = sl.status;
        if (r == DYC_OK && cudaStreamWaitEvent(s->exec, sl.up, 0) != cudaSuccess) r = DYC_ECUDA;
        if (r == DYC_OK && s->scfg.coalesce) {
            // each staging slot's buffers get their own captured launch graph
            r = dyc_set_apply(s->set, sl.d_off, sl.h_off, sl.d_ops, sl.d_keys, sl.d_vals,
                              sl.d_out, sl.d_bits, DYC_FLAG_GRAPH, s->exec);
        } else if (r == DYC_OK) {
            Req *q = sl.reqs[0];
            r = dyc_apply(s->members[q->tenant], sl.d_ops, sl.d_keys, sl.d_vals, q->n, sl.d_out,
                          sl.d_bits, 0, s->exec);
        }
        if (r == DYC_OK && cudaStreamSynchronize(s->exec) != cudaSuccess) r = DYC_ECUDA;
        const double busy = std::chrono::duration<double>(Clock::now() - t0).count();
        dyc_op_stats os{};
        if (r == DYC_OK) {
            if (s->scfg.coalesce) dyc_set_last_stats(s->set, &os);
            else dyc_last_stats(s->members[sl.reqs[0]->tenant], &os);
        }
        const uint64_t tb = r == DYC_OK ? table_device_bytes(s) : 0;
        sl.status = r;  // the completer downloads the results (the step has finished)
        std::lock_guard<std::mutex> g(s->mu);
        if (r == DYC_OK) s->table_bytes = tb;
        s->st.steps++;
        s->st.busy_seconds += busy;
        if (s->st.steps > 1) s->st.exec_idle_seconds += idle;  // not the wait for the first
        s->st.upload_late_steps += late ? 1 : 0;
        s->st.split_steps += os.split_phases;
        s->st.resizes_up += os.resizes_up;
        s->st.resizes_down += os.resizes_down;
        if (os.resizes_up || os.resizes_down) s->st.resize_step_seconds += busy;
        s->st.max_step_ops = std::max(s->st.max_step_ops, sl.n);
        s->to_complete.push_back(b);
        s->cv.notify_all();
    }
    std::lock_guard<std::mutex> g(s->mu);
    s->exec_done = true;
    s->cv.notify_all();
}

void completer(dyc_server *s) {
    cudaSetDevice(s->device);
    for (;;) {
        int b;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv.wait(lk, [&] { return !s->to_complete.empty() || s->exec_done; });
            if (s->to_complete.empty()) break;
            b = s->to_complete.front();
            s->to_complete.pop_front();
        }
        Slot &sl = s->slot[b];
        if (sl.status == DYC_OK) {
            cudaError_t e = cudaMemcpyAsync(sl.h_out, sl.d_out, sl.n * s->vb,
                                            cudaMemcpyDeviceToHost, s->down);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(sl.h_bits, sl.d_bits, (sl.n + 31) / 32 * 4,
                                    cudaMemcpyDeviceToHost, s->down);
            if (e == cudaSuccess) e = cudaEventRecord(sl.down, s->down);
            if (e == cudaSuccess) e = cudaEventSynchronize(sl.down);
            if (e != cudaSuccess) sl.status = DYC_ECUDA;
        }
        if (sl.status != DYC_OK) {
            finish_slot_error(s, sl, sl.status);
        } else {
            s->comp_pool.run(sl.reqs.size(), [&](uint64_t i) {
                const Req *r = sl.reqs[i];
                if (r->out) memcpy(r->out, sl.h_out + r->pos * s->vb, r->n * s->vb);
                if (r->bits) extract_bits(sl.h_bits, r->pos, r->n, r->bits);
            });
        }
        const auto now = Clock::now();
        std::lock_guard<std::mutex> g(s->mu);
        for (Req *r : sl.reqs) {
            r->done = true;
            r->t_done = now;
            s->pending_growth -= r->growth;
            s->st.requests++;
            s->st.ops += r->n;
        }
        sl.reqs.clear();
        s->free_slots.push_back(b);
        s->in_flight--;
        s->completions++;
        s->cv.notify_all();
    }
}

dyc_status free_server(dyc_server *s) {
    if (!s) return DYC_OK;
    cudaSetDevice(s->device);
    for (Slot &sl : s->slot) {
        if (sl.h_ops) cudaFreeHost(sl.h_ops);
        if (sl.d_ops) cudaFree(sl.d_ops);
        if (sl.up) cudaEventDestroy(sl.up);
        if (sl.down) cudaEventDestroy(sl.down);
    }
    if (s->up) cudaStreamDestroy(s->up);
    if (s->down) cudaStreamDestroy(s->down);
    if (s->exec) cudaStreamDestroy(s->exec);
    if (s->set) dyc_set_destroy(s->set);
    for (auto &kv : s->live) delete kv.second;  // queued requests are live too
    delete s;
    return DYC_OK;
}

}  // namespace

extern "C" {

void dyc_server_config_default(dyc_server_config *c) {
    if (!c) return;
    memset(c, 0, sizeof(*c));
    c->max_step_ops = 1ull << 22;
    c->coalesce = 1;
    c->pool_reserve_bytes = DYC_POOL_RESERVE_AUTO;
}

dyc_status dyc_server_create(const dyc_config *table_cfg, uint32_t ntenants,
                             const uint64_t *sizes, const dyc_server_config *cfg,
                             dyc_server **out) {
    if (!table_cfg || !sizes || !out || ntenants == 0) return DYC_EINVAL;
    *out = nullptr;
    dyc_server *s = new (std::nothrow) dyc_server();
    if (!s) return DYC_ENOMEM;
    if (cfg) s->scfg = *cfg;
    else dyc_server_config_default(&s->scfg);
    if (s->scfg.max_step_ops == 0) s->scfg.max_step_ops = 1ull << 22;
    if (s->scfg.max_step_ops >= (1ull << 31)) {
        delete s;
        return DYC_EINVAL;
    }
    s->tcfg = *table_cfg;
    s->ntenants = ntenants;
    s->kb = (int)table_cfg->key_bytes;
    s->vb = (int)table_cfg->value_bytes;
    s->device = table_cfg->device;
    s->slot_bytes = s->kb == 4 ? 8 : 16;
    dyc_status r = dyc_set_create(table_cfg, ntenants, sizes, nullptr, &s->set);
    if (r != DYC_OK) {
        free_server(s);
        return r;
    }
    s->members.resize(ntenants);
    for (uint32_t t = 0; t < ntenants; ++t) dyc_set_table(s->set, t, &s->members[t]);
    const uint64_t m = s->scfg.max_step_ops;
    // one block per slot side: ops, keys, vals, out, bits, offsets
    auto al = [](uint64_t x) { return (x + 255) & ~(uint64_t)255; };
    const uint64_t o_keys = al(m), o_vals = o_keys + al(m * s->kb), o_out = o_vals + al(m * s->vb),
                   o_bits = o_out + al(m * s->vb), o_off = o_bits + al((m / 32 + 1) * 4),
                   bytes = o_off + al((uint64_t)(ntenants + 1) * 4);
    cudaError_t e = cudaSetDevice(s->device);
    for (int i = 0; i < kSlots && e == cudaSuccess; ++i) {
        Slot &sl = s->slot[i];
        void *h = nullptr, *d = nullptr;
        e = dyc::lib_malloc_host(&h, bytes);
        if (e == cudaSuccess) e = dyc::lib_malloc(&d, bytes);
        if (e != cudaSuccess) {
            if (h) cudaFreeHost(h);
            break;
        }
        char *hc = (char *)h, *dc = (char *)d;
        sl.h_ops = (uint8_t *)hc;
        sl.d_ops = (uint8_t *)dc;
        sl.h_keys = hc + o_keys;
        sl.d_keys = dc + o_keys;
        sl.h_vals = hc + o_vals;
        sl.d_vals = dc + o_vals;
        sl.h_out = hc + o_out;
        sl.d_out = dc + o_out;
        sl.h_bits = (uint32_t *)(hc + o_bits);
        sl.d_bits = (uint32_t *)(dc + o_bits);
        sl.h_off = (uint32_t *)(hc + o_off);
        sl.d_off = (uint32_t *)(dc + o_off);
        e = cudaEventCreateWithFlags(&sl.up, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.down, cudaEventDisableTiming);
        s->free_slots.push_back(i);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->up, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->down, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->exec, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        free_server(s);
        return e == cudaErrorMemoryAllocation ? DYC_ENOMEM : DYC_ECUDA;
    }
    // staging plus the set's batch scratch (about 160 bytes an op at this
    // step size) count against the cap from the start
    s->fixed_bytes = kSlots * bytes + m * 160;
    s->table_bytes = table_device_bytes(s);
    // replaced subtables the set keeps for reuse count against the cap: at
    // most an eighth of the headroom goes to them
    if (s->scfg.hbm_cap_bytes) {
        const uint64_t used = s->fixed_bytes + s->table_bytes;
        const uint64_t head = s->scfg.hbm_cap_bytes > used ? s->scfg.hbm_cap_bytes - used : 0;
        r = dyc_set_spare_cache(s->set, std::min<uint64_t>(head / 8, s->table_bytes / 4));
        if (r != DYC_OK) {
            free_server(s);
            return r;
        }
    }
    // growth headroom mapped into the allocation pool now rather than by the
    // first resizes inside steps
    uint64_t reserve = s->scfg.pool_reserve_bytes;
    if (reserve == DYC_POOL_RESERVE_AUTO) {
        reserve = 2 * s->table_bytes;
        const uint64_t used = s->fixed_bytes + s->table_bytes;
        if (s->scfg.hbm_cap_bytes)
            reserve = std::min<uint64_t>(
                reserve, s->scfg.hbm_cap_bytes > used ? s->scfg.hbm_cap_bytes - used : 0);
    }
    if (reserve) {
        r = dyc_pool_reserve(s->device, reserve);
        if (r != DYC_OK && r != DYC_ENOMEM) {  // a reserve that does not fit is only skipped
            free_server(s);
            return r;
        }
    }
    s->t_comp = std::thread(completer, s);
    s->t_exec = std::thread(executor, s);
    s->t_asm = std::thread(assembler, s);
    *out = s;
    return DYC_OK;
}

dyc_status dyc_server_destroy(dyc_server *s) {
    if (!s) return DYC_OK;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
        s->cv.notify_all();
    }
    s->t_asm.join();
    s->t_exec.join();
    s->t_comp.join();
    return free_server(s);
}

dyc_status dyc_server_submit(dyc_server *s, uint32_t tenant, const uint8_t *h_ops,
                             const void *h_keys, const void *h_vals, uint64_t n,
                             void *h_vals_out, uint32_t *h_bits_out, uint64_t *ticket) {
    if (!s || !ticket || tenant >= s->ntenants) return DYC_EINVAL;
    if (n == 0 || n > s->scfg.max_step_ops || !h_ops || !h_keys || !h_vals) return DYC_EINVAL;
    Req *r = new (std::nothrow) Req();
    if (!r) return DYC_ENOMEM;
    uint64_t ins = 0;
    for (uint64_t i = 0; i < n; ++i) ins += h_ops[i] == DYC_OP_INSERT;
    r->tenant = tenant;
    r->ops = h_ops;
    r->keys = h_keys;
    r->vals = h_vals;
    r->n = n;
    r->out = h_vals_out;
    r->bits = h_bits_out;
    // every insert may add a slot at the upper load bound, and a resize holds
    // the old and the doubled subtable at once
    r->growth = (uint64_t)((double)(ins * s->slot_bytes) * 2.0 / s->tcfg.upper_load);
    r->t_submit = Clock::now();
    std::lock_guard<std::mutex> g(s->mu);
    if (s->stop) {
        delete r;
        return DYC_EINVAL;
    }
    r->ticket = s->next_ticket++;
    s->live[r->ticket] = r;
    s->queue.push_back(r);
    *ticket = r->ticket;
    s->cv.notify_all();
    return DYC_OK;
}

dyc_status dyc_server_wait(dyc_server *s, uint64_t ticket, int64_t timeout_ms,
                           dyc_status *req_status, uint64_t *latency_ns) {
    if (!s) return DYC_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->live.find(ticket);
    if (it == s->live.end()) return DYC_EINVAL;
    Req *r = it->second;
    auto ready = [&] { return r->done; };
    if (timeout_ms < 0) s->cv.wait(lk, ready);
    else if (!s->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) return DYC_ETIMEOUT;
    if (req_status) *req_status = r->status;
    if (latency_ns)
        *latency_ns = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
                          r->t_done - r->t_submit).count();
    s->live.erase(it);
    delete r;
    return DYC_OK;
}

dyc_status dyc_server_stats_get(dyc_server *s, dyc_server_stats *out) {
    if (!s || !out) return DYC_EINVAL;
    std::lock_guard<std::mutex> g(s->mu);
    *out = s->st;
    out->device_bytes = s->fixed_bytes + s->table_bytes;
    return DYC_OK;
}

dyc_status dyc_server_set(dyc_server *s, dyc_set **out) {
    if (!s || !out) return DYC_EINVAL;
    *out = s->set;
    return DYC_OK;
}

}  // extern "C"
