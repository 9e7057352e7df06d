// Serving form: a request loop with continuous admission over the register engine.
//
// A request is one register's life in qvnt terms: `QReg::with_state(n, state)`
// (src/register/quant.rs:113-150), then 1..k calls, each an `apply` of the next slice of its gate list
// (quant.rs:376-395) or a `measure_mask(mask)` with an injected draw (quant.rs:490-501), on a state
// that stays resident in HBM between the calls.
//
// `slots` worker threads each run one request at a time on the request's own CUDA stream, so the
// kernels of different requests overlap on the device.  A worker that frees up admits, among the
// queued requests whose state fits the HBM budget next to the running ones, the one with the least
// estimated work discounted by its waiting time (shortest first, with ageing); requests of 24 qubits
// or more may hold at most a quarter of the slots.
// Registers are pooled by size and reused through `qvnt_reg_reset`, so steady-state admission
// allocates nothing and never hits the device-wide synchronisation of cudaFree; idle pooled
// registers are freed only when a new size needs their memory.  Streams of small registers get the
// higher stream priority, and every server register launches one CTA per tile (not a persistent
// grid), so the blocks of small requests overtake the long passes of large ones at tile granularity.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "engine.h"

namespace {

using Clock = std::chrono::steady_clock;

constexpr uint32_t kMagicServer = 0x51535256u;
constexpr double kAgeScale = 1.0;  // seconds: waiting time that discounts a request's work by e
// Requests whose state is at least kLargeBytes are "large": at most a quarter of the slots (and at
// most 8) run them at once, so that long requests cannot hold every slot while short ones queue.
constexpr uint64_t kLargeBytes = 16ull << 24;  // a 24-qubit state

struct Request {
    uint64_t id = 0;
    uint32_t n = 0;
    uint64_t state = 0;
    std::vector<qvnt_gate> gates;
    std::vector<qvnt_call> calls;
    double arrival = 0.0;
    bool keep_amplitudes = false;
    bool detached = false;
    uint64_t footprint = 0;
    double work = 0.0;  // amplitudes x gates (+ amplitudes per measurement)
    // results
    int status = QVNT_OK;
    std::string error;
    std::vector<uint64_t> results;
    std::vector<double> amplitudes;
    double latency = 0.0;
    bool done = false;
};

uint64_t reg_bytes(uint32_t n) {
    const uint64_t len = n < 3 ? 8 : (1ull << n);
    return len * 16 + (1ull << 20);  // state + reduction scratch and small buffers
}

}  // namespace

struct qvnt_server {
    uint32_t magic = 0;
    qvnt_ctx* ctx = nullptr;
    uint64_t budget = 0;
    uint32_t slots = 0;
    uint32_t max_queue = 0;
    Clock::time_point t0;
    int prio_least = 0, prio_greatest = 0;

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    std::deque<Request*> queue;
    std::unordered_map<uint64_t, Request*> requests;  // submitted, not yet released
    uint64_t next_id = 1;
    // memory: bytes of running requests' registers + bytes of idle pooled registers
    uint64_t bytes_active = 0, bytes_idle = 0;
    std::multimap<uint32_t, std::pair<qvnt_reg*, uint64_t>> idle;  // pooled registers (bytes) by qubit count
    std::vector<qvnt_reg*> to_free;
    // statistics
    uint64_t submitted = 0, shed = 0, completed = 0, failed = 0, running = 0, peak_running = 0;
    uint64_t large_running = 0;
    std::vector<double> latencies;
    std::vector<std::thread> workers;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

int priority_for(const qvnt_server* s, uint32_t n) {
    if (n <= 16) return s->prio_greatest;
    if (n <= 22) return (s->prio_greatest + s->prio_least) / 2;
    return s->prio_least;
}

// Picks the request to admit (caller holds the lock): among the queued requests whose state fits
// next to the running ones, the least estimated work (amplitudes x gates) discounted by waiting time,
// work * exp(-age / kAgeScale): short requests go first, and a long one overtakes a fresh short one
// after waiting about kAgeScale * ln(work ratio).  Returns queue.end() when none fits.
std::deque<Request*>::iterator pick(qvnt_server* s) {
    const double t = s->now();
    const uint64_t max_large = std::max<uint64_t>(1, std::min<uint64_t>(8, s->slots / 4));
    auto best = s->queue.end();
    double best_score = 0.0;
    for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
        // idle pooled registers are reused or evicted, so only running requests hold memory
        if (s->bytes_active + (*it)->footprint > s->budget) continue;
        if ((*it)->footprint >= kLargeBytes && s->large_running >= max_large) continue;
        const double score = (*it)->work * std::exp(-(t - (*it)->arrival) / kAgeScale);
        if (best == s->queue.end() || score < best_score) {
            best = it;
            best_score = score;
        }
    }
    return best;
}

int run_request(Request* r, qvnt_reg* reg) {
    int st = QVNT_OK;
    size_t g0 = 0;
    r->results.assign(r->calls.size(), 0);
    for (size_t c = 0; c < r->calls.size() && !st; ++c) {
        const qvnt_call& call = r->calls[c];
        if (call.op == QVNT_CALL_APPLY) {
            st = qvnt_reg_apply(reg, r->gates.data() + g0, (size_t)call.gate_count);
            g0 += call.gate_count;
        } else {
            uint64_t v = 0;
            st = qvnt_reg_measure_mask(reg, call.mask, call.u01, &v);
            r->results[c] = v;
        }
    }
    if (!st && r->keep_amplitudes) {
        r->amplitudes.resize(2 * (r->n < 3 ? 8 : (1ull << r->n)));
        st = qvnt_reg_get_amplitudes(reg, r->amplitudes.data());
    }
    if (!st) st = qvnt_reg_sync(reg);
    return st;
}

void worker(qvnt_server* s) {
    cudaSetDevice(s->ctx->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        std::deque<Request*>::iterator it;
        s->cv_work.wait(lk, [&] { return s->stop || (!s->queue.empty() && (it = pick(s)) != s->queue.end()); });
        if (s->stop) break;
        Request* r = *it;
        s->queue.erase(it);
        // a pooled register of this size, or fresh memory (evicting idle registers of other sizes)
        qvnt_reg* reg = nullptr;
        auto pooled = s->idle.find(r->n);
        if (pooled != s->idle.end()) {
            reg = pooled->second.first;
            s->bytes_idle -= pooled->second.second;
            r->footprint = std::max(r->footprint, pooled->second.second);
            s->idle.erase(pooled);
        } else {
            while (s->bytes_active + s->bytes_idle + r->footprint > s->budget && !s->idle.empty()) {
                auto victim = std::prev(s->idle.end());  // the widest idle register
                s->bytes_idle -= victim->second.second;
                s->to_free.push_back(victim->second.first);
                s->idle.erase(victim);
            }
        }
        s->bytes_active += r->footprint;
        s->running += 1;
        const bool large = r->footprint >= kLargeBytes;
        if (large) s->large_running += 1;
        s->peak_running = std::max(s->peak_running, s->running);
        std::vector<qvnt_reg*> frees;
        frees.swap(s->to_free);
        lk.unlock();

        for (qvnt_reg* f : frees) qvnt_reg_destroy(f);
        int st = QVNT_OK;
        if (reg) {
            st = qvnt_reg_reset(reg, r->state);
        } else {
            st = qvnt_reg_create(s->ctx, r->n, r->state, &reg);
            if (!st) st = qvnt::reg_set_priority(reg, priority_for(s, r->n));
            if (!st) reg->tile_grid = true;
        }
        if (!st) st = run_request(r, reg);
        std::string err = st ? qvnt_last_error() : std::string();
        if (st && reg) {
            qvnt_reg_destroy(reg);  // its state is unknown: do not pool it
            reg = nullptr;
        }

        lk.lock();
        r->status = st;
        r->error = err;
        r->latency = s->now() - r->arrival;
        r->done = true;
        s->bytes_active -= r->footprint;
        s->running -= 1;
        if (large) s->large_running -= 1;
        if (reg) {
            s->idle.emplace(r->n, std::make_pair(reg, r->footprint));
            s->bytes_idle += r->footprint;
        }
        if (st) {
            s->failed += 1;
        } else {
            s->completed += 1;
            s->latencies.push_back(r->latency);
        }
        if (r->detached) {
            s->requests.erase(r->id);
            delete r;
        }
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

bool server_ok(const qvnt_server* s) { return s && s->magic == kMagicServer; }

#define CHECK_SERVER(s) \
    if (!server_ok(s)) return qvnt::set_error(QVNT_ERR_BAD_HANDLE, "invalid server handle")

}  // namespace

using qvnt::set_error;

extern "C" int qvnt_server_create(qvnt_ctx* ctx, uint64_t hbm_budget_bytes, uint32_t slots, uint32_t max_queue,
                                  qvnt_server** out) {
    if (!qvnt::ctx_valid(ctx)) return set_error(QVNT_ERR_BAD_HANDLE, "invalid context handle");
    if (!out) return set_error(QVNT_ERR_BAD_ARG, "null output pointer");
    if (slots == 0 || slots > 256) return set_error(QVNT_ERR_BAD_ARG, "slots = %u outside [1, 256]", slots);
    if (hbm_budget_bytes < (1ull << 24)) return set_error(QVNT_ERR_BAD_ARG, "HBM budget below 16 MiB");
    QVNT_CUDA_TRY(cudaSetDevice(ctx->device));
    qvnt_server* s = new qvnt_server();
    s->ctx = ctx;
    s->budget = hbm_budget_bytes;
    s->slots = slots;
    s->max_queue = max_queue ? max_queue : 4096;
    s->t0 = Clock::now();
    cudaDeviceGetStreamPriorityRange(&s->prio_least, &s->prio_greatest);
    s->magic = kMagicServer;
    for (uint32_t i = 0; i < slots; ++i) s->workers.emplace_back(worker, s);
    *out = s;
    return QVNT_OK;
}

extern "C" int qvnt_server_clock(qvnt_server* s, double* now_s) {
    CHECK_SERVER(s);
    if (now_s) *now_s = s->now();
    return QVNT_OK;
}

extern "C" int qvnt_server_submit(qvnt_server* s, uint32_t q_num, uint64_t state, const qvnt_gate* gates,
                                  const qvnt_call* calls, uint32_t ncalls, double arrival_s, int flags,
                                  uint64_t* id) {
    CHECK_SERVER(s);
    if (!id) return set_error(QVNT_ERR_BAD_ARG, "null id pointer");
    if (q_num > 34) return set_error(QVNT_ERR_BAD_ARG, "q_num %u > 34", q_num);
    if (ncalls && !calls) return set_error(QVNT_ERR_BAD_ARG, "null call list");
    const uint64_t len = q_num < 3 ? 8 : (1ull << q_num);
    if (state >= len) return set_error(QVNT_ERR_BAD_MASK, "state %llu out of range", (unsigned long long)state);
    uint64_t ng = 0;
    for (uint32_t c = 0; c < ncalls; ++c) {
        if (calls[c].op == QVNT_CALL_APPLY) {
            ng += calls[c].gate_count;
        } else if (calls[c].op == QVNT_CALL_MEASURE) {
            if (calls[c].mask & ~(len - 1)) return set_error(QVNT_ERR_BAD_MASK, "call %u: mask outside the register", c);
            if (!(calls[c].u01 >= 0.0 && calls[c].u01 < 1.0)) return set_error(QVNT_ERR_BAD_ARG, "call %u: u01", c);
        } else {
            return set_error(QVNT_ERR_BAD_ARG, "call %u: unknown op %u", c, calls[c].op);
        }
    }
    if (ng && !gates) return set_error(QVNT_ERR_BAD_ARG, "null gate list");
    for (uint64_t g = 0; g < ng; ++g) {
        const int st = qvnt::validate_gate(gates[g], len);
        if (st) return set_error(st, "gate %llu: %s", (unsigned long long)g, qvnt_last_error());
    }
    const uint64_t fp = reg_bytes(q_num) + ((flags & QVNT_SUBMIT_KEEP_AMPLITUDES) ? len * 16 : 0);
    if (fp > s->budget) return set_error(QVNT_ERR_OOM, "request needs %llu bytes, budget %llu",
                                         (unsigned long long)fp, (unsigned long long)s->budget);
    Request* r = new Request();
    r->n = q_num;
    r->state = state;
    r->gates.assign(gates, gates + ng);
    r->calls.assign(calls, calls + ncalls);
    r->keep_amplitudes = (flags & QVNT_SUBMIT_KEEP_AMPLITUDES) != 0;
    r->detached = (flags & QVNT_SUBMIT_DETACHED) != 0;
    r->footprint = fp;
    r->work = (double)len * (double)(ng + ncalls);
    std::lock_guard<std::mutex> lk(s->mu);
    r->arrival = arrival_s >= 0.0 ? arrival_s : s->now();
    if (s->queue.size() >= s->max_queue) {
        s->shed += 1;
        delete r;
        return set_error(QVNT_ERR_BUSY, "admission queue full (%u requests)", s->max_queue);
    }
    r->id = s->next_id++;
    s->submitted += 1;
    s->requests[r->id] = r;
    s->queue.push_back(r);
    *id = r->id;
    s->cv_work.notify_one();
    return QVNT_OK;
}

extern "C" int qvnt_server_wait(qvnt_server* s, uint64_t id, double timeout_s, uint64_t* results, double* amplitudes,
                                double* latency_s) {
    CHECK_SERVER(s);
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(id);
    if (it == s->requests.end() || it->second->detached)
        return set_error(QVNT_ERR_BAD_ARG, "unknown or detached request %llu", (unsigned long long)id);
    Request* r = it->second;
    auto ready = [&] { return r->done; };
    if (timeout_s >= 0.0) {
        if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready))
            return set_error(QVNT_ERR_TIMEOUT, "request %llu not finished", (unsigned long long)id);
    } else {
        s->cv_done.wait(lk, ready);
    }
    s->requests.erase(it);
    lk.unlock();
    const int st = r->status;
    if (st) {
        set_error(st, "request %llu: %s", (unsigned long long)id, r->error.c_str());
    } else {
        if (results && !r->results.empty()) memcpy(results, r->results.data(), r->results.size() * sizeof(uint64_t));
        if (amplitudes && !r->amplitudes.empty())
            memcpy(amplitudes, r->amplitudes.data(), r->amplitudes.size() * sizeof(double));
        if (latency_s) *latency_s = r->latency;
    }
    delete r;
    return st;
}

extern "C" int qvnt_server_stats(qvnt_server* s, qvnt_server_counters* out) {
    CHECK_SERVER(s);
    if (!out) return set_error(QVNT_ERR_BAD_ARG, "null output");
    std::lock_guard<std::mutex> lk(s->mu);
    out->submitted = s->submitted;
    out->shed = s->shed;
    out->completed = s->completed;
    out->failed = s->failed;
    out->queued = s->queue.size();
    out->running = s->running;
    out->peak_running = s->peak_running;
    out->bytes_active = s->bytes_active;
    out->bytes_pooled = s->bytes_idle;
    out->now_s = s->now();
    return QVNT_OK;
}

extern "C" int qvnt_server_latencies(qvnt_server* s, double* out, size_t cap, size_t* count) {
    CHECK_SERVER(s);
    std::lock_guard<std::mutex> lk(s->mu);
    const size_t n = std::min(cap, s->latencies.size());
    if (out && n) memcpy(out, s->latencies.data(), n * sizeof(double));
    if (count) *count = s->latencies.size();
    return QVNT_OK;
}

extern "C" int qvnt_server_queued_ages(qvnt_server* s, double* out, size_t cap, size_t* count) {
    CHECK_SERVER(s);
    std::lock_guard<std::mutex> lk(s->mu);
    const double t = s->now();
    size_t i = 0;
    for (const Request* r : s->queue) {
        if (out && i < cap) out[i] = t - r->arrival;
        ++i;
    }
    if (count) *count = i;
    return QVNT_OK;
}

extern "C" int qvnt_server_destroy(qvnt_server* s) {
    CHECK_SERVER(s);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        for (Request* r : s->queue) {
            r->status = QVNT_ERR_BUSY;
            r->error = "server destroyed before admission";
            r->done = true;
        }
        s->cv_work.notify_all();
        s->cv_done.notify_all();
    }
    for (std::thread& t : s->workers) t.join();  // running requests finish first
    for (auto& kv : s->requests) delete kv.second;
    for (auto& kv : s->idle) qvnt_reg_destroy(kv.second.first);
    for (qvnt_reg* r : s->to_free) qvnt_reg_destroy(r);
    s->magic = 0;
    delete s;
    return QVNT_OK;
}
