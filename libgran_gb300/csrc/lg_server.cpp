// lg_server.cpp -- continuous-batching serving loop for aggregate-mechanics requests.
//
// Requests (an aggregate's state and a step budget) arrive at any time. Each tick the server
//   1. admits queued requests, first come first served with backfill, while their device
//      footprint fits the memory budget: a request becomes a resident engine handle (its state,
//      springs and bonds stay in HBM until it finishes) with its own CUDA stream;
//   2. keeps every resident request two rebuild periods ahead on its own stream (graph replays;
//      completion is tracked with events, no global synchronisation), so requests of different
//      sizes progress at their own pace and their kernels overlap on the device;
//   3. retires requests whose budget is spent: observables and positions are copied back, the
//      handle is destroyed and its memory returns to the budget.
// A request's result does not depend on what else is resident (each is its own handle), so a
// request gives the same result alone and in the mix. Latency is measured on the host from
// submission to retirement.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "lg_engine_internal.h"

namespace {

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
    int64_t id = 0;
    int64_t n = 0;
    int64_t nsteps = 0, done_steps = 0;
    std::vector<double> x0, v0;
    int64_t bytes = 0;
    int32_t state = LG_REQ_QUEUED;
    lg_system *sys = nullptr;
    double t_submit = 0, t_admit = 0, t_done = 0;
    lg_observables obs{};
    std::vector<double> x_final;
    std::string error;
    int64_t enqueued_steps = 0;
    std::deque<std::pair<cudaEvent_t, int64_t>> inflight;  // (event after a period, its steps)
    std::vector<cudaEvent_t> free_events;
};

constexpr int kPeriodsAhead = 2;

}  // namespace

struct lg_server {
    lg_system_desc tmpl{};
    int64_t budget = 0, used = 0, peak = 0;
    int64_t rebuild_every = 20;
    double dt = 0;
    int device = 0;
    int64_t next_id = 1;
    std::deque<int64_t> queue;
    std::vector<int64_t> active;
    std::unordered_map<int64_t, Request> reqs;
    std::vector<double> latencies;
    int64_t completed = 0, rejected = 0, failed = 0, cancelled = 0;
    int64_t particle_steps = 0;
    int32_t inject_alloc_failures = 0;
    int32_t backfill = 1;
};

// Device bytes of one request: state and its ping-pong copies, float-float copies, pair slots (two
// buffers), bonds, facet springs, list scratch, observables scratch, plus a fixed overhead.
extern "C" int64_t lg_estimate_device_bytes(const lg_system_desc *d, int64_t n) {
    if (!d || n < 1) return -1;
    const int64_t cap = d->pairs == LG_PAIRS_VERLET ? (d->max_neighbors > 0 ? d->max_neighbors : 64) : std::max<int64_t>(n - 1, 1);
    const int64_t nbuf = d->pairs == LG_PAIRS_VERLET ? 2 : 1;
    int64_t b = 10 * 32 * n;                                  // x, th, v[2], w[2], a, al (+ slack)
    b += 320 * n;                                             // float-float state (two x32, v32; s32) and partial sums
    b += nbuf * cap * n * (4 + 4 + 72 + 5) + nbuf * 8 * n;   // nbr, flags, springs, near lists, row lengths
    b += 8 * n * (1 + 1 + 8 + 72);                            // bonds (up to 8 per particle)
    b += 72 * std::max(d->n_facets, 1) * n;                   // facet springs
    b += 4 * 8 * n + 4 * 4 * n;                               // list scratch
    b += 20 * 8 * n;                                          // observables scratch
    if (d->precision == LG_PRECISION_FP64 && cap * n <= ((int64_t)1 << 21))
        b += 48 * cap * n;                                    // pair-parallel kernel scratch
    return b + (4 << 20);                                     // fixed overhead
}

extern "C" int lg_server_create(const lg_system_desc *tmpl, int64_t budget_bytes, int64_t rebuild_every, double dt,
                                int device, lg_server **out) {
    if (!tmpl || !out) return lg_fail(LG_E_INVALID, "lg_server_create: null argument");
    if (budget_bytes <= 0) return lg_fail(LG_E_INVALID, "lg_server_create: budget must be positive");
    if (rebuild_every < 1) return lg_fail(LG_E_INVALID, "lg_server_create: rebuild_every must be >= 1");
    if (tmpl->hold_mask || tmpl->unary_hook)
        return lg_fail(LG_E_INVALID, "lg_server_create: a request template holds no per-particle mask or unary hook");
    if (!(dt > 0) || !std::isfinite(dt)) return lg_fail(LG_E_INVALID, "lg_server_create: dt must be positive");
    lg_server *s = new (std::nothrow) lg_server();
    if (!s) return lg_fail(LG_E_NOMEM, "lg_server_create: host allocation failed");
    s->tmpl = *tmpl;
    s->budget = budget_bytes;
    s->rebuild_every = rebuild_every;
    s->dt = dt;
    s->device = device;
    *out = s;
    return LG_OK;
}

static void release_request(lg_server *s, Request &r) {
    if (r.sys) {
        cudaStreamSynchronize(r.sys->stream);
        for (auto &p : r.inflight) cudaEventDestroy(p.first);
        for (auto e : r.free_events) cudaEventDestroy(e);
        r.inflight.clear();
        r.free_events.clear();
        lg_destroy(r.sys);
        r.sys = nullptr;
        s->used -= r.bytes;
    }
}

extern "C" int lg_server_destroy(lg_server *s) {
    if (!s) return LG_OK;
    for (auto &kv : s->reqs) release_request(s, kv.second);
    delete s;
    return LG_OK;
}

extern "C" int lg_server_submit(lg_server *s, int64_t n, const double *x0, const double *v0, int64_t nsteps,
                                int64_t *request_id) {
    if (!s || !request_id) return lg_fail(LG_E_INVALID, "lg_server_submit: null argument");
    *request_id = 0;
    if (n < 1 || !x0) return lg_fail(LG_E_INVALID, "lg_server_submit: malformed request (n = %lld)", (long long)n);
    if (nsteps < 1) return lg_fail(LG_E_INVALID, "lg_server_submit: malformed request (nsteps = %lld)", (long long)nsteps);
    for (int64_t q = 0; q < 3 * n; ++q)
        if (!std::isfinite(x0[q]) || (v0 && !std::isfinite(v0[q])))
            return lg_fail(LG_E_INVALID, "lg_server_submit: malformed request (non-finite state)");
    const int64_t bytes = lg_estimate_device_bytes(&s->tmpl, n);
    if (bytes > s->budget) {
        s->rejected++;
        return lg_fail(LG_E_NOMEM, "lg_server_submit: request needs %lld bytes, more than the whole budget %lld",
                       (long long)bytes, (long long)s->budget);
    }
    Request r;
    r.id = s->next_id++;
    r.n = n;
    r.nsteps = nsteps;
    r.x0.assign(x0, x0 + 3 * n);
    r.v0.assign(3 * n, 0.0);
    if (v0) std::copy(v0, v0 + 3 * n, r.v0.begin());
    r.bytes = bytes;
    r.t_submit = now_ms();
    *request_id = r.id;
    s->queue.push_back(r.id);
    s->reqs.emplace(r.id, std::move(r));
    return LG_OK;
}

extern "C" int lg_server_cancel(lg_server *s, int64_t id) {
    if (!s) return lg_fail(LG_E_INVALID, "lg_server_cancel: null server");
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return lg_fail(LG_E_INVALID, "lg_server_cancel: unknown request %lld", (long long)id);
    Request &r = it->second;
    if (r.state == LG_REQ_QUEUED) {
        s->queue.erase(std::remove(s->queue.begin(), s->queue.end(), id), s->queue.end());
    } else if (r.state == LG_REQ_RUNNING) {
        if (r.sys) cudaStreamSynchronize(r.sys->stream);
        release_request(s, r);
        s->active.erase(std::remove(s->active.begin(), s->active.end(), id), s->active.end());
    } else {
        return LG_OK;  // already finished
    }
    r.state = LG_REQ_CANCELLED;
    r.t_done = now_ms();
    s->cancelled++;
    return LG_OK;
}

extern "C" int lg_server_inject_alloc_failures(lg_server *s, int32_t count) {
    if (!s) return lg_fail(LG_E_INVALID, "lg_server_inject_alloc_failures: null server");
    s->inject_alloc_failures = count;
    return LG_OK;
}

static int admit(lg_server *s) {
    // first come first served; with backfill, later requests that fit may pass a head that does not
    for (auto it = s->queue.begin(); it != s->queue.end();) {
        Request &r = s->reqs[*it];
        if (s->used + r.bytes > s->budget) {
            if (!s->backfill) break;
            ++it;
            continue;
        }
        lg_system_desc d = s->tmpl;
        d.n_part = r.n;
        int rc;
        if (s->inject_alloc_failures > 0) {  // host-side stand-in for a failing device allocation
            s->inject_alloc_failures--;
            rc = lg_fail(LG_E_NOMEM, "cudaMalloc failed: out of memory (injected)");
        } else {
            std::vector<double> zeros(3 * r.n, 0.0);
            rc = lg_create(&d, r.x0.data(), r.v0.data(), zeros.data(), zeros.data(), nullptr, nullptr, 0, s->device,
                           &r.sys);
        }
        if (rc != LG_OK) {
            r.state = LG_REQ_FAILED;
            r.error = lg_last_error();
            r.t_done = now_ms();
            s->failed++;
            it = s->queue.erase(it);
            continue;
        }
        s->used += r.bytes;
        s->peak = std::max(s->peak, s->used);
        r.state = LG_REQ_RUNNING;
        r.t_admit = now_ms();
        r.x0.clear();
        r.x0.shrink_to_fit();
        r.v0.clear();
        r.v0.shrink_to_fit();
        s->active.push_back(r.id);
        it = s->queue.erase(it);
    }
    return LG_OK;
}

static void retire(lg_server *s, Request &r) {
    r.x_final.resize(3 * r.n);
    int rc = lg_get_observables(r.sys, &r.obs);  // synchronises the request's stream
    if (rc == LG_OK) rc = lg_get(r.sys, LG_FIELD_X, r.x_final.data());
    int32_t errs = 0;
    if (rc == LG_OK) rc = lg_get_device_errors(r.sys, &errs);
    std::string why = rc != LG_OK ? std::string(lg_last_error()) : std::string("device error word set");
    release_request(s, r);
    r.t_done = now_ms();
    if (rc != LG_OK || errs != 0) {
        r.state = LG_REQ_FAILED;
        r.error = why;
        s->failed++;
    } else {
        r.state = LG_REQ_DONE;
        s->completed++;
        s->latencies.push_back(r.t_done - r.t_submit);
    }
}

extern "C" int lg_server_tick(lg_server *s, int32_t *n_active, int32_t *n_queued, int32_t *n_retired) {
    if (!s) return lg_fail(LG_E_INVALID, "lg_server_tick: null server");
    const size_t queued_before = s->queue.size();
    int rc = admit(s);
    if (rc != LG_OK) return rc;
    bool progress = s->queue.size() != queued_before;
    const int64_t rb = s->tmpl.pairs == LG_PAIRS_VERLET ? s->rebuild_every : 0;
    // keep every resident request kPeriodsAhead periods ahead on its stream
    for (int64_t id : s->active) {
        Request &r = s->reqs[id];
        while ((int)r.inflight.size() < kPeriodsAhead && r.enqueued_steps < r.nsteps && r.state == LG_REQ_RUNNING) {
            const int64_t k = std::min(s->rebuild_every, r.nsteps - r.enqueued_steps);
            rc = lg_step(r.sys, s->dt, k, rb);
            cudaEvent_t ev = nullptr;
            if (rc == LG_OK) {
                if (!r.free_events.empty()) {
                    ev = r.free_events.back();
                    r.free_events.pop_back();
                } else if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
                    ev = nullptr;
                    rc = lg_fail(LG_E_CUDA, "cudaEventCreate failed");
                }
            }
            if (rc == LG_OK && cudaEventRecord(ev, r.sys->stream) != cudaSuccess) rc = lg_fail(LG_E_CUDA, "cudaEventRecord failed");
            if (rc != LG_OK) {
                r.state = LG_REQ_FAILED;
                r.error = lg_last_error();
                if (ev) r.free_events.push_back(ev);
                break;
            }
            r.inflight.emplace_back(ev, k);
            r.enqueued_steps += k;
        }
    }
    // collect finished periods; retire finished requests
    int32_t retired = 0;
    std::vector<int64_t> still;
    for (int64_t id : s->active) {
        Request &r = s->reqs[id];
        if (r.state == LG_REQ_FAILED) {
            release_request(s, r);
            r.t_done = now_ms();
            s->failed++;
            ++retired;
            progress = true;
            continue;
        }
        cudaError_t qe = cudaSuccess;
        while (!r.inflight.empty() && (qe = cudaEventQuery(r.inflight.front().first)) == cudaSuccess) {
            r.done_steps += r.inflight.front().second;
            s->particle_steps += r.inflight.front().second * r.n;
            r.free_events.push_back(r.inflight.front().first);
            r.inflight.pop_front();
            progress = true;
        }
        if (qe == cudaErrorNotReady) {
            cudaGetLastError();  // a pending event is not an error
        } else if (qe != cudaSuccess) {
            // the period failed on the device (or the context is lost): the request fails with the
            // error instead of staying active with an event that never completes
            cudaGetLastError();
            r.state = LG_REQ_FAILED;
            r.error = std::string("device error while running the request: ") + cudaGetErrorString(qe);
            release_request(s, r);
            r.t_done = now_ms();
            s->failed++;
            ++retired;
            progress = true;
            continue;
        }
        if (r.done_steps >= r.nsteps) {
            retire(s, r);
            ++retired;
            continue;
        }
        still.push_back(id);
    }
    s->active.swap(still);
    // nothing moved: wait for the oldest outstanding period instead of spinning
    if (!progress && !s->active.empty()) {
        Request &r = s->reqs[s->active.front()];
        if (!r.inflight.empty()) cudaEventSynchronize(r.inflight.front().first);
    }
    if (n_active) *n_active = (int32_t)s->active.size();
    if (n_queued) *n_queued = (int32_t)s->queue.size();
    if (n_retired) *n_retired = retired;
    return LG_OK;
}

extern "C" int lg_server_poll(lg_server *s, int64_t id, int32_t *state, lg_observables *obs, double *x_out,
                              double *latency_ms) {
    if (!s || !state) return lg_fail(LG_E_INVALID, "lg_server_poll: null argument");
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return lg_fail(LG_E_INVALID, "lg_server_poll: unknown request %lld", (long long)id);
    Request &r = it->second;
    *state = r.state;
    if (r.state == LG_REQ_DONE) {
        if (obs) *obs = r.obs;
        if (x_out) std::copy(r.x_final.begin(), r.x_final.end(), x_out);
    }
    if (latency_ms) *latency_ms = r.t_done > 0 ? r.t_done - r.t_submit : -1.0;
    if (r.state == LG_REQ_FAILED) lg_fail(LG_OK, "%s", r.error.c_str());
    return LG_OK;
}

// Forget a finished request (its result is no longer retrievable).
extern "C" int lg_server_release(lg_server *s, int64_t id) {
    if (!s) return lg_fail(LG_E_INVALID, "lg_server_release: null server");
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return LG_OK;
    if (it->second.state == LG_REQ_QUEUED || it->second.state == LG_REQ_RUNNING)
        return lg_fail(LG_E_STATE, "lg_server_release: request %lld is not finished", (long long)id);
    s->reqs.erase(it);
    return LG_OK;
}

extern "C" int lg_server_get_stats(lg_server *s, lg_server_stats *o) {
    if (!s || !o) return lg_fail(LG_E_INVALID, "lg_server_get_stats: null argument");
    memset(o, 0, sizeof(*o));
    o->budget_bytes = s->budget;
    o->used_bytes = s->used;
    o->peak_bytes = s->peak;
    o->active = (int64_t)s->active.size();
    o->queued = (int64_t)s->queue.size();
    o->completed = s->completed;
    o->rejected = s->rejected;
    o->failed = s->failed;
    o->cancelled = s->cancelled;
    o->particle_steps = s->particle_steps;
    if (!s->latencies.empty()) {
        std::vector<double> l = s->latencies;
        std::sort(l.begin(), l.end());
        auto pct = [&](double p) {
            double k = p * (double)(l.size() - 1);
            size_t a = (size_t)std::floor(k), b = std::min(a + 1, l.size() - 1);
            return l[a] + (l[b] - l[a]) * (k - (double)a);
        };
        o->p50_latency_ms = pct(0.50);
        o->p99_latency_ms = pct(0.99);
        o->max_latency_ms = l.back();
    }
    return LG_OK;
}
