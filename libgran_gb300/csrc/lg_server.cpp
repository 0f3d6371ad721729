// lg_server.cpp -- continuous-batching serving loop for aggregate-mechanics requests.
//
// Requests (an aggregate's state and a step budget) arrive at any time. The server keeps one batch
// handle, the arena, whose systems are slots of fixed capacities (size classes); a request occupies
// one slot from admission to retirement, and its state, bonds and spring history stay in HBM there.
// Every resident request advances in the same launches: one rebuild period of the arena at a time
// (graph-replayed), all slots together. Each tick
//   1. waits for the period in flight and counts its steps for every occupant;
//   2. retires requests whose step budget is spent: state and observables are copied back and the
//      slot is emptied;
//   3. at a rebuild boundary, admits queued requests into free slots (first come first served, with
//      backfill; the smallest free slot that holds the request): each request is first built as a
//      standalone handle from the template -- bond detection and its construction force
//      evaluation, exactly as it would start alone -- and then moved into the slot on the device;
//   4. launches the next period (up to the next boundary, or to the earliest budget end), and
//      builds standalone handles for queued requests while the GPU runs.
// A request therefore evolves as it would alone: bit for bit in FP64; in mixed precision too when
// the lone run uses the arena's Hamaker slicing (lg_server_stats.hamaker_slices, see
// lg_set_step_shape) and step budgets are multiples of the rebuild period. Latency is measured on
// the host from submission to retirement. The arena's device memory is charged against the budget
// when it is created; standalone handles while they exist.
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
    int32_t state = LG_REQ_QUEUED;
    int64_t slot = -1;
    lg_system *stage = nullptr;  // standalone handle built before admission
    int64_t stage_bytes = 0;
    double t_submit = 0, t_admit = 0, t_done = 0;
    lg_observables obs{};
    std::vector<double> x_final;
    std::string error;
};

// Most rebuild periods one tick runs without returning to the host.
constexpr int64_t kChunkPeriods = 8;

// Default slots: size classes 128 .. 8192 monomers, 8 slots each.
const int64_t kClasses[] = {128, 256, 512, 1024, 2048, 4096, 8192};

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
    // the arena and its slots
    std::vector<int64_t> caps;      // capacity of every slot
    std::vector<int64_t> occupant;  // request in every slot, -1: free
    lg_system *arena = nullptr;
    int64_t arena_bytes = 0;
    cudaEvent_t start_ev = nullptr, done_ev = nullptr;
    bool in_flight = false;
    int64_t flight_steps = 0;
    double device_ms = 0.0;  // device time of the periods run so far
    int64_t periods = 0;
};

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

static int64_t slots_bytes(const lg_server *s, const std::vector<int64_t> &caps) {
    int64_t n = 0;
    for (int64_t c : caps) n += c;
    lg_system_desc d = s->tmpl;
    if (d.max_neighbors <= 0) d.max_neighbors = 96;
    return lg_estimate_device_bytes(&d, std::max<int64_t>(n, 1));
}

// Default slots that fit half the budget (the rest for standalone handles): 8 slots per size class,
// halved while too large, then the largest classes dropped.
static std::vector<int64_t> default_slots(const lg_server *s) {
    for (int per = 8; per >= 1; per /= 2)
        for (int top = 7; top >= 1; --top) {
            std::vector<int64_t> caps;
            for (int c = 0; c < top; ++c)
                for (int k = 0; k < per; ++k) caps.push_back(kClasses[c]);
            if (slots_bytes(s, caps) <= s->budget / 2) return caps;
            if (per > 1) break;  // halve the counts before dropping classes
        }
    return std::vector<int64_t>(1, kClasses[0]);
}

extern "C" int lg_server_create(const lg_system_desc *tmpl, int64_t budget_bytes, int64_t rebuild_every, double dt,
                                int device, lg_server **out) {
    if (!tmpl || !out) return lg_fail(LG_E_INVALID, "lg_server_create: null argument");
    if (budget_bytes <= 0) return lg_fail(LG_E_INVALID, "lg_server_create: budget must be positive");
    if (rebuild_every < 1) return lg_fail(LG_E_INVALID, "lg_server_create: rebuild_every must be >= 1");
    if (tmpl->hold_mask || tmpl->unary_hook)
        return lg_fail(LG_E_INVALID, "lg_server_create: a request template holds no per-particle mask or unary hook");
    if (tmpl->pairs != LG_PAIRS_VERLET || tmpl->n_facets != 0 || tmpl->body.model != LG_BODY_NONE ||
        tmpl->binary_model == LG_BINARY_SINTER_CONNECTORS)
        return lg_fail(LG_E_INVALID, "lg_server_create: requests need LG_PAIRS_VERLET, no facets, no body force and "
                                     "no 5-connector model");
    if (!(dt > 0) || !std::isfinite(dt)) return lg_fail(LG_E_INVALID, "lg_server_create: dt must be positive");
    lg_server *s = new (std::nothrow) lg_server();
    if (!s) return lg_fail(LG_E_NOMEM, "lg_server_create: host allocation failed");
    s->tmpl = *tmpl;
    if (s->tmpl.max_neighbors <= 0) s->tmpl.max_neighbors = 96;  // slots and standalone handles share it
    s->budget = budget_bytes;
    s->rebuild_every = rebuild_every;
    s->dt = dt;
    s->device = device;
    s->caps = default_slots(s);
    s->occupant.assign(s->caps.size(), -1);
    *out = s;
    return LG_OK;
}

extern "C" int lg_server_set_slots(lg_server *s, const int64_t *caps, int64_t count) {
    if (!s || !caps || count < 1) return lg_fail(LG_E_INVALID, "lg_server_set_slots: bad arguments");
    if (s->arena || !s->active.empty()) return lg_fail(LG_E_STATE, "lg_server_set_slots: slots are already in use");
    std::vector<int64_t> c(caps, caps + count);
    for (int64_t v : c)
        if (v < 1) return lg_fail(LG_E_INVALID, "lg_server_set_slots: capacity %lld", (long long)v);
    const int64_t bytes = slots_bytes(s, c);
    if (bytes > s->budget)
        return lg_fail(LG_E_NOMEM, "lg_server_set_slots: the slots need %lld bytes, more than the budget %lld",
                       (long long)bytes, (long long)s->budget);
    s->caps = c;
    s->occupant.assign(c.size(), -1);
    return LG_OK;
}

static void drop_stage(lg_server *s, Request &r) {
    if (r.stage) {
        lg_destroy(r.stage);
        r.stage = nullptr;
        s->used -= r.stage_bytes;
        r.stage_bytes = 0;
    }
}

static int wait_flight(lg_server *s) {
    if (!s->in_flight) return LG_OK;
    const cudaError_t e = cudaEventSynchronize(s->done_ev);
    s->in_flight = false;
    if (e != cudaSuccess) {
        cudaGetLastError();
        return lg_fail(LG_E_CUDA, "serving period failed on the device: %s", cudaGetErrorString(e));
    }
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, s->start_ev, s->done_ev) == cudaSuccess) s->device_ms += ms;
    cudaGetLastError();
    s->periods++;
    for (int64_t id : s->active) {
        Request &r = s->reqs[id];
        r.done_steps += s->flight_steps;
        s->particle_steps += s->flight_steps * r.n;
    }
    return LG_OK;
}

static void fail_request(lg_server *s, Request &r, const std::string &why) {
    r.state = LG_REQ_FAILED;
    r.error = why;
    r.t_done = now_ms();
    s->failed++;
}

extern "C" int lg_server_destroy(lg_server *s) {
    if (!s) return LG_OK;
    if (s->in_flight) cudaEventSynchronize(s->done_ev);
    for (auto &kv : s->reqs) drop_stage(s, kv.second);
    if (s->arena) lg_destroy(s->arena);
    if (s->done_ev) cudaEventDestroy(s->done_ev);
    if (s->start_ev) cudaEventDestroy(s->start_ev);
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
    const int64_t largest = *std::max_element(s->caps.begin(), s->caps.end());
    if (n > largest) {
        s->rejected++;
        return lg_fail(LG_E_NOMEM, "lg_server_submit: a request of %lld particles is larger than the largest slot (%lld)",
                       (long long)n, (long long)largest);
    }
    Request r;
    r.id = s->next_id++;
    r.n = n;
    r.nsteps = nsteps;
    r.x0.assign(x0, x0 + 3 * n);
    r.v0.assign(3 * n, 0.0);
    if (v0) std::copy(v0, v0 + 3 * n, r.v0.begin());
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
        drop_stage(s, r);
    } else if (r.state == LG_REQ_RUNNING) {
        const int rc = wait_flight(s);  // the slot is emptied only while the arena is idle
        if (rc != LG_OK) return rc;
        if (r.slot >= 0) {
            lg_arena_clear(s->arena, r.slot);
            s->occupant[(size_t)r.slot] = -1;
            r.slot = -1;
        }
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

// The standalone handle of a queued request: bond detection and the construction force evaluation,
// as the request would start alone. A failure (including an injected one) fails the request.
static bool stage(lg_server *s, Request &r) {
    if (r.stage) return true;
    lg_system_desc d = s->tmpl;
    d.n_part = r.n;
    const int64_t bytes = lg_estimate_device_bytes(&d, r.n);
    if (s->used + bytes > s->budget) return false;  // later, when memory is free
    int rc;
    if (s->inject_alloc_failures > 0) {  // host-side stand-in for a failing device allocation
        s->inject_alloc_failures--;
        rc = lg_fail(LG_E_NOMEM, "cudaMalloc failed: out of memory (injected)");
    } else {
        rc = lg_create_staged(&d, r.x0.data(), r.v0.data(), s->device, &r.stage);
    }
    if (rc != LG_OK) {
        r.stage = nullptr;
        fail_request(s, r, lg_last_error());
        return false;
    }
    r.stage_bytes = bytes;
    s->used += bytes;
    s->peak = std::max(s->peak, s->used);
    return true;
}

static int ensure_arena(lg_server *s) {
    if (s->arena) return LG_OK;
    const int64_t bytes = slots_bytes(s, s->caps);
    if (s->used + bytes > s->budget)
        return lg_fail(LG_E_NOMEM, "serving slots need %lld bytes; %lld of the budget %lld are free", (long long)bytes,
                       (long long)(s->budget - s->used), (long long)s->budget);
    int rc = lg_arena_create(&s->tmpl, (int64_t)s->caps.size(), s->caps.data(), s->device, &s->arena);
    if (rc != LG_OK) return rc;
    if (cudaEventCreate(&s->done_ev) != cudaSuccess || cudaEventCreate(&s->start_ev) != cudaSuccess) {
        cudaGetLastError();
        return lg_fail(LG_E_CUDA, "cudaEventCreate failed");
    }
    s->arena_bytes = bytes;
    s->used += bytes;
    s->peak = std::max(s->peak, s->used);
    return LG_OK;
}

// The smallest free slot that holds n particles, or -1.
static int64_t free_slot(const lg_server *s, int64_t n) {
    int64_t best = -1;
    for (size_t q = 0; q < s->caps.size(); ++q)
        if (s->occupant[q] < 0 && s->caps[q] >= n && (best < 0 || s->caps[q] < s->caps[(size_t)best])) best = (int64_t)q;
    return best;
}

static void retire(lg_server *s, std::vector<int64_t> &done) {
    if (done.empty()) return;
    std::string why;
    int32_t errs = 0;
    if (lg_get_device_errors(s->arena, &errs) != LG_OK) why = lg_last_error();
    else if (errs != 0) why = "device error word set (" + std::to_string(errs) + ")";
    for (int64_t id : done) {
        Request &r = s->reqs[id];
        r.x_final.resize(3 * r.n);
        // observables over the occupant's own particles; the radius of gyration from its positions
        int rr = why.empty() ? lg_arena_observables(s->arena, r.slot, r.n, &r.obs) : LG_E_STATE;
        if (rr == LG_OK) rr = lg_arena_read(s->arena, r.slot, r.n, r.x_final.data(), nullptr, nullptr, nullptr);
        if (rr == LG_OK) {
            const double *c = r.obs.center_of_mass;
            double rg = 0.0;
            for (int64_t i = 0; i < r.n; ++i)
                for (int k = 0; k < 3; ++k) rg += (r.x_final[3 * i + k] - c[k]) * (r.x_final[3 * i + k] - c[k]);
            r.obs.radius_of_gyration = std::sqrt(rg / (double)r.n);
        }
        lg_arena_clear(s->arena, r.slot);
        s->occupant[(size_t)r.slot] = -1;
        r.slot = -1;
        r.t_done = now_ms();
        if (rr != LG_OK) {
            fail_request(s, r, why.empty() ? std::string(lg_last_error()) : why);
        } else {
            r.state = LG_REQ_DONE;
            s->completed++;
            s->latencies.push_back(r.t_done - r.t_submit);
        }
    }
}

extern "C" int lg_server_tick(lg_server *s, int32_t *n_active, int32_t *n_queued, int32_t *n_retired) {
    if (!s) return lg_fail(LG_E_INVALID, "lg_server_tick: null server");
    int rc = wait_flight(s);
    if (rc != LG_OK) {  // the period failed: its occupants fail with it
        const std::string why = lg_last_error();
        for (int64_t id : s->active) {
            Request &r = s->reqs[id];
            if (s->arena && r.slot >= 0) lg_arena_clear(s->arena, r.slot);
            if (r.slot >= 0) s->occupant[(size_t)r.slot] = -1;
            r.slot = -1;
            fail_request(s, r, why);
        }
        s->active.clear();
    }
    // retire requests whose budget is spent
    std::vector<int64_t> done, still;
    for (int64_t id : s->active) (s->reqs[id].done_steps >= s->reqs[id].nsteps ? done : still).push_back(id);
    retire(s, done);
    s->active.swap(still);
    const int32_t retired = (int32_t)done.size();
    // admissions at a rebuild boundary: the occupant's rows start with the arena's next build
    const bool boundary = !s->arena || (s->arena->step_index % s->rebuild_every) == 0;
    if (boundary) {
        for (auto it = s->queue.begin(); it != s->queue.end();) {
            Request &r = s->reqs[*it];
            const int64_t q = free_slot(s, r.n);
            if (q < 0) {
                if (!s->backfill) break;
                ++it;
                continue;
            }
            if (!stage(s, r)) {
                if (r.state == LG_REQ_FAILED) {
                    it = s->queue.erase(it);
                    continue;
                }
                if (!s->backfill) break;
                ++it;
                continue;
            }
            rc = ensure_arena(s);
            if (rc == LG_OK) rc = lg_arena_import(s->arena, q, r.stage, r.x0.data());
            drop_stage(s, r);
            if (rc != LG_OK) {
                fail_request(s, r, lg_last_error());
                it = s->queue.erase(it);
                continue;
            }
            s->occupant[(size_t)q] = r.id;
            r.slot = q;
            r.state = LG_REQ_RUNNING;
            r.t_admit = now_ms();
            r.x0.clear();
            r.x0.shrink_to_fit();
            r.v0.clear();
            r.v0.shrink_to_fit();
            s->active.push_back(r.id);
            it = s->queue.erase(it);
        }
    }
    // the next periods of every occupant, in the same launches: up to the earliest budget end (the
    // budgets are known), to the next boundary when a queued request could take a free slot there,
    // and at most kChunkPeriods periods, so that the host returns between them only when it has
    // something to do
    if (!s->active.empty()) {
        const int64_t to_boundary = s->rebuild_every - (s->arena->step_index % s->rebuild_every);
        bool admit_next = false;
        for (int64_t id : s->queue)
            if (free_slot(s, s->reqs[id].n) >= 0) {
                admit_next = true;
                break;
            }
        int64_t k = admit_next ? to_boundary : to_boundary + (kChunkPeriods - 1) * s->rebuild_every;
        for (int64_t id : s->active) k = std::min(k, s->reqs[id].nsteps - s->reqs[id].done_steps);
        rc = cudaEventRecord(s->start_ev, s->arena->stream) == cudaSuccess
                 ? LG_OK : lg_fail(LG_E_CUDA, "cudaEventRecord failed");
        if (rc == LG_OK) rc = lg_step(s->arena, s->dt, k, s->rebuild_every);
        if (rc == LG_OK && cudaEventRecord(s->done_ev, s->arena->stream) != cudaSuccess) {
            cudaGetLastError();
            rc = lg_fail(LG_E_CUDA, "cudaEventRecord failed");
        }
        if (rc != LG_OK) return rc;
        s->in_flight = true;
        s->flight_steps = k;
    }
    // standalone handles for the head of the queue while the periods run: as many as there will be
    // free slots at the next return (free now, or freed by budgets ending), and a few more
    int64_t free_slots = 0;
    for (int64_t o : s->occupant) free_slots += o < 0 ? 1 : 0;
    for (int64_t id : s->active)
        if (s->reqs[id].done_steps + (s->in_flight ? s->flight_steps : 0) >= s->reqs[id].nsteps) ++free_slots;
    int64_t staged = 0;
    for (auto it = s->queue.begin(); it != s->queue.end() && staged < free_slots + 4;) {
        Request &r = s->reqs[*it];
        if (!stage(s, r) && r.state == LG_REQ_FAILED) {
            it = s->queue.erase(it);
            continue;
        }
        staged += r.stage ? 1 : 0;
        ++it;
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
    o->slots = (int64_t)s->caps.size();
    for (size_t q = 0; q < s->caps.size(); ++q) {
        o->slot_particles += s->caps[q];
        if (s->occupant[q] >= 0) {
            o->slots_busy++;
            o->resident_particles += s->reqs[s->occupant[q]].n;
        }
    }
    o->hamaker_slices = s->tmpl.precision == LG_PRECISION_MIXED ? lg::mixed_hamaker_slices(o->slot_particles) : 0;
    o->device_ms = s->device_ms;
    o->periods = s->periods;
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
