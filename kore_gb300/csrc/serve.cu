// Serving queue (kore_batch_*, include/kore_gpu.h): eigen and forced solves of
// different pencils run by worker threads, each request on its own plan and CUDA
// stream, admitted by an upper bound of its device memory against a budget, with a
// cache of uploaded and factorised plans keyed by the caller's pencil name.
//
// The reference has no counterpart: it runs one bin/solve.py process per problem.
// A request does what one such run does (kore_eigs at its target, or kore_solve at
// its shift) on a plan of its own, so its result does not depend on what else runs.
#include "kore_internal.cuh"
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;

// backward error above which a mixed-precision forced solve is redone with FP64 factors
constexpr double kForcedEscalateTol = 1e-10;

double ms_since(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// Eigen slots of a shared plan: eigen requests of one pencil run together in the
// batched engine (kore_eigs_engine), up to this many at a time.
constexpr int kServeSlots = 4;

// A plan of one pencil, idle in the cache or in use by one request (forced) or by the
// eigen engine (eigen requests of its pencil).
struct CachedPlan {
    uint64_t key = 0;
    kore_plan *plan = nullptr;
    int64_t bytes = 0;          // charged against the budget (estimate, then the larger of it and the plan's own count)
    bool busy = false;
    bool engine = false;        // busy running the eigen engine: new eigen requests of this key join it
    bool factored = false;      // one shift factorised (forced requests)
    double sre = 0, sim = 0;
    int prec = -1;
    int slots = 0;              // eigen slots reserved (kore_factor_reserve), 0 if the plan holds one shift
    int slot_prec = -1;         // precision of the reserved slots
    int engine_prec = -1;       // precision of the running engine
    bool slot_valid[kServeSlots] = {};
    uint64_t last_use = 0;
};

struct Request {
    kore_request r;
    uint64_t ticket = 0;
    Clock::time_point t_submit, t_start, t_end;
    int status = KORE_EPENDING;
    bool done = false;
    bool by_engine = false;     // started and finished by an eigen engine's source
    int64_t est = -1;           // estimate of a new plan for this request
};

}  // namespace

struct kore_batch {
    int device = 0;
    int64_t budget = 0;
    int64_t used = 0;           // bytes of cached and in-use plans plus reservations
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> queue;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    std::vector<std::unique_ptr<CachedPlan>> plans;
    std::vector<std::thread> workers;
    bool stop = false;
    uint64_t next_ticket = 1, clock = 0;
    int64_t submitted = 0, finished = 0, running = 0, hits = 0, created = 0, evicted = 0;
    int64_t joined = 0;         // eigen requests admitted into a running engine's free slot
};

namespace {

constexpr double kHoldBackMs = 200.0;   // a request waiting longer than this blocks new starts

// Largest ncv an engine slot holds (the engine's basis size).
constexpr int kServeMaxNcv = 64;

bool shared_eigen(const kore_request &r) { return r.kind == KORE_REQ_EIGEN && r.pencil_key != 0; }

int estimate(const kore_request &r, int64_t *bytes) {
    if (r.kind == KORE_REQ_EIGEN)
        return kore_plan_estimate_bytes(r.pencil, r.precision, shared_eigen(r) ? kServeSlots : 1, kServeMaxNcv, bytes);
    return kore_plan_estimate_bytes(r.pencil, r.precision, 1, 0, bytes);
}

// An idle plan of this key factorised at this shift and precision, else an idle plan of
// this key, else null.  Caller holds the lock.
CachedPlan *find_idle(kore_batch *b, const kore_request &r, bool *hit) {
    *hit = false;
    if (r.pencil_key == 0) return nullptr;
    CachedPlan *any = nullptr;
    for (auto &c : b->plans) {
        if (c->busy || c->key != r.pencil_key) continue;
        if (r.kind == KORE_REQ_FORCED && c->factored && c->prec == r.precision && c->sre == r.sigma_re &&
            c->sim == r.sigma_im) {
            *hit = true;
            return c.get();
        }
        if (!any) any = c.get();
    }
    return any;
}

// Free idle cached plans, oldest first, until `need` more bytes fit.  Caller holds the lock.
bool make_room(kore_batch *b, int64_t need) {
    while (b->used + need > b->budget) {
        CachedPlan *old = nullptr;
        size_t at = 0;
        for (size_t i = 0; i < b->plans.size(); ++i) {
            CachedPlan *c = b->plans[i].get();
            if (!c->busy && (!old || c->last_use < old->last_use)) { old = c; at = i; }
        }
        if (!old) return false;
        b->used -= old->bytes;
        kore_plan_destroy(old->plan);
        b->plans.erase(b->plans.begin() + (std::ptrdiff_t)at);
        ++b->evicted;
    }
    return true;
}

// True when an engine of this request's pencil and precision is running.  Caller holds
// the lock.
bool engine_running(kore_batch *b, const kore_request &r) {
    for (auto &c : b->plans)
        if (c->engine && c->key == r.pencil_key && c->engine_prec == r.precision) return true;
    return false;
}

// Pick the next request that can start and reserve its plan.  Caller holds the lock.
Request *admit(kore_batch *b, CachedPlan **slot) {
    const auto now = Clock::now();
    for (auto it = b->queue.begin(); it != b->queue.end(); ++it) {
        Request *q = *it;
        // an eigen request of a pencil whose engine is running joins that engine when a
        // slot frees up; it does not start on a second plan
        if (shared_eigen(q->r) && engine_running(b, q->r)) continue;
        bool hit = false;
        CachedPlan *c = find_idle(b, q->r, &hit);
        if (c) {
            c->busy = true;
            c->last_use = ++b->clock;
            if (hit) ++b->hits;
            *slot = c;
            b->queue.erase(it);
            return q;
        }
        if (q->est < 0 && estimate(q->r, &q->est) != KORE_OK) {
            // unusable pencil: finish it with the error right away
            q->status = KORE_EINVAL;
            *slot = nullptr;
            b->queue.erase(it);
            return q;
        }
        if (q->est > b->budget) {
            q->status = KORE_ENOMEM;
            *slot = nullptr;
            b->queue.erase(it);
            return q;
        }
        if (make_room(b, q->est)) {
            auto cp = std::make_unique<CachedPlan>();
            cp->key = q->r.pencil_key;
            cp->bytes = q->est;
            cp->busy = true;
            cp->last_use = ++b->clock;
            b->used += q->est;
            *slot = cp.get();
            b->plans.push_back(std::move(cp));
            b->queue.erase(it);
            return q;
        }
        // does not fit yet: let later requests start unless this one has waited too long
        if (ms_since(q->t_submit, now) > kHoldBackMs) return nullptr;
    }
    return nullptr;
}

// Requests for the eigen engine of one plan: the admitted request first, then queued
// eigen requests of the same pencil and precision as slots free up.
struct ServeSource : EigsSource {
    kore_batch *b;
    CachedPlan *c;
    Request *first;
    bool gave_first = false;
    static void fill(Request *q, EigsTarget *t) {
        const kore_request &r = q->r;
        t->opts = r.opts;
        t->opts.target_re = r.sigma_re;
        t->opts.target_im = r.sigma_im;
        t->evals = r.evals;
        t->evecs = r.evecs;
        t->max_pairs = r.max_pairs;
        t->nconv = r.nconv;
        t->stats = r.stats;
        t->tag = q;
    }
    bool next(EigsTarget *t) override {
        if (!gave_first) {
            gave_first = true;
            fill(first, t);
            return true;
        }
        std::lock_guard<std::mutex> lk(b->mu);
        if (b->stop) return false;
        for (auto it = b->queue.begin(); it != b->queue.end(); ++it) {
            Request *q = *it;
            if (!shared_eigen(q->r) || q->r.pencil_key != c->key || q->r.precision != c->engine_prec) continue;
            if (!q->r.evals || !q->r.nconv || q->r.max_pairs <= 0) continue;   // left to a worker (EINVAL)
            b->queue.erase(it);
            q->t_start = Clock::now();
            q->by_engine = true;
            ++b->running;
            ++b->joined;
            fill(q, t);
            return true;
        }
        return false;
    }
    void finished(const EigsTarget &t, int status) override {
        Request *q = static_cast<Request *>(t.tag);
        if (t.reused) {
            std::lock_guard<std::mutex> lk(b->mu);
            ++b->hits;
        }
        if (q == first) {   // the worker finishes the request it admitted
            first->status = status;
            return;
        }
        {
            std::lock_guard<std::mutex> lk(b->mu);
            q->t_end = Clock::now();
            q->status = status;
            q->done = true;
            --b->running;
            ++b->finished;
            if (q->r.timing_ms) {
                q->r.timing_ms[0] = ms_since(q->t_submit, q->t_start);
                q->r.timing_ms[1] = ms_since(q->t_start, q->t_end);
                q->r.timing_ms[2] = ms_since(q->t_submit, q->t_end);
            }
        }
        b->cv_done.notify_all();
    }
};

int run_request(kore_batch *b, Request *q, CachedPlan *c) {
    const kore_request &r = q->r;
    if (!c->plan) {
        KORE_TRY(kore_plan_create(r.pencil, b->device, &c->plan));
        std::lock_guard<std::mutex> lk(b->mu);
        ++b->created;
    }
    if (r.kind == KORE_REQ_EIGEN) {
        if (!r.evals || !r.nconv || r.max_pairs <= 0) return KORE_EINVAL;
        // the batched engine on this plan's slots (one slot for an unshared pencil)
        const int nslot = shared_eigen(r) ? kServeSlots : 1;
        if (c->slots != nslot || c->slot_prec != r.precision) {
            c->slots = 0;
            c->factored = false;
            for (bool &v : c->slot_valid) v = false;
            KORE_TRY(kore_factor_reserve(c->plan, nslot, r.precision));
            c->slots = nslot;
            c->slot_prec = r.precision;
        }
        ServeSource src;
        src.b = b; src.c = c; src.first = q;
        q->status = KORE_EPENDING;
        const int rc = kore_eigs_engine(c->plan, &src, c->slot_valid, kServeMaxNcv);
        if (rc != KORE_OK) {
            c->slots = 0;
            for (bool &v : c->slot_valid) v = false;
            return rc;
        }
        // the slots keep their factors: a later request at one of their shifts reuses them
        return q->status;
    }
    if (c->slots != 0) {   // the plan held eigen slots: back to one shift
        c->slots = 0;
        c->slot_prec = -1;
        for (bool &v : c->slot_valid) v = false;
    }
    if (!(c->factored && c->prec == r.precision && c->sre == r.sigma_re && c->sim == r.sigma_im)) {
        c->factored = false;
        KORE_TRY(kore_factor(c->plan, r.sigma_re, r.sigma_im, r.precision));
        c->factored = true;
        c->prec = r.precision;
        c->sre = r.sigma_re;
        c->sim = r.sigma_im;
    }
    if (r.kind != KORE_REQ_FORCED || !r.rhs || !r.x) return KORE_EINVAL;
    const int64_t n = r.pencil->n;
    const double sc = (r.rhs_scale != 0.0) ? 1.0 / r.rhs_scale : 1.0;
    std::vector<double> rhs(r.rhs, r.rhs + 2 * n);
    if (sc != 1.0)
        for (double &v : rhs) v *= sc;
    kore_stats st{};
    int rc = kore_solve(c->plan, rhs.data(), r.x, 1, r.refine_tol, &st);
    // mixed precision: a refinement that stopped above the forced solve's bound (the
    // complex64 factors of a badly conditioned shift do not contract the error) is
    // redone with FP64 factors, which the cache then holds for this shift
    if (rc == KORE_OK && r.precision == KORE_PREC_MIXED && !(st.solve_resid_max <= kForcedEscalateTol)) {
        c->factored = false;
        KORE_TRY(kore_factor(c->plan, r.sigma_re, r.sigma_im, KORE_PREC_FP64));
        c->factored = true;
        c->prec = KORE_PREC_FP64;
        rc = kore_solve(c->plan, rhs.data(), r.x, 1, 0.0, &st);
        st.escalated = 1;
    }
    if (r.stats) *r.stats = st;
    return rc;
}

void worker(kore_batch *b) {
    cudaSetDevice(b->device);
    for (;;) {
        Request *q = nullptr;
        CachedPlan *c = nullptr;
        {
            std::unique_lock<std::mutex> lk(b->mu);
            for (;;) {
                if (b->stop) return;
                if (!b->queue.empty()) {
                    q = admit(b, &c);
                    if (q) break;
                }
                // nothing startable: wait for a new request or a finished one (with a
                // timeout so that the hold-back rule is re-checked)
                b->cv_work.wait_for(lk, std::chrono::milliseconds(20));
            }
            q->t_start = Clock::now();
            if (c) {
                ++b->running;
                if (shared_eigen(q->r)) {
                    c->engine = true;
                    c->engine_prec = q->r.precision;
                }
            }
        }
        int st = q->status;
        if (c) st = run_request(b, q, c);
        {
            std::lock_guard<std::mutex> lk(b->mu);
            q->t_end = Clock::now();
            q->status = st;
            q->done = true;
            if (c) {
                --b->running;
                c->busy = false;
                c->engine = false;
                c->last_use = ++b->clock;
                int64_t actual = 0;
                if (c->plan && kore_plan_bytes(c->plan, &actual) == KORE_OK && actual > c->bytes) {
                    b->used += actual - c->bytes;
                    c->bytes = actual;
                }
                if (st != KORE_OK) c->factored = false;
                if (c->key == 0 || !c->plan || st == KORE_ENOMEM || st == KORE_ECUDA) {
                    // not shared, or in an unknown state: free it
                    b->used -= c->bytes;
                    if (c->plan) kore_plan_destroy(c->plan);
                    for (size_t i = 0; i < b->plans.size(); ++i)
                        if (b->plans[i].get() == c) { b->plans.erase(b->plans.begin() + (std::ptrdiff_t)i); break; }
                }
            }
            ++b->finished;
            if (q->r.timing_ms) {
                q->r.timing_ms[0] = ms_since(q->t_submit, q->t_start);
                q->r.timing_ms[1] = ms_since(q->t_start, q->t_end);
                q->r.timing_ms[2] = ms_since(q->t_submit, q->t_end);
            }
        }
        b->cv_done.notify_all();
        b->cv_work.notify_all();
    }
}

}  // namespace

extern "C" {

int kore_batch_create(int device, int64_t hbm_budget, int workers, kore_batch **out) {
    if (!out || workers <= 0 || workers > 64) return KORE_EINVAL;
    *out = nullptr;
    int prev = -1;
    cudaGetDevice(&prev);
    KORE_CUDA_TRY(cudaSetDevice(device));
    size_t fr = 0, tot = 0;
    const cudaError_t e = cudaMemGetInfo(&fr, &tot);
    if (prev >= 0) cudaSetDevice(prev);
    if (e != cudaSuccess) return KORE_ECUDA;
    auto b = std::make_unique<kore_batch>();
    b->device = device;
    b->budget = (hbm_budget > 0) ? hbm_budget : (int64_t)(0.9 * (double)fr);
    for (int i = 0; i < workers; ++i) b->workers.emplace_back(worker, b.get());
    *out = b.release();
    return KORE_OK;
}

int kore_batch_submit(kore_batch *b, const kore_request *req, uint64_t *ticket) {
    if (!b || !req || !ticket || !req->pencil) return KORE_EINVAL;
    if (req->kind != KORE_REQ_EIGEN && req->kind != KORE_REQ_FORCED) return KORE_EINVAL;
    auto q = std::make_unique<Request>();
    q->r = *req;
    q->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(b->mu);
        if (b->stop) return KORE_EINVAL;
        q->ticket = b->next_ticket++;
        *ticket = q->ticket;
        b->queue.push_back(q.get());
        b->reqs.emplace(q->ticket, std::move(q));
        ++b->submitted;
    }
    b->cv_work.notify_one();
    return KORE_OK;
}

int kore_batch_poll(kore_batch *b, uint64_t ticket, int wait_ms, int *status) {
    if (!b || !status) return KORE_EINVAL;
    std::unique_lock<std::mutex> lk(b->mu);
    auto it = b->reqs.find(ticket);
    if (it == b->reqs.end()) return KORE_EINVAL;
    Request *q = it->second.get();
    if (!q->done) {
        if (wait_ms < 0) b->cv_done.wait(lk, [&] { return q->done; });
        else if (wait_ms > 0) b->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return q->done; });
    }
    if (!q->done) return KORE_EPENDING;
    *status = q->status;
    b->reqs.erase(it);
    return KORE_OK;
}

int kore_batch_stats(kore_batch *b, int64_t *out) {
    if (!b || !out) return KORE_EINVAL;
    std::lock_guard<std::mutex> lk(b->mu);
    out[0] = b->submitted;
    out[1] = b->finished;
    out[2] = b->running;
    out[3] = (int64_t)b->queue.size();
    out[4] = b->used;
    out[5] = b->hits;
    out[6] = b->created;
    out[7] = b->evicted;
    out[8] = b->joined;
    return KORE_OK;
}

int kore_batch_destroy(kore_batch *b) {
    if (!b) return KORE_OK;
    {
        std::lock_guard<std::mutex> lk(b->mu);
        for (Request *q : b->queue) {
            q->status = KORE_ECANCELLED;
            q->done = true;
        }
        b->queue.clear();
        b->stop = true;
    }
    b->cv_work.notify_all();
    b->cv_done.notify_all();
    for (auto &t : b->workers) t.join();
    for (auto &c : b->plans)
        if (c->plan) kore_plan_destroy(c->plan);
    delete b;
    return KORE_OK;
}

}  // extern "C"
