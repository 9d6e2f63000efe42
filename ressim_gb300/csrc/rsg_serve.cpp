// Serving form of the solver: continuous batching of independent Newton systems over worker slots.
//
// Each slot is a host thread with its own solver handle (own CUDA stream, own device memory). Requests wait in
// arrival order; the head of the queue is admitted as soon as a slot is free and its estimated device footprint
// fits in what the admitted requests leave of the budget. A small head (one SM's worth of rows) takes the small
// requests queued behind it along, up to 64, and the slot solves them in one block-diagonal batch. Admitted requests run concurrently on their slots'
// streams, so a request that arrives while others are on the GPU overlaps with them on the device; its matrix,
// factors, hierarchy and Krylov state stay resident until it completes, and the slot then keeps the plan for the
// next request of the same pattern (counted against the budget; released, stream-ordered, when an admission needs
// the room). A request is solved exactly as it would be alone: a plan that depends on its pattern only,
// deterministic kernels, nothing shared with the other slots but the device.
#include "rsg.h"
#include "rsg_impl.h"

#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

namespace rsg {
void set_last_error(const std::string& msg);
}

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    long long id = 0;
    int n = 0, nb = 0;
    std::vector<int> rp, ci;                  // the server's copy (rsg_submit); empty when the caller lends its arrays
    std::vector<double> val, b, x;
    const int* prp = nullptr;                 // what the solve reads: the copy, or the caller's arrays (rsg_submit_view)
    const int* pci = nullptr;
    const double* pval = nullptr;
    const double* pb = nullptr;
    double tol = 1e-6;
    int maxit = 100;
    size_t est = 0;
    bool done = false;
    rsg_result res{};
    Clock::time_point tSubmit, tStart, tEnd;
};

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// Device bytes a request will hold (an upper estimate of what its handle allocates: values twice, factors and
// their slot copy, plan arrays, Krylov vectors, CPR hierarchy and second-stage arrays, GMRES basis).
size_t footprint(int n, long long nnzb, const rsg_options& o) {
    const double N = double(n), E = double(nnzb);
    double bytes = E * (2 * 72.0 + 100.0) + N * 700.0;           // values + staging, plan arrays, level / slot plan
    bytes += o.precision == RSG_FP64 ? E * 72.0 + N * 512.0 : E * 108.0 + N * 256.0;   // factors (+ lean work)
    bytes += N * 3 * 8 * 14;                                      // Krylov and staging vectors
    if (o.precond == RSG_PREC_CPR || o.precond == RSG_PREC_CPR_DEVICE) bytes += E * 40.0 + N * 600.0;
    if (o.krylov == RSG_KRYLOV_GMRES || o.gmres_fallback) bytes += N * 3 * 8 * (2.0 * (o.restart > 0 ? o.restart : 40) + 3);
    return size_t(bytes) + (size_t(16) << 20);
}

}  // namespace

struct rsg_server {
    rsg_options opt{};
    int slots = 1;
    size_t budget = 0;
    std::mutex mu;
    std::condition_variable cvWork, cvDone;
    std::deque<std::shared_ptr<Request>> queue;
    std::unordered_map<long long, std::shared_ptr<Request>> live;
    size_t inUse = 0;
    int running = 0;
    long long nextId = 0;
    bool stop = false;
    bool hold = false;                        // admission paused (rsg_server_hold)
    std::vector<std::thread> workers;
    std::vector<rsg_solver*> handles, grid, bilu;   // per slot: the configured handle (batches of small requests), one
                                                    // with the grid-wide sweeps (larger requests), and two BILU0 handles
                                                    // (thread-block and grid-wide sweeps) for patterns CPR cannot take
    // Resident plans: after a request (or batch) a handle keeps its plan -- pattern plan, hierarchy, factors, Krylov
    // state -- so that the next request with the same pattern (the next Newton iteration of a simulator, or the
    // same ensemble at the next step) only uploads values, as the engine reuses its Schur plan by pattern hash
    // (engine/src/bsr.cpp:759-769). A resident plan counts against the budget; when an admission needs its room,
    // the plans of idle slots are released first. cached[4 * slot + k]: bytes held by handle k of the slot
    // (0 handles, 1 grid, 2 and 3 bilu), idle; busy[slot]: the slot is running work.
    std::vector<size_t> cached;
    std::vector<char> busy;
    size_t cachedTotal = 0;
    Clock::time_point t0 = Clock::now();      // the server's clock origin (start_ms / end_ms of the results)
};

namespace {

// A request of at most kBatchRows block rows runs on one SM (thread-block sweeps) and is batched with the small
// requests queued behind it; a larger one is solved alone by the grid-wide sweeps, where a lone system gets the whole
// GPU. The choice depends on the request alone, so its result does not depend on what else is queued.
constexpr int kBatchRows = 32768;
constexpr int kMaxBatch = 64;
constexpr long long kMaxBatchRowsTotal = 1 << 21;

void run_request(rsg_server* S, int slot, Request& R) {
    rsg_solver* h = R.n > kBatchRows && S->grid[size_t(slot)] ? S->grid[size_t(slot)] : S->handles[size_t(slot)];
    int prec = S->opt.precond;
    int rc = rsg_set_matrix(h, R.n, R.nb, R.prp, R.pci, R.pval);
    if (rc == RSG_OK) rc = rsg_setup(h, nullptr);
    if (rc == RSG_EINVAL && (prec == RSG_PREC_CPR || prec == RSG_PREC_CPR_DEVICE)) {   // CPR needs a structurally symmetric pattern: BILU0
        rsg_release(h);
        const bool large = R.n > kBatchRows;                      // the grid-wide sweeps for a large request, as for CPR
        rsg_solver*& fb = S->bilu[size_t(2 * slot + (large ? 1 : 0))];
        if (!fb) {
            rsg_options o = S->opt;
            o.precond = RSG_PREC_BILU0;
            if (large) o.sweep = 2;
            rsg_create(&fb, &o);
        }
        if (fb) {
            h = fb;
            prec = RSG_PREC_BILU0;
            rc = rsg_set_matrix(h, R.n, R.nb, R.prp, R.pci, R.pval);
            if (rc == RSG_OK) rc = rsg_setup(h, nullptr);
        }
    }
    R.res.precond = prec;
    R.res.slot = slot;
    int its = 0;
    double rr = 0;
    if (rc == RSG_OK) {
        R.x.assign(size_t(R.n) * size_t(R.nb), 0.0);
        rc = rsg_solve(h, R.pb, R.x.data(), R.tol, R.maxit, &its, &rr);
    }
    rsg_stats st{};
    rsg_get_stats(h, &st);
    R.res.status = rc;
    R.res.iterations = its;
    R.res.rel_residual = rr;
    R.res.true_rel_residual = rc >= 0 ? st.true_rel_residual : -1.0;
    R.res.device_bytes = st.device_bytes;
}


// Small requests of a batch: one block-diagonal solve (every system's kernels and reductions are its own, so each
// result is the one it has alone). Patterns the batch cannot take (CPR on a pattern that is not structurally
// symmetric) fall back to one request at a time.
void run_batch(rsg_server* S, int slot, std::vector<std::shared_ptr<Request>>& B) {
    rsg_solver* h = S->handles[size_t(slot)];
    const int ns = int(B.size());
    const size_t nsz = static_cast<size_t>(ns);
    std::vector<int> n(nsz);
    std::vector<const int*> rp(nsz), ci(nsz);
    std::vector<const double*> val(nsz);
    std::vector<double> b, x;
    for (int k = 0; k < ns; ++k) {
        Request& R = *B[size_t(k)];
        n[size_t(k)] = R.n;
        rp[size_t(k)] = R.prp;
        ci[size_t(k)] = R.pci;
        val[size_t(k)] = R.pval;
        b.insert(b.end(), R.pb, R.pb + size_t(R.n) * size_t(R.nb));
    }
    int rc = rsg_set_batch(h, ns, rsg::NB, n.data(), rp.data(), ci.data(), val.data());
    if (rc == RSG_OK) rc = rsg_setup(h, nullptr);
    if (rc != RSG_OK) {
        rsg_release(h);
        for (auto& R : B) run_request(S, slot, *R);
        return;
    }
    x.assign(b.size(), 0.0);
    int its = 0;
    double rr = 0;
    rc = rsg_solve(h, b.data(), x.data(), B[0]->tol, B[0]->maxit, &its, &rr);
    std::vector<int> sits(nsz), sst(nsz, rc < 0 ? rc : RSG_OK);
    std::vector<double> srr(nsz), strue(nsz, -1.0);
    if (rc >= 0) {
        rsg_batch_results(h, sits.data(), srr.data(), strue.data());
        rsg_batch_status(h, sst.data());
    }
    rsg_stats st{};
    rsg_get_stats(h, &st);
    size_t off = 0;
    for (int k = 0; k < ns; ++k) {
        Request& R = *B[size_t(k)];
        const size_t N = size_t(R.n) * size_t(R.nb);
        R.x.assign(x.begin() + long(off), x.begin() + long(off + N));
        off += N;
        R.res.status = sst[size_t(k)];
        R.res.iterations = sits[size_t(k)];
        R.res.rel_residual = srr[size_t(k)];
        R.res.true_rel_residual = strue[size_t(k)];
        R.res.device_bytes = st.device_bytes;
        R.res.precond = S->opt.precond;
        R.res.slot = slot;
        R.res.batch = ns;
    }
}

rsg_solver* slot_handle(rsg_server* S, int slot, int k) {
    if (k == 0) return S->handles[size_t(slot)];
    if (k == 1) return S->grid[size_t(slot)];
    return S->bilu[size_t(2 * slot + (k - 2))];
}

// release idle resident plans (other slots first, then the caller's own) until `need` more bytes fit; with S->mu held
void evict_idle(rsg_server* S, int self, size_t need) {
    for (int pass = 0; pass < 2; ++pass)
        for (int q = 0; q < S->slots; ++q) {
            if ((pass == 0) == (q == self) || S->busy[size_t(q)]) continue;
            for (int k = 0; k < 4; ++k) {
                if (S->inUse + S->cachedTotal + need <= S->budget) return;
                size_t& c = S->cached[size_t(4 * q + k)];
                if (!c) continue;
                rsg_release(slot_handle(S, q, k));
                S->cachedTotal -= c;
                c = 0;
            }
        }
}

// the work of a slot takes the resident plan of the handle it runs on over: that plan is now part of the running
// footprint (a plan for another pattern is freed by the set-up of the new one before it allocates); the slot's other
// handles keep theirs, still counted
void take_cached(rsg_server* S, int slot, int k) {
    size_t& c = S->cached[size_t(4 * slot + k)];
    S->cachedTotal -= c;
    c = 0;
}

// after a run: what each of the slot's handles holds stays resident (idle)
void keep_cached(rsg_server* S, int slot) {
    for (int k = 0; k < 4; ++k) {
        rsg_solver* h = slot_handle(S, slot, k);
        size_t& c = S->cached[size_t(4 * slot + k)];
        S->cachedTotal -= c;
        c = 0;
        if (!h) continue;
        rsg_stats st{};
        rsg_get_stats(h, &st);
        c = st.device_bytes;
        S->cachedTotal += c;
    }
}

void worker(rsg_server* S, int slot) {
    for (;;) {
        std::vector<std::shared_ptr<Request>> B;
        size_t est = 0;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cvWork.wait(lk, [&] {
                if (S->stop) return true;
                if (S->queue.empty() || S->hold) return false;
                const size_t e = S->queue.front()->est;
                if (S->budget == 0) return true;
                if (S->running > 0 && S->inUse + e > S->budget) return false;
                if (S->inUse + S->cachedTotal + e > S->budget) evict_idle(S, slot, e);
                return true;                                      // alone on the device: admitted whatever its size
            });
            if (S->stop) return;
            S->busy[size_t(slot)] = 1;
            B.push_back(S->queue.front());
            S->queue.pop_front();
            est = B[0]->est;
            if (B[0]->n <= kBatchRows) {                         // gather the small requests queued behind it
                long long rows = B[0]->n;
                while (!S->queue.empty() && int(B.size()) < kMaxBatch) {
                    const auto& F = S->queue.front();
                    if (F->n > kBatchRows || F->tol != B[0]->tol || F->maxit != B[0]->maxit || rows + F->n > kMaxBatchRowsTotal) break;
                    if (S->budget && S->inUse + S->cachedTotal + est + F->est > S->budget) break;
                    rows += F->n;
                    est += F->est;
                    B.push_back(F);
                    S->queue.pop_front();
                }
            }
            S->inUse += est;
            S->running += int(B.size());
            take_cached(S, slot, B.size() == 1 && B[0]->n > kBatchRows && S->grid[size_t(slot)] ? 1 : 0);
        }
        S->cvWork.notify_all();                                   // the next head may fit as well
        const Clock::time_point t0 = Clock::now();
        if (B.size() == 1) {
            run_request(S, slot, *B[0]);
            B[0]->res.batch = 1;
        } else {
            run_batch(S, slot, B);
        }
        const Clock::time_point t1 = Clock::now();
        for (auto& R : B) {
            R->tStart = t0;
            R->tEnd = t1;
            R->res.queue_ms = ms_between(R->tSubmit, t0);
            R->res.run_ms = ms_between(t0, t1);
            R->res.total_ms = ms_between(R->tSubmit, t1);
            R->res.start_ms = ms_between(S->t0, t0);
            R->res.end_ms = ms_between(S->t0, t1);
        }
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->inUse -= est;
            S->running -= int(B.size());
            keep_cached(S, slot);
            S->busy[size_t(slot)] = 0;
            for (auto& R : B) R->done = true;
        }
        S->cvDone.notify_all();
        S->cvWork.notify_all();
    }
}

}  // namespace

extern "C" {

int rsg_server_create(rsg_server** out, const rsg_options* opts, int slots, size_t mem_budget) {
    using rsg::set_last_error;
    if (!out) { set_last_error("null server pointer"); return RSG_EINVAL; }
    *out = nullptr;
    if (slots < 1 || slots > 256) { set_last_error("slots must be in [1, 256]"); return RSG_EINVAL; }
    rsg_server* S = new rsg_server();
    rsg_default_options(&S->opt);
    if (opts) S->opt = *opts;
    S->opt.mem_budget = 0;                                        // the server accounts for the budget
    S->slots = slots;
    S->budget = mem_budget;
    S->handles.assign(size_t(slots), nullptr);
    S->cached.assign(size_t(4 * slots), 0);
    S->busy.assign(size_t(slots), 0);
    S->grid.assign(size_t(slots), nullptr);
    S->bilu.assign(size_t(2 * slots), nullptr);
    rsg_options og = S->opt;
    og.sweep = 2;
    for (int i = 0; i < slots; ++i) {
        int rc = rsg_create(&S->handles[size_t(i)], &S->opt);
        if (rc == RSG_OK) rc = rsg_create(&S->grid[size_t(i)], &og);
        if (rc != RSG_OK) {
            for (rsg_solver* h : S->handles) rsg_destroy(h);
            for (rsg_solver* h : S->grid) rsg_destroy(h);
            delete S;
            return rc;                                            // the handle's message stays in rsg_last_error
        }
    }
    for (int i = 0; i < slots; ++i) S->workers.emplace_back(worker, S, i);
    *out = S;
    return RSG_OK;
}

int rsg_server_destroy(rsg_server* S) {
    if (!S) return RSG_OK;
    {
        std::unique_lock<std::mutex> lk(S->mu);
        for (auto& R : S->queue) {                                // dropped: a waiting poll returns RSG_ESTATE
            R->done = true;
            R->res.status = RSG_ESTATE;
        }
        S->queue.clear();
        S->cvDone.notify_all();
        S->cvDone.wait(lk, [&] { return S->running == 0; });
        S->stop = true;
    }
    S->cvWork.notify_all();
    for (auto& t : S->workers) t.join();
    for (rsg_solver* h : S->handles) rsg_destroy(h);
    for (rsg_solver* h : S->grid) rsg_destroy(h);
    for (rsg_solver* h : S->bilu) rsg_destroy(h);
    delete S;
    return RSG_OK;
}

}  // extern "C"

namespace {

// Queues one request. copy: the server keeps its own copy of the arrays (the caller may reuse them at once);
// otherwise it reads the caller's arrays in place until the request has finished.
long long submit(rsg_server* S, int n, int nb, const int* rowPtr, const int* col, const double* val, const double* b, double tol,
                 int maxIt, bool copy) {
    using rsg::set_last_error;
    if (!S || !rowPtr || !col || !val || !b) { set_last_error("null argument"); return RSG_EINVAL; }
    if (n <= 0 || nb != rsg::NB) { set_last_error("n must be > 0 and nb = 3"); return RSG_EINVAL; }
    const long long nnzb = rowPtr[n];
    if (nnzb <= 0) { set_last_error("empty matrix"); return RSG_EINVAL; }
    const size_t est = footprint(n, nnzb, S->opt);
    if (S->budget && est > S->budget) {
        set_last_error("request needs about " + std::to_string(est >> 20) + " MiB, more than the whole budget");
        return RSG_ENOMEM;
    }
    auto R = std::make_shared<Request>();
    R->n = n;
    R->nb = nb;
    if (copy) {
        R->rp.assign(rowPtr, rowPtr + n + 1);
        R->ci.assign(col, col + nnzb);
        R->val.assign(val, val + nnzb * nb * nb);
        R->b.assign(b, b + size_t(n) * size_t(nb));
        R->prp = R->rp.data();
        R->pci = R->ci.data();
        R->pval = R->val.data();
        R->pb = R->b.data();
    } else {
        R->prp = rowPtr;
        R->pci = col;
        R->pval = val;
        R->pb = b;
    }
    R->tol = tol;
    R->maxit = maxIt;
    R->est = est;
    R->tSubmit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        R->id = S->nextId++;
        S->live[R->id] = R;
        S->queue.push_back(R);
    }
    S->cvWork.notify_all();
    return R->id;
}

}  // namespace

extern "C" {

long long rsg_submit(rsg_server* S, int n, int nb, const int* rowPtr, const int* col, const double* val, const double* b, double tol,
                     int maxIt) {
    return submit(S, n, nb, rowPtr, col, val, b, tol, maxIt, true);
}

long long rsg_submit_view(rsg_server* S, int n, int nb, const int* rowPtr, const int* col, const double* val, const double* b,
                          double tol, int maxIt) {
    return submit(S, n, nb, rowPtr, col, val, b, tol, maxIt, false);
}

int rsg_poll(rsg_server* S, long long id, int wait, double* x, rsg_result* res) {
    using rsg::set_last_error;
    if (!S) { rsg::set_last_error("null server"); return RSG_EINVAL; }
    std::shared_ptr<Request> R;
    {
        std::unique_lock<std::mutex> lk(S->mu);
        auto it = S->live.find(id);
        if (it == S->live.end()) { set_last_error("unknown request id"); return RSG_EINVAL; }
        R = it->second;
        if (!R->done) {
            if (!wait) return 0;
            S->cvDone.wait(lk, [&] { return R->done; });
        }
        S->live.erase(id);
    }
    if (x && !R->x.empty()) std::copy(R->x.begin(), R->x.end(), x);
    if (res) *res = R->res;
    return 1;
}

size_t rsg_request_bytes(const rsg_options* opts, int n, long long nnzb) {
    rsg_options o;
    rsg_default_options(&o);
    if (opts) o = *opts;
    return footprint(n, nnzb, o);
}

int rsg_server_hold(rsg_server* S, int hold) {
    if (!S) { rsg::set_last_error("null server"); return RSG_EINVAL; }
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->hold = hold != 0;
    }
    S->cvWork.notify_all();
    return RSG_OK;
}

int rsg_server_load(rsg_server* S, int* queued, int* running, size_t* bytes) {
    if (!S) return RSG_EINVAL;
    std::lock_guard<std::mutex> lk(S->mu);
    if (queued) *queued = int(S->queue.size());
    if (running) *running = S->running;
    if (bytes) *bytes = S->inUse + S->cachedTotal;
    return RSG_OK;
}

}  // extern "C"
