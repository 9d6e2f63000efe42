// C ABI of the rsg solver: handle lifecycle, uploads with pattern reuse, device set-up, Krylov drivers.
#include "rsg.h"
#include "rsg_impl.h"
#include "rsg_generic.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <future>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

using namespace rsg;

namespace {
thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

}  // namespace

namespace rsg {
// error text for entry points outside this file (thread-local, read by rsg_last_error)
void set_last_error(const std::string& msg) { g_err = msg; }
}  // namespace rsg

namespace {

#define RSG_CUDA(call)                                                                                  \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) return fail(RSG_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Device allocations of a handle, stream-ordered on the handle's stream (cudaMallocAsync / cudaFreeAsync): a
// handle that frees its plan does not synchronise the device under the other handles' work (serving slots).
struct DevMem {
    std::vector<std::pair<void*, size_t>> blocks;
    size_t bytes = 0, budget = 0;
    cudaStream_t st = nullptr;
    int alloc(void** p, size_t n) {
        if (n == 0) n = 16;
        if (budget && bytes + n > budget) return fail(RSG_ENOMEM, "device memory budget exhausted");
        cudaError_t e = cudaMallocAsync(p, n, st);
        if (e != cudaSuccess) return fail(RSG_ENOMEM, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
        blocks.push_back({*p, n});
        bytes += n;
        return RSG_OK;
    }
    void release(void* p) {
        if (!p) return;
        for (size_t k = 0; k < blocks.size(); ++k)
            if (blocks[k].first == p) {
                cudaFreeAsync(p, st);
                bytes -= blocks[k].second;
                blocks.erase(blocks.begin() + long(k));
                return;
            }
    }
    void release_all() {
        for (auto& b : blocks) cudaFreeAsync(b.first, st);
        blocks.clear();
        bytes = 0;
    }
};

template <class T>
int dalloc(DevMem& M, T** p, size_t count) {
    return M.alloc(reinterpret_cast<void**>(p), count * sizeof(T));
}
}  // namespace

struct rsg_solver {
    rsg_options opt{};
    int device = 0;
    cudaStream_t stream = nullptr;
    DevMem mem;
    DevMem pmem;                 // pattern-plan allocations (freed on pattern change)
    // plan
    HostPlan plan;
    DevPlan dp;
    bool havePlan = false, haveMatrix = false, haveSetup = false;
    int nsys = 0;
    // matrix values and preconditioner storage
    double* val = nullptr;
    double* lu = nullptr;
    float* luf = nullptr;
    double* work = nullptr;
    double* dinv = nullptr;
    SplitFactors<double> s64;
    SplitFactors<float> s32;
    bool cta = false;
    bool splitCpr = false;       // CPR on the thread-block path: V-cycle grid-wide (PrecDev::split)
    bool escalated = false;      // precision form: failed systems re-solved with FP64 sweep vectors (until the next set-up)
    // CPR: device AMG of the batch (allocated in pmem; built at the first CPR set-up of a pattern)
    DevAmg amg;
    bool haveAmg = false;
    int amgLevels = 0;
    int* d_nfb = nullptr;
    // vectors
    BicgVecs V{};
    double *b = nullptr, *xout = nullptr, *tmp = nullptr;   // level-space b / x, original-order staging
    double* val0 = nullptr;      // matrix values as uploaded (original block order), gathered into val
    // sync-free state, reductions, scalars
    SweepState S{};
    ReduceState R{};
    KScal* ks = nullptr;
    int* d_active = nullptr;
    int* d_err = nullptr;
    int* d_nreg = nullptr;
    double* d_trueres = nullptr;
    int* h_pin = nullptr;        // pinned: [0] active, [1] err, [2] nreg
    int epoch = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // graph of `check_every` iterations
    cudaGraphExec_t gexec = nullptr;
    int gIters = 0, gKind = -1;
    // GMRES (allocated at the first GMRES solve of a plan): state, graphs of its phases
    // ([0] cycle start, [1 + j] inner step j, [m + 1] cycle end), BiCGSTAB result kept for the fallback
    GmState gm{};
    std::vector<cudaGraphExec_t> gmExec;
    int gmKind = -1;
    double* xPrev = nullptr;
    KScal* ksPrev = nullptr;
    // FP64 defect correction (rsg_solve_refined): level-space b, accumulated x, residual, per-system relative residual
    double *refB = nullptr, *refX = nullptr, *refR = nullptr, *refRel = nullptr;
    // results
    rsg_stats st{};
    long long launches = 0;
    std::vector<KScal> hks;
    std::vector<double> htrue;
    // launch shapes (every choice gives the same results bit for bit) and how they were chosen
    struct Tune {
        int split = -1;              // CPR form on the thread-block path: -1 as planned (splitCpr), 0 one kernel, 1 split
        int vform = 3;
        int cpr2Threads = 256;
        std::string desc = "defaults";
    } tune;
    unsigned long long patHash = 0;   // FNV-1a of the plan's pattern (0: not computed)
    // device well Schur complement (rsg_set_jacobian*): host plan, its device copy (pattern part and value maps), the
    // Jacobian values (or the caller's device pointer), full and reduced vectors of the solve
    WsPlan ws;
    WsDev wsd;
    DevMem wsPat, wsVal;
    bool wsPlanned = false, wsValues = false, jac = false;
    double* jval = nullptr;
    const double* jv = nullptr;
    double *wsB = nullptr, *wsX = nullptr, *wsBc = nullptr, *wsXc = nullptr;
    // block sizes other than 3 (compositional / thermal callers): the block-size-generic path, one system per handle
    GenEngine* gen = nullptr;
    bool genActive = false;
    std::mutex mu;
};

namespace {

void drop_gm_graphs(rsg_solver* h);

void free_plan(rsg_solver* h) {
    if (h->gexec) { cudaGraphExecDestroy(h->gexec); h->gexec = nullptr; }
    drop_gm_graphs(h);
    h->gmExec.clear();
    h->gm = GmState{}; h->gmKind = -1; h->xPrev = nullptr; h->ksPrev = nullptr;
    h->refB = h->refX = h->refR = h->refRel = nullptr;
    h->pmem.release_all();
    h->dp = DevPlan{};
    h->val = nullptr; h->lu = nullptr; h->luf = nullptr; h->work = nullptr; h->dinv = nullptr;
    h->s64 = SplitFactors<double>{}; h->s32 = SplitFactors<float>{}; h->cta = false;
    h->amg = DevAmg{}; h->haveAmg = false; h->amgLevels = 0; h->d_nfb = nullptr;
    h->V = BicgVecs{};
    h->b = h->xout = h->tmp = nullptr;
    h->S = SweepState{};
    h->R = ReduceState{};
    h->ks = nullptr; h->d_trueres = nullptr;
    h->havePlan = h->haveMatrix = h->haveSetup = false;
    if (h->gen) { gen_destroy(h->gen); h->gen = nullptr; }
    h->genActive = false;
}

template <class T>
int upload(DevMem& M, T** d, const std::vector<T>& v, cudaStream_t st, size_t pad = 0) {
    int rc = dalloc(M, d, v.size() + pad);
    if (rc) return rc;
    if (!v.empty()) RSG_CUDA(cudaMemcpyAsync(*d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    return RSG_OK;
}

int alloc_plan(rsg_solver* h) {
    HostPlan& P = h->plan;
    DevMem& M = h->pmem;
    M.budget = h->opt.mem_budget ? (h->opt.mem_budget > h->mem.bytes ? h->opt.mem_budget - h->mem.bytes : 1) : 0;
    DevPlan& D = h->dp;
    cudaStream_t st = h->stream;
    D.n = P.n; D.nnzb = P.nnzb; D.nsys = P.nsys; D.ntiles = int(P.tileSys.size());
    int rc;
    if ((rc = upload(M, &D.rowPtr, P.rowPtr, st)) || (rc = upload(M, &D.col, P.col, st)) || (rc = upload(M, &D.diag, P.diag, st)) ||
        (rc = upload(M, &D.ford, P.ford, st)) || (rc = upload(M, &D.bord, P.bord, st)) || (rc = upload(M, &D.elimPtr, P.elimPtr, st)) ||
        (rc = upload(M, &D.elimT, P.elimT, st)) || (rc = upload(M, &D.elimQ, P.elimQ, st)) || (rc = upload(M, &D.rowSys, P.rowSys, st)) ||
        (rc = upload(M, &D.tileRow0, P.tileRow0, st)) || (rc = upload(M, &D.tileSys, P.tileSys, st)) ||
        (rc = upload(M, &D.sysTile0, P.sysTile0, st)) || (rc = upload(M, &D.sysRow0, P.sysRow0, st)) ||
        (rc = upload(M, &D.perm, P.perm, st)) || (rc = upload(M, &D.valSrc, P.valSrc, st)) ||
        (rc = upload(M, &D.lvlStart, P.lvlStart, st)) || (rc = upload(M, &D.sysLvl0, P.sysLvl0, st)) ||
        (rc = upload(M, reinterpret_cast<int**>(&D.Lslot), P.Lslot, st)) || (rc = upload(M, &D.LslotSrc, P.LslotSrc, st)) ||
        (rc = upload(M, &D.LovCol, P.LovCol, st)) || (rc = upload(M, &D.LovSrc, P.LovSrc, st)) ||
        (rc = upload(M, reinterpret_cast<int**>(&D.Uslot), P.Uslot, st)) || (rc = upload(M, &D.UslotSrc, P.UslotSrc, st)) ||
        (rc = upload(M, &D.UovCol, P.UovCol, st)) || (rc = upload(M, &D.UovSrc, P.UovSrc, st)) || (rc = upload(M, &D.Dsrc, P.Dsrc, st)))
        return rc;
    {   // (first row, rows) of every row's forward level: the component-major layout of the sweep records
        std::vector<int> rl(size_t(P.n) * 2, 0);
        for (int sy = 0; sy < P.nsys; ++sy)
            for (int q = P.sysLvl0[size_t(sy)]; q + 1 < P.sysLvl0[size_t(sy) + 1]; ++q)
                for (int k = P.lvlStart[size_t(q)]; k < P.lvlStart[size_t(q) + 1]; ++k) {
                    rl[size_t(k) * 2] = P.lvlStart[size_t(q)];
                    rl[size_t(k) * 2 + 1] = P.lvlStart[size_t(q) + 1] - P.lvlStart[size_t(q)];
                }
        if ((rc = upload(M, reinterpret_cast<int**>(&D.rowLevel), rl, st))) return rc;
    }
    D.spmvFma = h->opt.fma != 0;
    D.nLov = int(P.LovCol.size());
    D.nUov = int(P.UovCol.size());
    D.maxSysRows = P.maxSysRows;
    {
        int maxLv = 1;
        for (int s = 0; s < P.nsys; ++s) maxLv = std::max(maxLv, P.sysLvl0[size_t(s) + 1] - P.sysLvl0[size_t(s)] - 1);
        D.sweepBlocks = sweep_blocks_for(double(P.n) / double(maxLv), h->opt.sweep_inflight);
    }
    h->cta = h->opt.sweep != 2 && cta_sweep_supported(D, P);
    if ((h->opt.sweep == 1 || h->opt.sweep == 3) && !h->cta)
        return fail(RSG_EINVAL, "thread-block sweeps need a structurally symmetric pattern of <= 32768 block rows per system");
    // CPR on the thread-block path: for a batch, the V-cycle's passes grid-wide (all systems at once, the whole
    // GPU's loads in flight); a single system keeps the one-kernel form (one launch per application instead of a
    // launch per pass). Both give the same results bit for bit, so a system's result does not depend on its batch.
    h->splitCpr = h->cta && (h->opt.sweep == 3 || (h->opt.sweep == 0 && P.nsys > 1));
    const size_t N = size_t(P.n) * NB, E = size_t(P.nnzb) * NB2;
    if ((rc = dalloc(M, &h->val, E)) || (rc = dalloc(M, &h->val0, E)) || (rc = dalloc(M, &h->b, N)) || (rc = dalloc(M, &h->xout, N)) ||
        (rc = dalloc(M, &h->tmp, N)))
        return rc;
    double** vecs[] = {&h->V.x, &h->V.r, &h->V.rh, &h->V.p, &h->V.v, &h->V.s, &h->V.t, &h->V.ph, &h->V.sh};
    for (double** v : vecs)
        if ((rc = dalloc(M, v, N))) return rc;
    if ((rc = dalloc(M, &h->S.flagF, size_t(P.n))) || (rc = dalloc(M, &h->S.flagB, size_t(P.n))) ||
        (rc = dalloc(M, &h->S.flagL, size_t(P.n))) || (rc = dalloc(M, &h->S.ctr, 4)))
        return rc;
    RSG_CUDA(cudaMemsetAsync(h->S.flagF, 0, sizeof(int) * size_t(P.n), st));
    RSG_CUDA(cudaMemsetAsync(h->S.flagB, 0, sizeof(int) * size_t(P.n), st));
    RSG_CUDA(cudaMemsetAsync(h->S.flagL, 0, sizeof(int) * size_t(P.n), st));
    RSG_CUDA(cudaMemsetAsync(h->S.ctr, 0, sizeof(unsigned) * 4, st));
    if ((rc = dalloc(M, &h->R.part, size_t(D.ntiles) * MAX_DOTS)) || (rc = dalloc(M, &h->R.done, 1)) ||
        (rc = dalloc(M, &h->R.sysdot, size_t(P.nsys) * MAX_DOTS)) || (rc = dalloc(M, &h->ks, size_t(P.nsys))) ||
        (rc = dalloc(M, &h->d_trueres, size_t(P.nsys))))
        return rc;
    RSG_CUDA(cudaMemsetAsync(h->R.done, 0, sizeof(unsigned), st));
    RSG_CUDA(cudaMemsetAsync(h->ks, 0, sizeof(KScal) * size_t(P.nsys), st));
    h->epoch = 0;
    h->havePlan = true;
    return RSG_OK;
}

// device-side status after a kernel sequence: timeouts become RSG_ETIMEOUT and the sweep state is reset
int check_device_errors(rsg_solver* h) {
    RSG_CUDA(cudaMemcpyAsync(h->h_pin + 1, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    RSG_CUDA(cudaStreamSynchronize(h->stream));
    if (h->h_pin[1] != 0) {
        const int e = h->h_pin[1];
        cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream);
        cudaMemsetAsync(h->S.flagF, 0, sizeof(int) * size_t(h->plan.n), h->stream);
        cudaMemsetAsync(h->S.flagB, 0, sizeof(int) * size_t(h->plan.n), h->stream);
        cudaMemsetAsync(h->S.ctr, 0, sizeof(unsigned) * 4, h->stream);
        cudaMemsetAsync(h->R.done, 0, sizeof(unsigned), h->stream);
        if (h->V.yt) cudaMemsetAsync(h->V.yt, 0, size_t(h->plan.n) * NB * sizeof(unsigned long long), h->stream);
        if (h->amg.gsFlag) {
            cudaMemsetAsync(h->amg.gsFlag, 0, 2 * size_t(std::max(h->amg.totRows, 1)) * sizeof(int), h->stream);
            cudaMemsetAsync(h->amg.gsCtr, 0, 4 * size_t(std::max(h->amg.maxL, 1)) * sizeof(unsigned), h->stream);
        }
        cudaStreamSynchronize(h->stream);
        if (e & ERR_TIMEOUT) return fail(RSG_ETIMEOUT, "a bounded device wait ran out (sweep dependency not satisfied)");
        return fail(RSG_ECUDA, "device error flag " + std::to_string(e));
    }
    return RSG_OK;
}

// kernel launches of one preconditioner application
int precond_launches(const PrecDev& M) {
    if (M.devcpr) return devcpr_launches(*M.amg);
    if (M.cpr && (!M.cta || M.split)) return cpr_grid_launches(*M.amg, M.split, M.vform);
    return M.cpr || M.cta || M.kind == 2 ? 1 : 2;
}

PrecDev prec_dev(rsg_solver* h) {
    PrecDev M;
    if (h->opt.precond == RSG_PREC_JACOBI) { M.kind = 2; M.dinv = h->dinv; }
    else if (h->opt.precision == RSG_MIXED) { M.kind = 1; M.luf = h->luf; }
    else if (h->opt.precision == RSG_MIXED_F32) { M.kind = h->escalated ? 1 : 3; M.luf = h->luf; }
    else { M.kind = 0; M.lu = h->lu; }
    M.val = h->val;
    M.y32 = h->V.y32;
    M.yt = h->V.yt;
    if (h->opt.precond == RSG_PREC_CPR && h->haveAmg) { M.cpr = true; M.amg = &h->amg; }
    if (h->opt.precond == RSG_PREC_CPR_DEVICE) { M.devcpr = true; M.kind = 4; M.amg = &h->amg; return M; }
    if (M.kind != 2 && h->cta) {
        M.smem = cta_sweep_smem(h->dp, M.kind == 3);
        M.cta = true;
        M.s64 = h->s64;
        M.s32 = h->s32;
        M.split = M.cpr && (h->tune.split >= 0 ? h->tune.split != 0 : h->splitCpr);
        M.vform = h->tune.vform;
        M.cpr2Threads = h->tune.cpr2Threads;
    }
    return M;
}

int set_values(rsg_solver* h, const std::vector<const double*>& vals, const std::vector<int>& nnzbs) {
    size_t off = 0;
    for (size_t s = 0; s < vals.size(); ++s) {
        const size_t cnt = size_t(nnzbs[s]) * NB2;
        if (cnt) RSG_CUDA(cudaMemcpyAsync(h->val0 + off, vals[s], cnt * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        off += cnt;
    }
    launch_gather_blocks(h->dp, h->val0, h->val, h->stream);   // into level space
    h->launches += 1;
    RSG_CUDA(cudaGetLastError());
    h->haveMatrix = true;
    h->haveSetup = false;
    return RSG_OK;
}

// the plan of a batch pattern (kept when the pattern is the plan's); nnzbs gets the blocks of every system
int set_batch_pattern(rsg_solver* h, int nsys, const int* n, const int* const* rowPtr, const int* const* col, std::vector<int>& nnzbs) {
    std::vector<int> sysRow0(size_t(nsys) + 1, 0);
    for (int s = 0; s < nsys; ++s) {
        if (n[s] < 1 || !rowPtr[s] || !col[s]) return fail(RSG_EINVAL, "set_batch: system " + std::to_string(s) + " is empty");
        sysRow0[size_t(s) + 1] = sysRow0[size_t(s)] + n[s];
    }
    nnzbs.assign(static_cast<size_t>(nsys), 0);
    for (int s = 0; s < nsys; ++s) nnzbs[size_t(s)] = rowPtr[s][n[s]];
    // the pattern of the current plan (a new Newton iteration or time step): values only, no pattern copy
    if (h->havePlan && same_batch_pattern(h->plan, nsys, n, rowPtr, col)) return RSG_OK;
    const int ntot = sysRow0[size_t(nsys)];
    // concatenated pattern of the block-diagonal batch
    std::vector<int> rp(size_t(ntot) + 1, 0), ci;
    size_t total = 0;
    for (int s = 0; s < nsys; ++s) total += size_t(rowPtr[s][n[s]]);
    ci.reserve(total);
    for (int s = 0; s < nsys; ++s) {
        const int r0 = sysRow0[size_t(s)];
        if (rowPtr[s][0] != 0) return fail(RSG_EINVAL, "rowPtr[0] must be 0 (system " + std::to_string(s) + ")");
        for (int i = 0; i < n[s]; ++i) {
            rp[size_t(r0 + i) + 1] = rp[size_t(r0)] + rowPtr[s][i + 1];
            for (int p = rowPtr[s][i]; p < rowPtr[s][i + 1]; ++p) {
                const int c = col[s][p];
                if (c < 0 || c >= n[s]) return fail(RSG_EINVAL, "column out of range in system " + std::to_string(s));
                ci.push_back(c + r0);
            }
        }
    }
    const bool same = h->havePlan && h->plan.nsys == nsys && h->plan.rowPtr0 == rp && h->plan.col0 == ci && h->plan.sysRow0 == sysRow0;
    if (!same) {
        free_plan(h);
        std::string err;
        if (h->opt.precond == RSG_PREC_MCBILU0) {
            // multicolour BILU0: the plan of P A P^T (its natural-order BILU0 is the multicolour one), mapped back to the
            // caller's rows and blocks
            std::vector<int> rp2, ci2, rowOrig, blockOrig;
            multicolour_batch(nsys, sysRow0, rp, ci, rp2, ci2, rowOrig, blockOrig);
            if (!build_plan(h->plan, nsys, sysRow0, rp2, ci2, err, host_threads())) return fail(RSG_EINVAL, err);
            HostPlan& P = h->plan;
            for (auto& v : P.perm) v = rowOrig[size_t(v)];
            for (int k = 0; k < P.n; ++k) P.iperm[size_t(P.perm[size_t(k)])] = k;
            for (auto& v : P.valSrc) v = blockOrig[size_t(v)];
            P.rowPtr0 = rp;
            P.col0 = ci;
        } else if (!build_plan(h->plan, nsys, sysRow0, rp, ci, err, host_threads())) {
            return fail(RSG_EINVAL, err);
        }
        int rc = alloc_plan(h);
        if (rc) { free_plan(h); return rc; }
        h->nsys = nsys;
    }
    return RSG_OK;
}

int do_set_batch(rsg_solver* h, int nsys, int nb, const int* n, const int* const* rowPtr, const int* const* col,
                 const double* const* val) {
    if (nsys < 1 || !n || !rowPtr || !col || !val) return fail(RSG_EINVAL, "set_batch: null argument or nsys < 1");
    if (nb != NB) {
        // compositional (nb = nc + 1) and thermal blocks: the block-size-generic path (rsg_generic.cu)
        if (nb < 1 || nb > GEN_MAX_NB) return fail(RSG_EINVAL, "block size nb = " + std::to_string(nb) + " outside [1, 16]");
        if (nsys != 1) return fail(RSG_EINVAL, "block sizes other than 3 are solved one system per handle (nsys = 1)");
        if (!h->genActive) {
            free_plan(h);
            h->gen = gen_create(h->stream);
            h->genActive = true;
        }
        const int rc = gen_set_matrix(h->gen, h->opt, n[0], nb, rowPtr[0], col[0], val[0]);
        if (rc) return rc;
        h->haveMatrix = true;
        h->haveSetup = false;
        return RSG_OK;
    }
    if (h->genActive) free_plan(h);
    for (int s = 0; s < nsys; ++s)
        if (!val[s] || !rowPtr[s] || !col[s] || n[s] < 1) return fail(RSG_EINVAL, "set_batch: system " + std::to_string(s) + " is empty");
    // A new Newton iteration of the planned batch (same sizes): the values go up while another thread confirms the
    // pattern; if the pattern turns out to differ, the batch is planned again and its values uploaded again.
    if (h->havePlan && !h->jac && h->plan.nsys == nsys && int(h->plan.sysRow0.size()) == nsys + 1) {
        const HostPlan& P = h->plan;
        bool sizes = true;
        std::vector<int> nnzbs(static_cast<size_t>(nsys));
        for (int s = 0; s < nsys && sizes; ++s) {
            const size_t r0 = size_t(P.sysRow0[size_t(s)]), r1 = size_t(P.sysRow0[size_t(s) + 1]);
            nnzbs[size_t(s)] = rowPtr[s][n[s]];
            sizes = int(r1 - r0) == n[s] && P.rowPtr0[r1] - P.rowPtr0[r0] == nnzbs[size_t(s)];
        }
        if (sizes) {
            auto check = std::async(std::launch::async, [&] { return same_batch_pattern(P, nsys, n, rowPtr, col); });
            size_t off = 0;
            cudaError_t e = cudaSuccess;
            for (int s = 0; s < nsys && e == cudaSuccess; ++s) {
                const size_t cnt = size_t(nnzbs[size_t(s)]) * NB2;
                if (cnt) e = cudaMemcpyAsync(h->val0 + off, val[s], cnt * sizeof(double), cudaMemcpyHostToDevice, h->stream);
                off += cnt;
            }
            const bool same = check.get();
            if (e != cudaSuccess) return fail(RSG_ECUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
            if (same) {
                launch_gather_blocks(h->dp, h->val0, h->val, h->stream);   // into level space
                h->launches += 1;
                RSG_CUDA(cudaGetLastError());
                h->haveMatrix = true;
                h->haveSetup = false;
                return RSG_OK;
            }
        }
    }
    std::vector<int> nnzbs;
    int rc = set_batch_pattern(h, nsys, n, rowPtr, col, nnzbs);
    if (rc) return rc;
    h->jac = false;
    std::vector<const double*> vals(val, val + nsys);
    return set_values(h, vals, nnzbs);
}

// Jacobians with well rows (full scalar CSR per system, values on the host (hval) or in one device array (dval)):
// the well Schur complement on the device into the solver's block storage (rsg_wellschur.cu)
int do_set_jacobian(rsg_solver* h, int nsys, int nv, const int* nrows, const int* na, const int* nw, const int* const* rowPtr,
                    const int* const* col, const double* const* hval, const double* dval) {
    if (nsys < 1 || !nrows || !na || !nw || !rowPtr || !col || (!hval && !dval)) return fail(RSG_EINVAL, "set_jacobian: null argument");
    if (nv != NB) return fail(RSG_EINVAL, "only nv = 3 (black-oil) is supported, got nv = " + std::to_string(nv));
    for (int s = 0; s < nsys; ++s)
        if (!rowPtr[s] || !col[s] || (hval && !hval[s])) return fail(RSG_EINVAL, "set_jacobian: system " + std::to_string(s) + " is empty");
    cudaStream_t st = h->stream;
    int rc;
    if (!h->wsPlanned || !ws_same_pattern(h->ws, nsys, nv, nrows, na, nw, rowPtr, col)) {
        h->wsPat.release_all();
        h->wsVal.release_all();
        h->wsd = WsDev{};
        h->wsPlanned = h->wsValues = false;
        h->jval = h->wsB = h->wsX = h->wsBc = h->wsXc = nullptr;
        std::string err;
        if (!ws_plan_pattern(h->ws, nsys, nv, nrows, na, nw, rowPtr, col, err)) return fail(RSG_EINVAL, err);
        const WsPlan& W = h->ws;
        WsDev& D = h->wsd;
        DevMem& M = h->wsPat;
        D.ncpl = int(W.cplPos.size());
        D.nwell = int(W.diagPos.size());
        D.nred = W.red0.back();
        if ((rc = upload(M, &D.cplPos, W.cplPos, st)) || (rc = upload(M, &D.diagPos, W.diagPos, st)) || (rc = upload(M, &D.wcBeg, W.wcBeg, st)) ||
            (rc = upload(M, &D.wcPos, W.wcPos, st)) || (rc = upload(M, &D.wcRed, W.wcRed, st)) || (rc = upload(M, &D.wwBeg, W.wwBeg, st)) ||
            (rc = upload(M, &D.wwPos, W.wwPos, st)) || (rc = upload(M, &D.wellFull, W.wellFull, st)) || (rc = upload(M, &D.redFull, W.redFull, st)) ||
            (rc = dalloc(M, &D.mask, size_t(std::max(D.ncpl, 1)))) || (rc = dalloc(M, &D.wellOk, size_t(std::max(D.nwell, 1)))) ||
            (rc = dalloc(M, &h->jval, size_t(W.jEnt0.back()))) || (rc = dalloc(M, &h->wsB, size_t(W.full0.back()))) ||
            (rc = dalloc(M, &h->wsX, size_t(W.full0.back()))) || (rc = dalloc(M, &h->wsBc, size_t(D.nred))) ||
            (rc = dalloc(M, &h->wsXc, size_t(D.nred))))
            return rc;
        h->wsPlanned = true;
    }
    const WsPlan& W = h->ws;
    if (dval) {
        h->jv = dval;
    } else {
        for (int s = 0; s < nsys; ++s) {
            const size_t cnt = size_t(W.jEnt0[size_t(s) + 1] - W.jEnt0[size_t(s)]);
            if (cnt) RSG_CUDA(cudaMemcpyAsync(h->jval + W.jEnt0[size_t(s)], hval[s], cnt * sizeof(double), cudaMemcpyHostToDevice, st));
        }
        h->jv = h->jval;
    }
    // the value-dependent inputs of the plan: which couplings are nonzero, whether every well row is usable
    launch_ws_check(h->wsd, h->jv, st);
    h->launches += 1;
    std::vector<unsigned char> mask(size_t(h->wsd.ncpl)), ok(size_t(h->wsd.nwell));
    if (!mask.empty()) RSG_CUDA(cudaMemcpyAsync(mask.data(), h->wsd.mask, mask.size(), cudaMemcpyDeviceToHost, st));
    if (!ok.empty()) RSG_CUDA(cudaMemcpyAsync(ok.data(), h->wsd.wellOk, ok.size(), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    for (size_t w = 0; w < ok.size(); ++w)
        if (!ok[w]) {
            h->wsValues = false;
            return fail(RSG_EINVAL, "well row " + std::to_string(w) + " has no usable BHP derivative or couples wells: the engine keeps "
                                    "the full system (engine/src/bsr.cpp:742-748)");
        }
    if (!h->wsValues || mask != W.mask || !h->havePlan) {
        std::string err;
        if (!ws_plan_values(h->ws, mask, err)) return fail(RSG_EINVAL, err);
        std::vector<int> nS(na, na + nsys), nnzbs;
        std::vector<const int*> rpS(static_cast<size_t>(nsys)), ciS(static_cast<size_t>(nsys));
        for (int s = 0; s < nsys; ++s) { rpS[size_t(s)] = W.srp[size_t(s)].data(); ciS[size_t(s)] = W.sci[size_t(s)].data(); }
        if ((rc = set_batch_pattern(h, nsys, nS.data(), rpS.data(), ciS.data(), nnzbs))) return rc;
        h->wsVal.release_all();
        WsDev& D = h->wsd;
        DevMem& M = h->wsVal;
        D.nval = (long long)W.sBase.size();
        D.nfill = int(W.fillScalar.size());
        if ((rc = upload(M, &D.sBase, W.sBase, st)) || (rc = upload(M, &D.fillScalar, W.fillScalar, st)) ||
            (rc = upload(M, &D.fillBeg, W.fillBeg, st)) || (rc = upload(M, &D.tCw, W.tCw, st)) || (rc = upload(M, &D.tDiag, W.tDiag, st)) ||
            (rc = upload(M, &D.tWc, W.tWc, st)) || (rc = upload(M, &D.rBeg, W.rBeg, st)) || (rc = upload(M, &D.rCw, W.rCw, st)) ||
            (rc = upload(M, &D.rDiag, W.rDiag, st)) || (rc = upload(M, &D.rWellFull, W.rWellFull, st)))
            return rc;
        h->wsValues = true;
    }
    launch_ws_values(h->wsd, h->jv, h->val0, st);
    launch_gather_blocks(h->dp, h->val0, h->val, st);
    h->launches += 3;
    RSG_CUDA(cudaGetLastError());
    h->jac = true;
    h->haveMatrix = true;
    h->haveSetup = false;
    return RSG_OK;
}

template <class T>
int alloc_split(rsg_solver* h, SplitFactors<T>& F) {
    int rc;
    if ((rc = dalloc(h->pmem, &F.L, size_t(h->dp.n) * LREC)) || (rc = dalloc(h->pmem, &F.UD, size_t(h->dp.n) * UREC)) ||
        (rc = dalloc(h->pmem, &F.Lov, size_t(h->dp.nLov) * NB2)) || (rc = dalloc(h->pmem, &F.Uov, size_t(h->dp.nUov) * NB2)))
        return rc;
    return RSG_OK;
}

int ensure_precond_storage(rsg_solver* h) {
    const size_t E = size_t(h->plan.nnzb) * NB2;
    int rc;
    if (h->opt.precond == RSG_PREC_CPR_DEVICE) return RSG_OK;    // its arrays live with the hierarchy
    if (h->opt.precond == RSG_PREC_JACOBI) {
        if (!h->dinv && (rc = dalloc(h->pmem, &h->dinv, size_t(h->plan.n) * NB2))) return rc;
    } else if (h->opt.precision == RSG_MIXED || h->opt.precision == RSG_MIXED_F32) {
        if (!h->luf && (rc = dalloc(h->pmem, &h->luf, E))) return rc;
        if (!h->work && (rc = dalloc(h->pmem, &h->work, E))) return rc;
        if (h->opt.precision == RSG_MIXED_F32 && !h->V.y32 && (rc = dalloc(h->pmem, &h->V.y32, size_t(h->plan.n) * NB))) return rc;
        if (h->opt.precision == RSG_MIXED_F32 && !h->V.yt) {
            if ((rc = dalloc(h->pmem, &h->V.yt, size_t(h->plan.n) * NB))) return rc;
            RSG_CUDA(cudaMemsetAsync(h->V.yt, 0, size_t(h->plan.n) * NB * sizeof(unsigned long long), h->stream));
        }
        if (h->cta && !h->s32.L && (rc = alloc_split(h, h->s32))) return rc;
    } else {
        if (!h->lu && (rc = dalloc(h->pmem, &h->lu, E))) return rc;
        if (h->cta && !h->s64.L && (rc = alloc_split(h, h->s64))) return rc;
    }
    return RSG_OK;
}

// Gauss-Seidel schedule of one AMG level: the reference's natural-order sweep as forward levels of its lower
// dependencies (identity row list, engine/src/amg.cpp:98-113), or, for the FP32 precision forms, a multicolour sweep:
// greedy colours assigned in the level's natural order, rows ordered by (colour, natural index); rows of one
// colour are independent, so a sweep is one step per colour.
void gs_schedule(const AmgLevel& A, bool mc, std::vector<int>& rows, std::vector<int>& start) {
    rows.resize(size_t(A.n));
    if (!mc) {
        std::iota(rows.begin(), rows.end(), 0);
        start = A.lvlStart;
        return;
    }
    std::vector<int> colr(size_t(A.n), -1);
    std::vector<char> used;
    int nc = 0;
    for (int I = 0; I < A.n; ++I) {
        const int k = A.iperm[size_t(I)];
        used.assign(size_t(nc) + 1, 0);
        for (int p = A.rp[size_t(k)]; p < A.rp[size_t(k) + 1]; ++p) {
            const int j = A.ci[size_t(p)];
            if (j != k && colr[size_t(j)] >= 0) used[size_t(colr[size_t(j)])] = 1;
        }
        int c = 0;
        while (used[size_t(c)]) ++c;
        colr[size_t(k)] = c;
        nc = std::max(nc, c + 1);
    }
    start.assign(size_t(nc) + 1, 0);
    for (int k = 0; k < A.n; ++k) start[size_t(colr[size_t(k)]) + 1]++;
    for (int c = 0; c < nc; ++c) start[size_t(c) + 1] += start[size_t(c)];
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int I = 0; I < A.n; ++I) {
        const int k = A.iperm[size_t(I)];
        rows[size_t(fill[size_t(colr[size_t(k)])]++)] = k;
    }
}

// Device layout of the batch's AMG hierarchies (level-major concatenation, see DevAmg) and its upload.
int build_dev_amg(rsg_solver* h, const std::vector<SysAmg>& H) {
    DevAmg& G = h->amg;
    DevMem& M = h->pmem;
    const int nsys = int(H.size());
    int maxL = 0;
    for (const auto& s : H) maxL = std::max(maxL, int(s.lv.size()));
    G.nsys = nsys;
    G.maxL = maxL;
    std::vector<AmgSysLv> lv(size_t(nsys) * maxL);
    const bool mc = h->opt.precision != RSG_FP64;
    std::vector<std::vector<int>> schRows(size_t(nsys) * maxL), schStart(size_t(nsys) * maxL);
    for (int s = 0; s < nsys; ++s)
        for (int l = 0; l < int(H[size_t(s)].lv.size()); ++l)
            gs_schedule(H[size_t(s)].lv[size_t(l)], mc, schRows[size_t(s) * maxL + l], schStart[size_t(s) * maxL + l]);
    int rows = 0, rps = 0, ents = 0, lvls = 0, mems = 0, aps = 0, lus = 0, lurows = 0, slots = 0;
    std::vector<int> sysRows(size_t(nsys), 0);
    G.levelEntBeg.assign(size_t(maxL) + 1, 0);
    G.levelApBeg.assign(size_t(maxL) + 1, 0);
    G.levelRowBeg.assign(size_t(maxL) + 1, 0);
    std::vector<int> apOff(size_t(nsys) * maxL, 0);
    for (int l = 0; l < maxL; ++l) {
        G.levelEntBeg[size_t(l)] = ents;
        G.levelApBeg[size_t(l)] = aps;
        G.levelRowBeg[size_t(l)] = rows;
        for (int s = 0; s < nsys; ++s) {
            if (l >= int(H[size_t(s)].lv.size())) continue;
            const AmgLevel& A = H[size_t(s)].lv[size_t(l)];
            AmgSysLv& d = lv[size_t(s) * maxL + l];
            d.n = A.n;
            d.nnz = int(A.ci.size());
            d.nl = int(schStart[size_t(s) * maxL + l].size()) - 1;
            d.mc = mc ? 1 : 0;
            d.rowOff = rows; d.rpOff = rps; d.entOff = ents; d.lvlOff = lvls; d.memOff = mems;
            d.W = l == 0 ? AMG_W0 : AMG_W1;
            d.slotOff = slots;
            d.locOff = sysRows[size_t(s)];
            slots += A.n * d.W;
            sysRows[size_t(s)] += A.n;
            apOff[size_t(s) * maxL + l] = aps;
            if (l == 0 && ents != h->plan.rowPtr[size_t(h->plan.sysRow0[size_t(s)])])
                return fail(RSG_EINVAL, "internal: AMG level 0 does not match the block pattern");
            rows += A.n; rps += A.n + 1; ents += d.nnz; lvls += d.nl + 1; mems += int(A.mem.size());
            aps += l > 0 ? int(A.apPtr.size()) - 1 : 0;
            if (l + 1 == int(H[size_t(s)].lv.size())) {
                d.coarse = 1;
                d.dense = H[size_t(s)].coarseDense ? 1 : 0;
                if (d.dense) { d.luOff = lus; d.luRowOff = lurows; lus += A.n * A.n; lurows += A.n; G.maxCoarse = std::max(G.maxCoarse, A.n); }
            }
        }
    }
    G.levelEntBeg[size_t(maxL)] = ents;
    G.levelApBeg[size_t(maxL)] = aps;
    G.levelRowBeg[size_t(maxL)] = rows;
    G.totRows = rows; G.totEnt = ents; G.nAP = aps; G.totLu = lus; G.totLuRows = lurows;
    G.totSlots = slots;
    G.maxSysAmgRows = 0;
    for (int r : sysRows) G.maxSysAmgRows = std::max(G.maxSysAmgRows, r);
    G.maxSysLoRows = 0;
    for (int s = 0; s < nsys; ++s)
        G.maxSysLoRows = std::max(G.maxSysLoRows, sysRows[size_t(s)] - (H[size_t(s)].lv.empty() ? 0 : H[size_t(s)].lv[0].n));
    // V-cycle row slots: first W off-diagonal entries of every row in row order, the rest from the CSR
    std::vector<int> slotSrc(size_t(std::max(slots, 1)), -1), slotCol(size_t(std::max(slots, 1)), -1), meta(size_t(rows) * 4, -1);
    for (int l = 0; l < maxL; ++l)
        for (int s = 0; s < nsys; ++s) {
            if (l >= int(H[size_t(s)].lv.size())) continue;
            const AmgLevel& A = H[size_t(s)].lv[size_t(l)];
            const AmgSysLv& d = lv[size_t(s) * maxL + l];
            for (int k = 0; k < A.n; ++k) {
                const int p0 = A.rp[size_t(k)], p1 = A.rp[size_t(k) + 1], pd = A.diag[size_t(k)];
                int* m = &meta[size_t(d.rowOff + k) * 4];
                m[0] = pd - p0;
                m[1] = p1 - p0 - 1;
                m[2] = -1;
                m[3] = pd;
                for (int p = p0, j = 0; p < p1 && j < d.W; ++p) {
                    if (p == pd) continue;
                    slotSrc[size_t(d.slotOff) + size_t(k) * d.W + size_t(j)] = d.entOff + p;
                    slotCol[size_t(d.slotOff) + size_t(k) * d.W + size_t(j)] = A.ci[size_t(p)];
                    if (j == d.W - 1) m[2] = p + 1;   // the row continues here (diagonal and / or further entries)
                    ++j;
                }
            }
        }
    // ci (and the value arrays) carry OV_CHUNK - 1 entries past the last row: the sweeps read a row's entries
    // after its slots in chunks of OV_CHUNK
    std::vector<int> rp(static_cast<size_t>(rps)), ci(static_cast<size_t>(ents) + OV_CHUNK - 1, 0), dg(static_cast<size_t>(rows)),
        lvl(static_cast<size_t>(lvls)), agg(static_cast<size_t>(rows), 0), memPtr(static_cast<size_t>(rps), 0),
        mem(static_cast<size_t>(mems)), dgG(static_cast<size_t>(rows)), luPerm(static_cast<size_t>(std::max(lurows, 1)), 0),
        gsRows(static_cast<size_t>(std::max(rows, 1)), 0);
    std::vector<int> apPtr(size_t(aps) + 1, 0), apSrc, acPtr(size_t(ents) + 1, 0), acSrc;
    for (int l = 0; l < maxL; ++l)
        for (int s = 0; s < nsys; ++s) {
            if (l >= int(H[size_t(s)].lv.size())) continue;
            const AmgLevel& A = H[size_t(s)].lv[size_t(l)];
            const AmgSysLv& d = lv[size_t(s) * maxL + l];
            std::copy(A.rp.begin(), A.rp.end(), rp.begin() + d.rpOff);
            std::copy(A.ci.begin(), A.ci.end(), ci.begin() + d.entOff);
            std::copy(A.diag.begin(), A.diag.end(), dg.begin() + d.rowOff);
            std::copy(schStart[size_t(s) * maxL + l].begin(), schStart[size_t(s) * maxL + l].end(), lvl.begin() + d.lvlOff);
            std::copy(schRows[size_t(s) * maxL + l].begin(), schRows[size_t(s) * maxL + l].end(), gsRows.begin() + d.rowOff);
            for (int k = 0; k < A.n; ++k) dgG[size_t(d.rowOff + k)] = d.entOff + A.diag[size_t(k)];
            if (!A.agg.empty()) std::copy(A.agg.begin(), A.agg.end(), agg.begin() + d.rowOff);
            if (l > 0) {
                const AmgSysLv& f = lv[size_t(s) * maxL + l - 1];
                std::copy(A.memPtr.begin(), A.memPtr.end(), memPtr.begin() + d.rpOff);
                std::copy(A.mem.begin(), A.mem.end(), mem.begin() + d.memOff);
                const int a0 = apOff[size_t(s) * maxL + l];
                for (size_t e = 0; e + 1 < A.apPtr.size(); ++e) {
                    for (int q = A.apPtr[e]; q < A.apPtr[e + 1]; ++q) apSrc.push_back(f.entOff + A.apSrc[size_t(q)]);
                    apPtr[size_t(a0) + e + 1] = int(apSrc.size());
                }
                for (int e = 0; e < d.nnz; ++e) {
                    for (int q = A.acPtr[size_t(e)]; q < A.acPtr[size_t(e) + 1]; ++q) acSrc.push_back(a0 + A.acSrc[size_t(q)]);
                    acPtr[size_t(d.entOff + e) + 1] = int(acSrc.size());
                }
            } else {
                for (int e = 0; e < d.nnz; ++e) acPtr[size_t(d.entOff + e) + 1] = int(acSrc.size());
            }
            if (d.coarse && d.dense) std::copy(A.perm.begin(), A.perm.end(), luPerm.begin() + d.luRowOff);
        }
    // grid-wide V-cycle: (system, level) descriptor and wave (schedule level) of every row, and the levels that are
    // some system's coarsest without a dense LU
    std::vector<int> rowLv(static_cast<size_t>(std::max(rows, 1)), 0), wave(static_cast<size_t>(std::max(rows, 1)), 0);
    G.coarseGsLevels.clear();
    for (int l = 0; l < maxL; ++l) {
        bool gsCoarse = false;
        for (int s = 0; s < nsys; ++s) {
            if (l >= int(H[size_t(s)].lv.size())) continue;
            const AmgSysLv& d = lv[size_t(s) * maxL + l];
            const std::vector<int>& st0 = schStart[size_t(s) * maxL + l];
            const std::vector<int>& rw = schRows[size_t(s) * maxL + l];
            for (int k = 0; k < d.n; ++k) rowLv[size_t(d.rowOff + k)] = s * maxL + l;
            for (size_t g = 0; g + 1 < st0.size(); ++g)
                for (int q = st0[g]; q < st0[g + 1]; ++q) wave[size_t(d.rowOff + rw[size_t(q)])] = int(g);
            gsCoarse |= d.coarse && !d.dense;
        }
        if (gsCoarse) G.coarseGsLevels.push_back(l);
    }
    // the sync-free sweeps may take "updated before" from the entry position when it agrees with the waves everywhere
    G.posOrder = true;
    for (int l = 0; l < maxL && G.posOrder; ++l)
        for (int s = 0; s < nsys && G.posOrder; ++s) {
            if (l >= int(H[size_t(s)].lv.size())) continue;
            const AmgSysLv& d = lv[size_t(s) * maxL + l];
            const AmgLevel& A = H[size_t(s)].lv[size_t(l)];
            for (int k = 0; k < A.n && G.posOrder; ++k) {
                const int wk = wave[size_t(d.rowOff + k)], pd = A.diag[size_t(k)];
                for (int p = A.rp[size_t(k)]; p < A.rp[size_t(k) + 1]; ++p) {
                    if (p == pd) continue;
                    const bool earlier = wave[size_t(d.rowOff + A.ci[size_t(p)])] < wk;
                    if (earlier != (p < pd)) { G.posOrder = false; break; }
                }
            }
        }
    G.gsBlocks.assign(size_t(maxL), 1);
    for (int l = 0; l < maxL; ++l) {
        int maxNl = 1;
        for (int s = 0; s < nsys; ++s)
            if (l < int(H[size_t(s)].lv.size())) maxNl = std::max(maxNl, lv[size_t(s) * maxL + l].nl);
        G.gsBlocks[size_t(l)] = sweep_blocks_for(double(G.levelRowBeg[size_t(l) + 1] - G.levelRowBeg[size_t(l)]) / maxNl, h->opt.sweep_inflight);
    }
    // colour-major rows of every level that is smoothed (multicolour schedule only): colour c of every system, then
    // c + 1; colours from colTail on (all of them small) are swept together by one sync-free pass
    constexpr int kTailRows = 2048;
    std::vector<int4> cdesc;
    G.colBeg.assign(size_t(maxL), std::vector<int>());
    G.colTail.assign(size_t(maxL), 0);
    if (mc)
        for (int l = 0; l < maxL; ++l) {
            int ncol = 0;
            for (int s = 0; s < nsys; ++s)
                if (l < int(H[size_t(s)].lv.size()) && !lv[size_t(s) * maxL + l].coarse) ncol = std::max(ncol, lv[size_t(s) * maxL + l].nl);
            std::vector<int>& cb = G.colBeg[size_t(l)];
            cb.assign(size_t(ncol) + 1, int(cdesc.size()));
            for (int c = 0; c < ncol; ++c) {
                cb[size_t(c)] = int(cdesc.size());
                for (int s = 0; s < nsys; ++s) {
                    if (l >= int(H[size_t(s)].lv.size())) continue;
                    const AmgSysLv& d = lv[size_t(s) * maxL + l];
                    if (d.coarse || c >= d.nl) continue;
                    const AmgLevel& A = H[size_t(s)].lv[size_t(l)];
                    const std::vector<int>& st0 = schStart[size_t(s) * maxL + l];
                    const std::vector<int>& rw = schRows[size_t(s) * maxL + l];
                    for (int g = st0[size_t(c)]; g < st0[size_t(c) + 1]; ++g) {
                        const int k = rw[size_t(g)];
                        cdesc.push_back(make_int4(d.rowOff + k, d.entOff + A.rp[size_t(k)], d.entOff + A.rp[size_t(k) + 1],
                                                  d.entOff + A.diag[size_t(k)]));
                    }
                }
            }
            cb[size_t(ncol)] = int(cdesc.size());
            int tail = ncol;
            while (tail > 0 && cb[size_t(tail)] - cb[size_t(tail) - 1] < kTailRows) --tail;
            G.colTail[size_t(l)] = tail;
        }
    if (cdesc.empty()) cdesc.push_back(make_int4(0, 0, 0, 0));
    std::vector<int> gci(static_cast<size_t>(std::max(ents, 1)), 0);
    for (int l = 0; l < maxL; ++l)
        for (int s = 0; s < nsys; ++s) {
            if (l >= int(H[size_t(s)].lv.size())) continue;
            const AmgSysLv& d = lv[size_t(s) * maxL + l];
            const AmgLevel& A = H[size_t(s)].lv[size_t(l)];
            for (int e = 0; e < d.nnz; ++e) gci[size_t(d.entOff + e)] = d.rowOff + A.ci[size_t(e)];
        }
    // pointer arrays are prefix sums over the level-major order: fill gaps (levels absent for some systems)
    for (size_t e = 1; e < apPtr.size(); ++e) apPtr[e] = std::max(apPtr[e], apPtr[e - 1]);
    for (size_t e = 1; e < acPtr.size(); ++e) acPtr[e] = std::max(acPtr[e], acPtr[e - 1]);
    if (apSrc.empty()) apSrc.push_back(0);
    if (acSrc.empty()) acSrc.push_back(0);
    int rc;
    cudaStream_t st = h->stream;
    if ((rc = dalloc(M, &G.lv, lv.size())) || (rc = upload(M, &G.rp, rp, st)) || (rc = upload(M, &G.ci, ci, st)) ||
        (rc = upload(M, &G.diag, dg, st)) || (rc = upload(M, &G.lvl, lvl, st)) || (rc = upload(M, &G.agg, agg, st)) ||
        (rc = upload(M, &G.memPtr, memPtr, st)) || (rc = upload(M, &G.mem, mem, st)) || (rc = upload(M, &G.apPtr, apPtr, st)) ||
        (rc = upload(M, &G.apSrc, apSrc, st)) || (rc = upload(M, &G.acPtr, acPtr, st)) || (rc = upload(M, &G.acSrc, acSrc, st)) ||
        (rc = upload(M, &G.diagGlob, dgG, st)) || (rc = upload(M, &G.luPerm, luPerm, st)) ||
        (rc = upload(M, &G.slotSrc, slotSrc, st)) || (rc = upload(M, &G.slotCol, slotCol, st)) || (rc = upload(M, &G.gsRows, gsRows, st)) ||
        (rc = upload(M, reinterpret_cast<int**>(&G.rowMeta), meta, st)) || (rc = upload(M, &G.rowLv, rowLv, st)) || (rc = upload(M, &G.cdesc, cdesc, st)) || (rc = upload(M, &G.gci, gci, st)) ||
        (rc = upload(M, &G.wave, wave, st)) || (rc = dalloc(M, &G.gsFlag, 2 * size_t(std::max(rows, 1)))) ||
        (rc = dalloc(M, &G.gsCtr, 4 * size_t(std::max(maxL, 1)))) || (rc = dalloc(M, &G.coarse64, size_t(std::max(nsys, 1)))))
        return rc;
    RSG_CUDA(cudaMemsetAsync(G.coarse64, 0, size_t(std::max(nsys, 1)) * sizeof(int), st));
    if (h->opt.precond == RSG_PREC_CPR_DEVICE) {              // the float CPR-AMG's arrays
        std::vector<size_t> woff(size_t(nsys), 0);
        size_t wtot = 0;
        for (int s = 0; s < nsys; ++s) {
            woff[size_t(s)] = wtot;
            const int L = int(H[size_t(s)].lv.size());
            const AmgSysLv& d = lv[size_t(s) * maxL + L - 1];
            if (d.dense) wtot += 2 * size_t(d.n) * size_t(d.n);
        }
        if ((rc = dalloc(M, &G.dinvf, size_t(std::max(rows, 1)))) || (rc = dalloc(M, &G.bjf, size_t(h->plan.n) * NB2)) ||
            (rc = dalloc(M, &G.dcOk, size_t(std::max(nsys, 1)))) || (rc = dalloc(M, &G.dcWork, std::max<size_t>(wtot, 1))) ||
            (rc = upload(M, &G.dcWorkOff, woff, st)))
            return rc;
    }
    RSG_CUDA(cudaMemsetAsync(G.gsFlag, 0, 2 * size_t(std::max(rows, 1)) * sizeof(int), st));
    RSG_CUDA(cudaMemsetAsync(G.gsCtr, 0, 4 * size_t(std::max(maxL, 1)) * sizeof(unsigned), st));
    {
        const size_t S = size_t(std::max(slots, 1)), R = size_t(std::max(rows, 1)), n = size_t(h->plan.n);
        const size_t nLo = size_t(h->dp.nLov) * 3, nUo = size_t(h->dp.nUov) * 3;
        if ((rc = dalloc(M, &G.slotVal, S)) || (rc = dalloc(M, &G.slotValf, S)) || (rc = dalloc(M, &G.diagVal, R)) ||
            (rc = dalloc(M, &G.diagValf, R)) || (rc = dalloc(M, &G.cin, size_t(std::max(lurows, 1)))) ||
            (rc = dalloc(M, &G.sp, n * SPREC)) || (rc = dalloc(M, &G.spf, n * SPREC)) || (rc = dalloc(M, &G.spLov, nLo)) ||
            (rc = dalloc(M, &G.spLovf, nLo)) || (rc = dalloc(M, &G.spUov, nUo)) || (rc = dalloc(M, &G.spUovf, nUo)))
            return rc;
    }
    RSG_CUDA(cudaMemcpyAsync(G.lv, lv.data(), lv.size() * sizeof(AmgSysLv), cudaMemcpyHostToDevice, st));
    if ((rc = dalloc(M, &G.val, size_t(ents) + OV_CHUNK - 1)) || (rc = dalloc(M, &G.valf, size_t(ents) + OV_CHUNK - 1)) || (rc = dalloc(M, &G.apVal, size_t(std::max(aps, 1)))) ||
        (rc = dalloc(M, &G.lu, size_t(std::max(lus, 1)))) || (rc = dalloc(M, &G.luf, size_t(std::max(lus, 1)))) ||
        (rc = dalloc(M, &G.invf, size_t(std::max(lus, 1)))) ||
        (rc = dalloc(M, &G.piv, size_t(std::max(lurows, 1)))) || (rc = dalloc(M, &G.x, size_t(rows))) || (rc = dalloc(M, &G.b, size_t(rows))) ||
        (rc = dalloc(M, &G.r, size_t(rows))) || (rc = dalloc(M, &G.xf, size_t(rows))) || (rc = dalloc(M, &G.bf, size_t(rows))) ||
        (rc = dalloc(M, &G.rf, size_t(rows))))
        return rc;
    // the fused V-cycle's phase table and barrier counter (the split CPR form)
    {
        std::vector<VPhase> ph;
        vcycle_phases(G, ph);
        G.nPhases = int(ph.size());
        G.coarseChunks = std::max(1, (G.maxCoarse + 255) / 256);
        if (!ph.empty() && ((rc = upload(M, &G.phases, ph, st)) || (rc = dalloc(M, &G.vbar, 1)))) return rc;
    }
    h->amgLevels = maxL;
    return RSG_OK;
}

// CPR set-up (BlockCPR::setup, engine/src/bsr.cpp:993-1059): weights, pressure matrix, hierarchy (host aggregation
// at the first set-up of a pattern, device Galerkin refresh afterwards), coarsest dense LU
int setup_cpr(rsg_solver* h, const double* acc) {
    const HostPlan& P = h->plan;
    const DevPlan& D = h->dp;
    cudaStream_t st = h->stream;
    int rc;
    DevAmg& G = h->amg;
    if (!G.w) {
        if ((rc = dalloc(h->pmem, &G.w, size_t(P.n) * 3)) || (rc = dalloc(h->pmem, &G.T, size_t(P.n) * 3)) ||
            (rc = dalloc(h->pmem, &G.acc, size_t(P.n) * 9)) || (rc = dalloc(h->pmem, &h->d_nfb, 1)))
            return rc;
    }
    const double* accLev = nullptr;
    if (acc) {   // caller's blocks in the original row order, staged through val0 (free after the value gather)
        RSG_CUDA(cudaMemcpyAsync(h->val0, acc, size_t(P.n) * 9 * sizeof(double), cudaMemcpyHostToDevice, st));
        launch_gather_acc(D, h->val0, G.acc, st);
        accLev = G.acc;
        h->launches += 1;
    }
    RSG_CUDA(cudaMemsetAsync(h->d_nfb, 0, sizeof(int), st));
    launch_cpr_weights(D, h->val, accLev, G.w, h->d_nfb, st);
    h->launches += 1;
    if (!h->haveAmg) {
        // first set-up of this pattern: the pressure matrix goes to the host for the aggregation
        double* ap = nullptr;
        if ((rc = dalloc(h->mem, &ap, size_t(P.nnzb)))) return rc;
        launch_cpr_pressure(D, h->val, G.w, ap, st);
        std::vector<double> hap(size_t(P.nnzb));
        cudaError_t e = cudaMemcpyAsync(hap.data(), ap, hap.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        h->mem.release(ap);
        if (e != cudaSuccess) return fail(RSG_ECUDA, std::string("pressure matrix copy: ") + cudaGetErrorString(e));
        std::vector<SysAmg> H(size_t(P.nsys));
        std::vector<std::string> errs(size_t(P.nsys));
        std::vector<char> ok(size_t(P.nsys), 1);
        const int hw = host_threads();
        const int nth = std::max(1, std::min(P.nsys, hw));
        const int inner = std::max(1, hw / nth);             // threads inside a system's plan (a lone large system)
        std::vector<std::thread> pool;
        for (int t = 0; t < nth; ++t)
            pool.emplace_back([&, t] {
                for (int s = t; s < P.nsys; s += nth) {
                    const int b0 = P.rowPtr[size_t(P.sysRow0[size_t(s)])], b1 = P.rowPtr[size_t(P.sysRow0[size_t(s) + 1])];
                    std::vector<double> ap0(hap.begin() + b0, hap.begin() + b1);
                    ok[size_t(s)] = amg_plan_system(P, s, ap0, H[size_t(s)], errs[size_t(s)], inner) ? 1 : 0;
                }
            });
        for (auto& th : pool) th.join();
        for (int s = 0; s < P.nsys; ++s)
            if (!ok[size_t(s)]) return fail(RSG_EINVAL, "AMG set-up of system " + std::to_string(s) + ": " + errs[size_t(s)]);
        if ((rc = build_dev_amg(h, H))) return rc;
        h->haveAmg = true;
    }
    launch_cpr_pressure(D, h->val, G.w, G.val, st);          // level 0 of every system = the block pattern
    launch_amg_refresh(G, st);
    if (h->opt.precond == RSG_PREC_CPR_DEVICE) {              // the float CPR-AMG: float values, its own set-up
        launch_amg_round(G, st);
        h->launches += 2 + 3 * std::max(0, G.maxL - 1) + launch_devcpr_setup(D, h->val, G, st);
        RSG_CUDA(cudaGetLastError());
        return RSG_OK;
    }
    launch_amg_coarse_lu(G, h->opt.precision != RSG_FP64, st);
    if (h->opt.precision != RSG_FP64) launch_amg_round(G, st);
    if (h->cta) {                                              // row slots of the thread-block application
        launch_amg_slots(G, h->opt.precision != RSG_FP64, st);
        launch_cpr_sp(D, h->val, G, h->opt.precision != RSG_FP64, st);
        h->launches += 2;
    }
    h->launches += 3 + 3 * std::max(0, G.maxL - 1) + (h->opt.precision != RSG_FP64 ? 2 : 0);
    RSG_CUDA(cudaGetLastError());
    return RSG_OK;
}

int precond_apply_dev(rsg_solver* h, const double* d_r, double* d_z) {
    const PrecDev M = prec_dev(h);
    if (M.devcpr) h->launches += launch_devcpr(h->dp, h->amg, h->val, 0, d_r, nullptr, nullptr, d_z, nullptr, h->stream);
    else if (M.cpr && M.cta && !M.split) { launch_cpr_cta(h->dp, M, *M.amg, 0, M.kind != 0, d_r, nullptr, nullptr, d_z, nullptr, h->stream); h->launches += 1; }
    else if (M.cpr) h->launches += launch_cpr_grid(h->dp, M, *M.amg, 0, d_r, nullptr, nullptr, d_z, nullptr, h->S, h->d_err, h->stream);
    else if (M.cta) { launch_ilu_cta_apply(h->dp, M, d_r, d_z, h->stream); h->launches += 1; }
    else if (M.kind == 0) { launch_ilu_apply_f64(h->dp, h->lu, d_r, d_z, h->S, h->d_err, h->stream); h->launches += 2; }
    else if (M.kind == 1) { launch_ilu_apply_mixed(h->dp, h->luf, d_r, d_z, h->S, h->d_err, h->stream); h->launches += 2; }
    else if (M.kind == 3) { launch_ilu_apply_f32(h->dp, h->luf, d_r, d_z, h->V.yt, h->S, h->d_err, h->stream); h->launches += 2; }
    else { launch_block_jacobi_apply(h->dp, h->dinv, d_r, d_z, h->stream); h->launches += 1; }
    RSG_CUDA(cudaGetLastError());
    return RSG_OK;
}

// ---- launch-shape autotuner. The candidates are timed on the handle's own system right after its first set-up
// (CUDA events on its stream, the preconditioner applied to a zero vector: the same work as any other), the fastest
// is kept and cached per (pattern, options) for the life of the process. Every candidate computes the same values
// bit for bit, so the choice changes time only.
unsigned long long pattern_hash(rsg_solver* h) {
    if (h->patHash) return h->patHash;
    unsigned long long x = 1469598103934665603ULL;
    auto mix = [&x](const std::vector<int>& v) {
        x ^= (unsigned long long)v.size() + 0x9e3779b97f4a7c15ULL;
        x *= 1099511628211ULL;
        for (int q : v) { x ^= (unsigned long long)(unsigned)q; x *= 1099511628211ULL; }
    };
    mix(h->plan.rowPtr0);
    mix(h->plan.col0);
    mix(h->plan.sysRow0);
    h->patHash = x ? x : 1;
    return h->patHash;
}

std::mutex g_tune_mu;
std::map<std::pair<unsigned long long, int>, rsg_solver::Tune> g_tune_cache;

// true when one fused application can be captured into a CUDA graph on this device (a cooperative kernel node)
bool fused_capturable(rsg_solver* h, const double* d_r, double* d_z) {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ex = nullptr;
    if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { cudaGetLastError(); return false; }
    precond_apply_dev(h, d_r, d_z);
    const cudaError_t e1 = cudaStreamEndCapture(h->stream, &g);
    bool ok = e1 == cudaSuccess && g && cudaGraphInstantiate(&ex, g, 0) == cudaSuccess;
    if (ex) cudaGraphExecDestroy(ex);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return ok;
}

int tune_shapes(rsg_solver* h) {
    rsg_solver::Tune t;
    const bool cprCta = h->opt.precond == RSG_PREC_CPR && h->cta && h->haveAmg;
    // a single system under the automatic sweep choice: the one-kernel application (one launch, one SM) and the split
    // form (the V-cycle's passes grid-wide) are both candidates; they give the same results bit for bit
    const bool free_split = cprCta && h->opt.sweep == 0 && h->plan.nsys == 1;
    const bool split = cprCta && (h->splitCpr || free_split);
    t.split = h->splitCpr ? 1 : 0;
    t.vform = h->opt.vcycle_form ? h->opt.vcycle_form : 3;
    if (t.vform == 1 && h->amg.nPhases == 0) t.vform = 2;                  // no phase table for this hierarchy
    t.cpr2Threads = h->opt.cpr2_threads ? h->opt.cpr2_threads : 256;
    const bool free_form = h->opt.vcycle_form == 0, free_thr = h->opt.cpr2_threads == 0;
    auto describe = [](const rsg_solver::Tune& c) {
        if (c.split == 0) return std::string("cpr_form=one-kernel");
        return std::string("vcycle_form=") + std::to_string(c.vform) + " cpr2_threads=" + std::to_string(c.cpr2Threads);
    };
    if (!split) { t.desc = "no split CPR: fixed shapes"; h->tune = t; return RSG_OK; }
    if (!h->opt.autotune || (!free_form && !free_thr && !free_split)) {
        t.desc = describe(t) + (h->opt.autotune ? " source=options" : " source=defaults");
        h->tune = t;
        return RSG_OK;
    }
    const int key2 = h->opt.precision * 1000 + h->opt.vcycle_form * 10000 + h->opt.cpr2_threads + h->device * 100000 +
                     (free_split ? 1000000 : 0);
    const auto key = std::make_pair(pattern_hash(h), key2);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) { h->tune = it->second; return RSG_OK; }
    }
    const size_t N = size_t(h->plan.n) * NB;
    RSG_CUDA(cudaMemsetAsync(h->tmp, 0, N * sizeof(double), h->stream));
    std::vector<rsg_solver::Tune> cand;
    if (free_split) {
        rsg_solver::Tune c;
        c.split = 0;
        cand.push_back(c);
    }
    for (int f : {3, 2, 1})
        for (int thr : {256, 512, 128}) {
            if (!free_form && f != t.vform) continue;
            if (!free_thr && thr != t.cpr2Threads) continue;
            if (f == 1 && h->amg.nPhases == 0) continue;
            rsg_solver::Tune c;
            c.split = 1;
            c.vform = f;
            c.cpr2Threads = thr;
            cand.push_back(c);
        }
    if (cand.empty()) { t.desc = describe(t) + " source=options"; h->tune = t; return RSG_OK; }
    bool fusedOk = true;
    float best = 1e30f;
    rsg_solver::Tune pick = cand.front();
    std::string timings;
    for (const auto& c : cand) {
        if (c.vform == 1 && !fusedOk) continue;
        h->tune = c;
        int rc = precond_apply_dev(h, h->tmp, h->xout);        // warm-up (first launch of the shape)
        if (rc) return rc;
        if (c.vform == 1 && !fused_capturable(h, h->tmp, h->xout)) { fusedOk = false; continue; }
        RSG_CUDA(cudaEventRecord(h->ev0, h->stream));
        for (int k = 0; k < 3; ++k)
            if ((rc = precond_apply_dev(h, h->tmp, h->xout))) return rc;
        RSG_CUDA(cudaEventRecord(h->ev1, h->stream));
        RSG_CUDA(cudaStreamSynchronize(h->stream));
        float ms = 0;
        cudaEventElapsedTime(&ms, h->ev0, h->ev1);
        ms /= 3;
        char buf[96];
        if (c.split == 0) std::snprintf(buf, sizeof(buf), "%sone-kernel %.3f ms", timings.empty() ? "" : ", ", ms);
        else std::snprintf(buf, sizeof(buf), "%sform%d/%d %.3f ms", timings.empty() ? "" : ", ", c.vform, c.cpr2Threads, ms);
        timings += buf;
        if (ms < best) { best = ms; pick = c; }
    }
    const int rce = check_device_errors(h);
    if (rce) return rce;
    pick.desc = describe(pick) + " source=tuned (CPR application: " + timings + (fusedOk ? "" : "; fused kernel not capturable here") + ")";
    h->tune = pick;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = pick;
    return RSG_OK;
}

int do_setup(rsg_solver* h, const double* acc) {
    if (!h->haveMatrix) return fail(RSG_ESTATE, "setup before set_matrix");
    if (h->genActive) {
        const int rc = gen_setup(h->gen, h->opt, acc);
        h->haveSetup = rc == RSG_OK;
        if (rc == RSG_OK) gen_stats(h->gen, &h->st);
        return rc;
    }
    h->escalated = false;
    h->st.escalated_systems = 0;
    const bool amgPrec = h->opt.precond == RSG_PREC_CPR || h->opt.precond == RSG_PREC_CPR_DEVICE;
    if (amgPrec && !h->plan.symmetric)
        return fail(RSG_EINVAL, "the CPR preconditioners need structurally symmetric systems");
    int rc = ensure_precond_storage(h);
    if (rc) return rc;
    RSG_CUDA(cudaMemsetAsync(h->d_nreg, 0, sizeof(int), h->stream));
    RSG_CUDA(cudaEventRecord(h->ev0, h->stream));
    if (amgPrec && (rc = setup_cpr(h, acc))) return rc;
    h->launches += 1;
    if (h->opt.precond == RSG_PREC_CPR_DEVICE) {
        // no BILU0: the second stage is block Jacobi (set up with the hierarchy)
    } else if (h->opt.precond == RSG_PREC_JACOBI) {
        launch_block_jacobi_setup(h->dp, h->val, h->dinv, h->d_nreg, h->stream);
    } else {
        ++h->epoch;
        if (h->opt.precision == RSG_MIXED || h->opt.precision == RSG_MIXED_F32) {
            if (h->cta && h->opt.precision == RSG_MIXED_F32) launch_factor_cta_f32(h->dp, h->val, h->luf, h->d_nreg, h->stream);
            else launch_factor_lean(h->dp, h->val, h->luf, h->work, h->S, h->epoch, h->d_nreg, h->d_err, h->stream);
            if (h->cta) { launch_pack_f32(h->dp, h->luf, h->s32, h->stream); h->launches += 1; }
        } else {
            launch_factor_f64(h->dp, h->val, h->lu, h->S, h->epoch, h->d_nreg, h->d_err, h->stream);
            if (h->cta) { launch_pack_f64(h->dp, h->lu, h->s64, h->stream); h->launches += 1; }
        }
    }
    RSG_CUDA(cudaGetLastError());
    RSG_CUDA(cudaEventRecord(h->ev1, h->stream));
    RSG_CUDA(cudaMemcpyAsync(h->h_pin + 2, h->d_nreg, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if ((rc = check_device_errors(h))) return rc;
    float ms = 0;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    h->st.setup_ms = ms;
    h->st.regularised_blocks = h->h_pin[2];
    h->st.amg_levels = amgPrec ? h->amgLevels : 0;
    h->haveSetup = true;
    return tune_shapes(h);
}

// what a captured graph depends on besides its iteration count: the preconditioner's kind and launch shapes
int graph_kind(const PrecDev& M) {
    // distinct fields: kind 0-3, the three form flags, V-cycle form 0-3, BILU0-stage thread count (256 / 512 / 128)
    return (M.kind & 3) | (M.cpr ? 4 : 0) | (M.cta ? 8 : 0) | (M.split ? 16 : 0) | ((M.vform & 3) << 5) |
           ((M.cpr2Threads >= 512 ? 1 : M.cpr2Threads <= 128 ? 2 : 0) << 7);
}

int launch_iterations(rsg_solver* h, int k) {
    const PrecDev M = prec_dev(h);
    h->launches += (long long)k * (3 + 2 * precond_launches(M));
    if (h->opt.use_graphs) {
        const int kind = graph_kind(M);
        if (!h->gexec || h->gIters != k || h->gKind != kind) {
            if (h->gexec) { cudaGraphExecDestroy(h->gexec); h->gexec = nullptr; }
            cudaGraph_t g = nullptr;
            RSG_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
            for (int i = 0; i < k; ++i) launch_bicg_iteration(h->dp, h->val, M, h->V, h->ks, h->R, h->S, h->d_active, h->d_err, h->stream);
            RSG_CUDA(cudaStreamEndCapture(h->stream, &g));
            cudaError_t e = cudaGraphInstantiate(&h->gexec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { h->gexec = nullptr; return fail(RSG_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e)); }
            h->gIters = k;
            h->gKind = kind;
        }
        RSG_CUDA(cudaGraphLaunch(h->gexec, h->stream));
    } else {
        for (int i = 0; i < k; ++i) launch_bicg_iteration(h->dp, h->val, M, h->V, h->ks, h->R, h->S, h->d_active, h->d_err, h->stream);
        RSG_CUDA(cudaGetLastError());
    }
    return RSG_OK;
}


// BiCGSTAB of every system from the gathered right-hand side h->b into h->V.x
int run_bicgstab(rsg_solver* h, double tol, int maxIt, bool onlyFailed = false) {
    const bool guard = h->opt.precision == RSG_MIXED_F32 && !h->escalated && h->opt.precond != RSG_PREC_CPR_DEVICE &&
                       h->opt.precond != RSG_PREC_JACOBI;
    launch_bicg_init(h->dp, h->b, h->V, h->ks, h->R, tol, maxIt, h->d_active, guard, onlyFailed, h->stream);
    h->launches += 1;
    RSG_CUDA(cudaGetLastError());
    const int chunk = h->opt.check_every > 0 ? h->opt.check_every : 4;
    int launched = 0, rc;
    for (;;) {
        RSG_CUDA(cudaMemcpyAsync(h->h_pin, h->d_active, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        RSG_CUDA(cudaStreamSynchronize(h->stream));
        if (h->h_pin[0] <= 0 || launched >= maxIt) break;
        if ((rc = launch_iterations(h, chunk))) return rc;
        launched += chunk;
    }
    return RSG_OK;
}

int ensure_gmres(rsg_solver* h) {
    if (h->gm.V) return RSG_OK;
    const int m = h->opt.restart > 0 ? h->opt.restart : 40;
    const size_t N = size_t(h->plan.n) * NB;
    GmState& G = h->gm;
    int rc;
    if ((rc = dalloc(h->pmem, &G.V, N * size_t(m + 1))) || (rc = dalloc(h->pmem, &G.Z, N * size_t(m))) || (rc = dalloc(h->pmem, &G.w, N)) ||
        (rc = dalloc(h->pmem, &G.H, gm_stride(m) * size_t(h->plan.nsys))) || (rc = dalloc(h->pmem, &G.inner, 2)))
        return rc;
    G.m = m;
    h->gmExec.assign(size_t(m) + 2, nullptr);
    return RSG_OK;
}

void drop_gm_graphs(rsg_solver* h) {
    for (auto& g : h->gmExec)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
}

// the launches of one GMRES phase: replayed from a cached graph (captured at first use) or issued directly
template <class F>
int gm_phase(rsg_solver* h, size_t idx, F&& launches) {
    if (!h->opt.use_graphs) {
        launches();
        RSG_CUDA(cudaGetLastError());
        return RSG_OK;
    }
    cudaGraphExec_t& ex = h->gmExec[idx];
    if (!ex) {
        cudaGraph_t g = nullptr;
        RSG_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        launches();
        RSG_CUDA(cudaStreamEndCapture(h->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { ex = nullptr; return fail(RSG_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e)); }
    }
    RSG_CUDA(cudaGraphLaunch(ex, h->stream));
    return RSG_OK;
}

// Restarted flexible GMRES(m) of the batch (engine/src/linsolve.cpp:218-273) from h->b into h->V.x. onlyFailed:
// systems whose status is ST_CONV keep their solution and are not restarted (the BiCGSTAB fallback).
int run_gmres(rsg_solver* h, double tol, int maxIt, bool onlyFailed) {
    int rc = ensure_gmres(h);
    if (rc) return rc;
    const PrecDev M = prec_dev(h);
    const int kind = graph_kind(M);
    if (kind != h->gmKind) { drop_gm_graphs(h); h->gmKind = kind; }
    GmState& G = h->gm;
    const int m = G.m;
    const size_t N = size_t(h->plan.n) * NB;
    launch_gm_init(h->dp, h->b, h->V.x, h->ks, h->R, tol, maxIt, onlyFailed, h->d_active, h->stream);
    h->launches += 1;
    RSG_CUDA(cudaGetLastError());
    const int check = h->opt.check_every > 0 ? h->opt.check_every : 4;
    for (int cycle = 0; cycle <= maxIt + 1; ++cycle) {   // every cycle adds an iteration to each system it keeps running
        RSG_CUDA(cudaMemcpyAsync(h->h_pin, h->d_active, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        RSG_CUDA(cudaStreamSynchronize(h->stream));
        if (h->h_pin[0] <= 0) break;
        if ((rc = gm_phase(h, 0, [&] { launch_gm_cycle_start(h->dp, h->val, h->b, h->V.x, G, h->ks, h->R, h->d_active, h->stream); })))
            return rc;
        h->launches += 2;
        for (int j = 0; j < m; ++j) {
            rc = gm_phase(h, size_t(1 + j), [&] {
                launch_precond_gm(h->dp, M, G.V + size_t(j) * N, G.Z + size_t(j) * N, h->ks, h->S, h->d_err, h->stream);
                launch_gm_step(h->dp, h->val, j, G, h->ks, h->R, h->d_active, h->stream);
            });
            if (rc) return rc;
            h->launches += precond_launches(M) + 3 + j;
            if ((j + 1) % check == 0 || j + 1 == m) {
                RSG_CUDA(cudaMemcpyAsync(h->h_pin + 3, G.inner, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
                RSG_CUDA(cudaStreamSynchronize(h->stream));
                if (h->h_pin[3] <= 0) break;
            }
        }
        if ((rc = gm_phase(h, size_t(m) + 1, [&] { launch_gm_cycle_end(h->dp, h->V.x, G, h->ks, h->d_active, h->stream); }))) return rc;
        h->launches += 3;
    }
    return RSG_OK;
}

// d_b, d_x: caller's vectors in the original row order; the solve runs in level space (h->b, h->V.x)
// Precision escalation of the all-FP32 preconditioner: on systems with extreme coefficient contrasts its FP32
// triangular sweeps can diverge (the divergence guard stops them early). The systems that did not converge are
// solved again from x = 0 with the same FP32 factors -- eliminated in FP64 on the thread-block path, as the grid
// path already has them -- and the sweep vector in FP64 (the mixed form); the converged systems keep their result.
int escalate(rsg_solver* h, double tol, int maxIt, bool gmres = false) {
    std::vector<KScal> k0(size_t(h->plan.nsys));
    RSG_CUDA(cudaMemcpyAsync(k0.data(), h->ks, sizeof(KScal) * k0.size(), cudaMemcpyDeviceToHost, h->stream));
    RSG_CUDA(cudaStreamSynchronize(h->stream));
    int failed = 0;
    for (const KScal& k : k0) failed += k.status != ST_CONV;
    if (!failed) return RSG_OK;
    if (h->cta) {
        ++h->epoch;
        launch_factor_lean(h->dp, h->val, h->luf, h->work, h->S, h->epoch, h->d_nreg, h->d_err, h->stream);
        launch_pack_f32(h->dp, h->luf, h->s32, h->stream);
        h->launches += 2;
        RSG_CUDA(cudaGetLastError());
    }
    h->escalated = true;
    h->st.escalated_systems = failed;
    return gmres ? run_gmres(h, tol, maxIt, true) : run_bicgstab(h, tol, maxIt, true);
}

int do_solve_device(rsg_solver* h, const double* d_b, double* d_x, double tol, int maxIt, int* iterations, double* relres) {
    if (h->genActive) {
        const int rc = gen_solve_device(h->gen, h->opt, d_b, d_x, tol, maxIt, iterations, relres);
        gen_stats(h->gen, &h->st);
        return rc;
    }
    if (!h->haveSetup) return fail(RSG_ESTATE, "solve before setup");
    if (!(tol > 0) || maxIt < 0) return fail(RSG_EINVAL, "tol must be > 0 and maxIt >= 0");
    RSG_CUDA(cudaEventRecord(h->ev0, h->stream));
    launch_gather_vec(h->dp, d_b, h->b, h->stream);
    h->launches += 3;   // gather, scatter, true residual
    RSG_CUDA(cudaGetLastError());
    int rc;
    if (h->opt.krylov == RSG_KRYLOV_GMRES) {
        if ((rc = run_gmres(h, tol, maxIt, false))) return rc;
        // precision form: systems GMRES left unconverged (the all-FP32 sweeps can stall on hard systems) are solved
        // again with FP64 sweep vectors, as after BiCGSTAB; converged systems keep their result
        if (h->opt.precision == RSG_MIXED_F32 && h->opt.precond != RSG_PREC_CPR_DEVICE && h->opt.precond != RSG_PREC_JACOBI &&
            !h->escalated && (rc = escalate(h, tol, maxIt, true)))
            return rc;
    } else {
        if ((rc = run_bicgstab(h, tol, maxIt))) return rc;
        if (h->opt.precision == RSG_MIXED_F32 && h->opt.precond != RSG_PREC_CPR_DEVICE && h->opt.precond != RSG_PREC_JACOBI &&
            !h->escalated && (rc = escalate(h, tol, maxIt)))
            return rc;
        if (h->opt.gmres_fallback) {
            // systems that did not converge are solved again with GMRES from x = 0; per system the result with the
            // smaller recursive residual is kept (engine/src/simulator.cpp:3388-3398)
            std::vector<KScal> k0(size_t(h->plan.nsys));
            RSG_CUDA(cudaMemcpyAsync(k0.data(), h->ks, sizeof(KScal) * k0.size(), cudaMemcpyDeviceToHost, h->stream));
            RSG_CUDA(cudaStreamSynchronize(h->stream));
            bool failed = false;
            for (const KScal& k : k0) failed |= k.status != ST_CONV;
            if (failed) {
                const size_t N = size_t(h->plan.n) * NB;
                if (!h->xPrev && ((rc = dalloc(h->pmem, &h->xPrev, N)) || (rc = dalloc(h->pmem, &h->ksPrev, size_t(h->plan.nsys)))))
                    return rc;
                RSG_CUDA(cudaMemcpyAsync(h->xPrev, h->V.x, N * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
                RSG_CUDA(cudaMemcpyAsync(h->ksPrev, h->ks, sizeof(KScal) * size_t(h->plan.nsys), cudaMemcpyDeviceToDevice, h->stream));
                if ((rc = run_gmres(h, tol, maxIt, true))) return rc;
                launch_gm_pick(h->dp, h->V.x, h->xPrev, h->ksPrev, h->ks, h->stream);
                h->launches += 2;
                RSG_CUDA(cudaGetLastError());
            }
        }
    }
    launch_scatter_vec(h->dp, h->V.x, d_x, h->stream);
    RSG_CUDA(cudaEventRecord(h->ev1, h->stream));
    launch_true_residual(h->dp, h->val, h->b, h->V.x, nullptr, h->R, h->d_trueres, h->stream);
    RSG_CUDA(cudaGetLastError());
    if ((rc = check_device_errors(h))) return rc;
    h->hks.resize(size_t(h->plan.nsys));
    h->htrue.resize(size_t(h->plan.nsys));
    RSG_CUDA(cudaMemcpyAsync(h->hks.data(), h->ks, sizeof(KScal) * h->hks.size(), cudaMemcpyDeviceToHost, h->stream));
    RSG_CUDA(cudaMemcpyAsync(h->htrue.data(), h->d_trueres, sizeof(double) * h->htrue.size(), cudaMemcpyDeviceToHost, h->stream));
    RSG_CUDA(cudaStreamSynchronize(h->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    int maxits = 0, conv = 1, brk = 0;
    double mrel = 0, mtrue = 0;
    for (size_t s = 0; s < h->hks.size(); ++s) {
        const KScal& k = h->hks[s];
        maxits = std::max(maxits, k.its);
        mrel = std::max(mrel, k.relres);
        mtrue = std::max(mtrue, h->htrue[s]);
        if (k.status != ST_CONV) conv = 0;
        if (k.status == ST_BREAKDOWN) brk = 1;
    }
    h->st.iterations = maxits;
    h->st.converged = conv;
    h->st.rel_residual = mrel;
    h->st.true_rel_residual = mtrue;
    h->st.solve_ms = ms;
    h->st.device_bytes = h->mem.bytes + h->pmem.bytes;
    if (iterations) *iterations = maxits;
    if (relres) *relres = mrel;
    if (conv) return RSG_OK;
    if (brk) return fail(RSG_EBREAKDOWN, "Krylov breakdown before convergence");
    return RSG_ENOTCONV;
}

// FP64 defect correction around the handle's own solver (refineWithDevice, engine/src/bsr.cpp:1373-1396), per system
// of the batch: x = 0, r = b; up to maxOuter times, while ||r|| / ||b|| > tol, solve A d = r with the handle's solver
// to innerTol = clamp(10 tol, 1e-4, 1e-2) and at most innerIt iterations, x += d, r = b - A x (FP64 SpMV and norms on
// the device). A system already within the tolerance gets a zero right-hand side, so its correction is exactly zero.
// Iterations are the sum of the inner iterations; a system converges when its final FP64 residual is within tol.
int do_solve_refined(rsg_solver* h, const double* d_b, double* d_x, double tol, int maxOuter, int innerIt, int* iterations,
                     double* relres) {
    if (!h->haveSetup) return fail(RSG_ESTATE, "solve before setup");
    if (!(tol > 0) || maxOuter < 0 || innerIt < 0) return fail(RSG_EINVAL, "tol must be > 0, maxOuter and innerIt >= 0");
    const size_t N = size_t(h->plan.n) * NB;
    const int ns = h->plan.nsys;
    int rc;
    if (!h->refB && ((rc = dalloc(h->pmem, &h->refB, N)) || (rc = dalloc(h->pmem, &h->refX, N)) || (rc = dalloc(h->pmem, &h->refR, N)) ||
                     (rc = dalloc(h->pmem, &h->refRel, size_t(ns)))))
        return rc;
    RSG_CUDA(cudaEventRecord(h->ev0, h->stream));
    launch_gather_vec(h->dp, d_b, h->refB, h->stream);
    RSG_CUDA(cudaMemsetAsync(h->refX, 0, N * sizeof(double), h->stream));
    h->launches += 1;
    const double innerTol = std::max(1e-4, std::min(1e-2, tol * 10));
    std::vector<int> its(size_t(ns), 0);
    std::vector<double> rel(size_t(ns), 0.0);
    std::vector<KScal> k(static_cast<size_t>(ns));
    // a system whose inner solve breaks down or ends non-finite stops refining with the x it has, as the reference
    // ends its loop when the device solve fails (engine/src/bsr.cpp:1387)
    std::vector<char> stopped(static_cast<size_t>(ns), 0);
    int escalatedMax = 0;
    for (int outer = 0;; ++outer) {
        // r = b - A x and ||r|| / ||b|| per system (0 for a zero right-hand side, which is converged)
        launch_true_residual(h->dp, h->val, h->refB, h->refX, h->refR, h->R, h->refRel, h->stream);
        h->launches += 1;
        RSG_CUDA(cudaGetLastError());
        RSG_CUDA(cudaMemcpyAsync(rel.data(), h->refRel, sizeof(double) * rel.size(), cudaMemcpyDeviceToHost, h->stream));
        RSG_CUDA(cudaStreamSynchronize(h->stream));
        bool any = false;
        for (int sy = 0; sy < ns; ++sy) {
            if (rel[size_t(sy)] <= tol || stopped[size_t(sy)]) {
                const size_t r0 = size_t(h->plan.sysRow0[size_t(sy)]) * NB, r1 = size_t(h->plan.sysRow0[size_t(sy) + 1]) * NB;
                RSG_CUDA(cudaMemsetAsync(h->refR + r0, 0, (r1 - r0) * sizeof(double), h->stream));
            } else {
                any = true;
            }
        }
        if (!any || outer >= maxOuter) break;
        double* bSave = h->b;
        h->b = h->refR;
        rc = h->opt.krylov == RSG_KRYLOV_GMRES ? run_gmres(h, innerTol, innerIt, false) : run_bicgstab(h, innerTol, innerIt);
        if (!rc && h->opt.precision == RSG_MIXED_F32 && h->opt.precond != RSG_PREC_CPR_DEVICE && h->opt.precond != RSG_PREC_JACOBI &&
            !h->escalated)
            rc = escalate(h, innerTol, innerIt, h->opt.krylov == RSG_KRYLOV_GMRES);
        h->b = bSave;
        if (rc) return rc;
        escalatedMax = std::max(escalatedMax, h->st.escalated_systems);
        RSG_CUDA(cudaMemcpyAsync(k.data(), h->ks, sizeof(KScal) * k.size(), cudaMemcpyDeviceToHost, h->stream));
        RSG_CUDA(cudaStreamSynchronize(h->stream));
        for (int sy = 0; sy < ns; ++sy) {
            if (rel[size_t(sy)] <= tol || stopped[size_t(sy)]) continue;
            its[size_t(sy)] += k[size_t(sy)].its;
            if (k[size_t(sy)].status == ST_BREAKDOWN || !std::isfinite(k[size_t(sy)].relres)) {
                stopped[size_t(sy)] = 1;                          // its correction is not added
                const size_t r0 = size_t(h->plan.sysRow0[size_t(sy)]) * NB, r1 = size_t(h->plan.sysRow0[size_t(sy) + 1]) * NB;
                RSG_CUDA(cudaMemsetAsync(h->V.x + r0, 0, (r1 - r0) * sizeof(double), h->stream));
            }
        }
        launch_vec_add(h->plan.n, h->refX, h->V.x, h->stream);
        h->launches += 1;
        RSG_CUDA(cudaGetLastError());
    }
    // results as the plain solve reports them: per system its, relres and status in the device scalars
    RSG_CUDA(cudaMemcpyAsync(k.data(), h->ks, sizeof(KScal) * k.size(), cudaMemcpyDeviceToHost, h->stream));
    RSG_CUDA(cudaStreamSynchronize(h->stream));
    for (int sy = 0; sy < ns; ++sy) {
        KScal& q = k[size_t(sy)];
        q.its = its[size_t(sy)];
        q.relres = rel[size_t(sy)];
        q.status = rel[size_t(sy)] <= tol ? ST_CONV : ST_MAXIT;
    }
    RSG_CUDA(cudaMemcpyAsync(h->ks, k.data(), sizeof(KScal) * k.size(), cudaMemcpyHostToDevice, h->stream));
    launch_scatter_vec(h->dp, h->refX, d_x, h->stream);
    RSG_CUDA(cudaEventRecord(h->ev1, h->stream));
    RSG_CUDA(cudaMemcpyAsync(h->d_trueres, h->refRel, sizeof(double) * size_t(ns), cudaMemcpyDeviceToDevice, h->stream));
    h->launches += 1;
    RSG_CUDA(cudaGetLastError());
    if ((rc = check_device_errors(h))) return rc;
    h->hks = k;
    h->htrue = rel;
    float ms = 0;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    int maxits = 0, conv = 1;
    double mrel = 0;
    for (int sy = 0; sy < ns; ++sy) {
        maxits = std::max(maxits, its[size_t(sy)]);
        mrel = std::max(mrel, rel[size_t(sy)]);
        conv &= rel[size_t(sy)] <= tol;
    }
    h->st.iterations = maxits;
    h->st.converged = conv;
    h->st.rel_residual = mrel;
    h->st.true_rel_residual = mrel;
    h->st.solve_ms = ms;
    h->st.escalated_systems = escalatedMax;
    h->st.device_bytes = h->mem.bytes + h->pmem.bytes;
    if (iterations) *iterations = maxits;
    if (relres) *relres = mrel;
    return conv ? RSG_OK : RSG_ENOTCONV;
}

// full right-hand sides (cells, then wells, per system) in, full solutions out: the reduction, the block solve, the
// recovery of the BHPs (WellSchur::reduceRhs / recover, engine/src/bsr.cpp:973-990), all on the device
int do_solve_jacobian(rsg_solver* h, const double* d_b, double* d_x, double tol, int maxIt, int* iterations, double* relres) {
    if (!h->jac || !h->wsValues) return fail(RSG_ESTATE, "solve_jacobian before set_jacobian");
    if (!h->haveSetup) return fail(RSG_ESTATE, "solve before setup");
    launch_ws_rhs(h->wsd, h->jv, d_b, h->wsBc, h->stream);
    h->launches += 1;
    const int rc = do_solve_device(h, h->wsBc, h->wsXc, tol, maxIt, iterations, relres);
    if (rc < 0) return rc;
    launch_ws_recover(h->wsd, h->jv, d_b, h->wsXc, d_x, h->stream);
    h->launches += 1;
    RSG_CUDA(cudaGetLastError());
    return rc;
}

}  // namespace

extern "C" {

int rsg_set_jacobian(rsg_solver* h, int nrows, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw) {
    if (!h) return fail(RSG_EINVAL, "null handle");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    return do_set_jacobian(h, 1, nv, &nrows, &na, &nw, &rowPtr, &col, &val, nullptr);
}

int rsg_set_jacobian_batch(rsg_solver* h, int nsys, int nv, const int* nrows, const int* na, const int* nw, const int* const* rowPtr,
                           const int* const* col, const double* const* val) {
    if (!h) return fail(RSG_EINVAL, "null handle");
    if (!val) return fail(RSG_EINVAL, "set_jacobian_batch: null values");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    return do_set_jacobian(h, nsys, nv, nrows, na, nw, rowPtr, col, val, nullptr);
}

int rsg_set_jacobian_device(rsg_solver* h, int nrows, const int* rowPtr, const int* col, const double* d_val, int na, int nv, int nw) {
    if (!h || !d_val) return fail(RSG_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    return do_set_jacobian(h, 1, nv, &nrows, &na, &nw, &rowPtr, &col, nullptr, d_val);
}

int rsg_solve_jacobian(rsg_solver* h, const double* b, double* x, double tol, int maxIt, int* iterations, double* relres) {
    if (!h || !b || !x) return fail(RSG_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    if (!h->jac || !h->wsPlanned) return fail(RSG_ESTATE, "solve_jacobian before set_jacobian");
    const size_t N = size_t(h->ws.full0.back());
    RSG_CUDA(cudaMemcpyAsync(h->wsB, b, N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    const int rc = do_solve_jacobian(h, h->wsB, h->wsX, tol, maxIt, iterations, relres);
    if (rc < 0) return rc;
    RSG_CUDA(cudaMemcpyAsync(x, h->wsX, N * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    RSG_CUDA(cudaStreamSynchronize(h->stream));
    return rc;
}

int rsg_solve_jacobian_device(rsg_solver* h, const double* d_b, double* d_x, double tol, int maxIt, int* iterations, double* relres) {
    if (!h || !d_b || !d_x) return fail(RSG_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    return do_solve_jacobian(h, d_b, d_x, tol, maxIt, iterations, relres);
}

int rsg_get_matrix(rsg_solver* h, int* rowPtr, int* col, double* val) {
    if (!h) return fail(RSG_EINVAL, "null handle");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    if (!h->haveMatrix) return fail(RSG_ESTATE, "get_matrix before set_matrix / set_jacobian");
    const HostPlan& P = h->plan;
    if (rowPtr) std::copy(P.rowPtr0.begin(), P.rowPtr0.end(), rowPtr);
    if (col) std::copy(P.col0.begin(), P.col0.end(), col);
    if (val) {
        RSG_CUDA(cudaMemcpyAsync(val, h->val0, size_t(P.nnzb) * NB2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        RSG_CUDA(cudaStreamSynchronize(h->stream));
    }
    return RSG_OK;
}

int rsg_matrix_size(rsg_solver* h, int* n, long long* nnzb) {
    if (!h) return fail(RSG_EINVAL, "null handle");
    std::lock_guard<std::mutex> lk(h->mu);
    if (!h->havePlan) return fail(RSG_ESTATE, "no matrix");
    if (n) *n = h->plan.n;
    if (nnzb) *nnzb = h->plan.nnzb;
    return RSG_OK;
}

const char* rsg_version(void) { return "rsg 0.1 (sm_103a)"; }
const char* rsg_last_error(void) { return g_err.c_str(); }

void rsg_default_options(rsg_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->precond = RSG_PREC_BILU0;
    o->krylov = RSG_KRYLOV_BICGSTAB;
    o->restart = 40;
    o->precision = RSG_FP64;
    o->gmres_fallback = 0;
    o->fma = 1;
    o->check_every = 4;
    o->use_graphs = 1;
    o->device = 0;
    o->mem_budget = 0;
    o->sweep = 0;
    o->autotune = 1;
    o->vcycle_form = 0;
    o->cpr2_threads = 0;
}

int rsg_create(rsg_solver** out, const rsg_options* opts) {
    if (!out) return fail(RSG_EINVAL, "null handle pointer");
    *out = nullptr;
    rsg_options o;
    rsg_default_options(&o);
    if (opts) o = *opts;
    if (o.precond < 0 || o.precond > 4 || o.krylov < 0 || o.krylov > 1 || o.precision < 0 || o.precision > 2 || o.sweep < 0 || o.sweep > 3)
        return fail(RSG_EINVAL, "invalid options");
    if (o.vcycle_form < 0 || o.vcycle_form > 3 ||
        (o.cpr2_threads != 0 && o.cpr2_threads != 128 && o.cpr2_threads != 256 && o.cpr2_threads != 512))
        return fail(RSG_EINVAL, "invalid launch shape options (vcycle_form 0..3, cpr2_threads 0 / 128 / 256 / 512)");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return fail(RSG_ECUDA, "no CUDA device available");
    if (o.device < 0 || o.device >= ndev) return fail(RSG_EINVAL, "device ordinal out of range");
    RSG_CUDA(cudaSetDevice(o.device));
    rsg_solver* h = new rsg_solver();
    h->opt = o;
    h->device = o.device;
    h->mem.budget = o.mem_budget;
    auto bail = [&](cudaError_t e, const char* what) {
        std::string m = std::string(what) + ": " + cudaGetErrorString(e);
        if (h->stream) cudaStreamDestroy(h->stream);
        delete h;
        return fail(RSG_ECUDA, m);
    };
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "cudaStreamCreate");
    h->mem.st = h->pmem.st = h->wsPat.st = h->wsVal.st = h->stream;
    if ((e = cudaEventCreate(&h->ev0)) != cudaSuccess) return bail(e, "cudaEventCreate");
    if ((e = cudaEventCreate(&h->ev1)) != cudaSuccess) return bail(e, "cudaEventCreate");
    if ((e = cudaMallocHost(&h->h_pin, 4 * sizeof(int))) != cudaSuccess) return bail(e, "cudaMallocHost");
    int rc;
    if ((rc = dalloc(h->mem, &h->d_active, 1)) || (rc = dalloc(h->mem, &h->d_err, 1)) || (rc = dalloc(h->mem, &h->d_nreg, 1))) {
        h->mem.release_all();
        cudaFreeHost(h->h_pin);
        cudaStreamDestroy(h->stream);
        delete h;
        return rc;
    }
    cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream);
    cudaMemsetAsync(h->d_active, 0, sizeof(int), h->stream);
    *out = h;
    return RSG_OK;
}

int rsg_destroy(rsg_solver* h) {
    if (!h) return RSG_OK;
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    free_plan(h);
    h->mem.release_all();
    if (h->h_pin) cudaFreeHost(h->h_pin);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return RSG_OK;
}

int rsg_release(rsg_solver* h) {
    if (!h) return fail(RSG_EINVAL, "null handle");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    free_plan(h);
    return RSG_OK;
}

int rsg_set_matrix(rsg_solver* h, int n, int nb, const int* rowPtr, const int* col, const double* val) {
    if (!h) return fail(RSG_EINVAL, "null handle");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    return do_set_batch(h, 1, nb, &n, &rowPtr, &col, &val);
}

int rsg_set_batch(rsg_solver* h, int nsys, int nb, const int* n, const int* const* rowPtr, const int* const* col,
                  const double* const* val) {
    if (!h) return fail(RSG_EINVAL, "null handle");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    return do_set_batch(h, nsys, nb, n, rowPtr, col, val);
}

int rsg_setup(rsg_solver* h, const double* acc) {
    if (!h) return fail(RSG_EINVAL, "null handle");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    return do_setup(h, acc);
}

int rsg_solve_device(rsg_solver* h, const double* d_b, double* d_x, double tol, int maxIt, int* iterations, double* relres) {
    if (!h || !d_b || !d_x) return fail(RSG_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    return do_solve_device(h, d_b, d_x, tol, maxIt, iterations, relres);
}

int rsg_solve(rsg_solver* h, const double* b, double* x, double tol, int maxIt, int* iterations, double* relres) {
    if (!h || !b || !x) return fail(RSG_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    if (h->genActive) {
        const int rc = gen_solve_host(h->gen, h->opt, b, x, tol, maxIt, iterations, relres);
        gen_stats(h->gen, &h->st);
        return rc;
    }
    if (!h->havePlan) return fail(RSG_ESTATE, "solve before set_matrix");
    const size_t N = size_t(h->plan.n) * NB;
    RSG_CUDA(cudaMemcpyAsync(h->tmp, b, N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    const int rc = do_solve_device(h, h->tmp, h->xout, tol, maxIt, iterations, relres);
    if (rc < 0) return rc;
    RSG_CUDA(cudaMemcpyAsync(x, h->xout, N * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    RSG_CUDA(cudaStreamSynchronize(h->stream));
    return rc;
}

int rsg_solve_refined(rsg_solver* h, const double* b, double* x, double tol, int maxOuter, int innerIt, int* iterations, double* relres) {
    if (!h || !b || !x) return fail(RSG_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    if (h->genActive) return fail(RSG_EINVAL, "FP64 defect correction is for nb = 3 (block sizes other than 3 already solve in FP64)");
    if (!h->havePlan) return fail(RSG_ESTATE, "solve before set_matrix");
    const size_t N = size_t(h->plan.n) * NB;
    RSG_CUDA(cudaMemcpyAsync(h->tmp, b, N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    const int rc = do_solve_refined(h, h->tmp, h->xout, tol, maxOuter, innerIt, iterations, relres);
    if (rc < 0) return rc;
    RSG_CUDA(cudaMemcpyAsync(x, h->xout, N * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    RSG_CUDA(cudaStreamSynchronize(h->stream));
    return rc;
}

int rsg_batch_results(rsg_solver* h, int* its, double* relres, double* true_relres) {
    if (!h) return fail(RSG_EINVAL, "null handle");
    for (size_t s = 0; s < h->hks.size(); ++s) {
        if (its) its[s] = h->hks[s].its;
        if (relres) relres[s] = h->hks[s].relres;
        if (true_relres) true_relres[s] = h->htrue[s];
    }
    return RSG_OK;
}

int rsg_batch_status(rsg_solver* h, int* status) {
    if (!h || !status) return fail(RSG_EINVAL, "null argument");
    for (size_t s = 0; s < h->hks.size(); ++s) {
        const int st = h->hks[s].status;
        status[s] = st == ST_CONV ? RSG_OK : (st == ST_BREAKDOWN ? RSG_EBREAKDOWN : RSG_ENOTCONV);
    }
    return RSG_OK;
}

int rsg_amg_level_sizes(rsg_solver* h, int maxlev, long long* rows, long long* nnz, long long* dense) {
    if (!h || maxlev < 0 || (maxlev > 0 && (!rows || !nnz))) return fail(RSG_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(h->mu);
    if (h->genActive) return gen_amg_level_sizes(h->gen, maxlev, rows, nnz, dense);
    if (!h->haveAmg) {
        fail(RSG_ESTATE, "no CPR hierarchy (setup not run, or not a CPR preconditioner)");
        return -1;
    }
    const DevAmg& G = h->amg;
    const int nl = std::min(maxlev, G.maxL);
    for (int l = 0; l < nl; ++l) {
        rows[l] = G.levelRowBeg[size_t(l) + 1] - G.levelRowBeg[size_t(l)];
        nnz[l] = G.levelEntBeg[size_t(l) + 1] - G.levelEntBeg[size_t(l)];
    }
    if (dense) *dense = G.totLu;
    return G.maxL;
}

int rsg_spmv_device(rsg_solver* h, const double* d_x, double* d_y) {
    if (!h || !d_x || !d_y) return fail(RSG_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    if (!h->haveMatrix) return fail(RSG_ESTATE, "spmv before set_matrix");
    if (h->genActive) return gen_spmv_device(h->gen, d_x, d_y);
    launch_gather_vec(h->dp, d_x, h->b, h->stream);
    launch_spmv_f64(h->dp, h->val, h->b, h->xout, h->stream);
    launch_scatter_vec(h->dp, h->xout, d_y, h->stream);
    h->launches += 3;
    RSG_CUDA(cudaGetLastError());
    return RSG_OK;
}

// level-space SpMV on the handle's own vectors (per-kernel timing)
int rsg_spmv_level_probe(rsg_solver* h, int reps) {
    if (!h || !h->haveMatrix || h->genActive) return fail(RSG_ESTATE, "spmv before set_matrix (nb = 3)");
    for (int r = 0; r < reps; ++r) launch_spmv_f64(h->dp, h->val, h->V.x, h->xout, h->stream);
    h->launches += reps;
    RSG_CUDA(cudaGetLastError());
    return RSG_OK;
}

int rsg_spmv(rsg_solver* h, const double* x, double* y) {
    if (!h || !x || !y) return fail(RSG_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    if (!h->haveMatrix) return fail(RSG_ESTATE, "spmv before set_matrix");
    if (h->genActive) return gen_spmv_host(h->gen, x, y);
    const size_t N = size_t(h->plan.n) * NB;
    RSG_CUDA(cudaMemcpyAsync(h->tmp, x, N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    launch_gather_vec(h->dp, h->tmp, h->b, h->stream);
    launch_spmv_f64(h->dp, h->val, h->b, h->xout, h->stream);
    launch_scatter_vec(h->dp, h->xout, h->tmp, h->stream);
    h->launches += 3;
    RSG_CUDA(cudaGetLastError());
    RSG_CUDA(cudaMemcpyAsync(y, h->tmp, N * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    RSG_CUDA(cudaStreamSynchronize(h->stream));
    return RSG_OK;
}

// level-space r -> level-space z

int rsg_precond_apply_device(rsg_solver* h, const double* d_r, double* d_z) {
    if (!h || !d_r || !d_z) return fail(RSG_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    if (!h->haveSetup) return fail(RSG_ESTATE, "precond_apply before setup");
    if (h->genActive) return gen_precond_device(h->gen, d_r, d_z);
    launch_gather_vec(h->dp, d_r, h->b, h->stream);
    int rc = precond_apply_dev(h, h->b, h->xout);
    if (rc) return rc;
    launch_scatter_vec(h->dp, h->xout, d_z, h->stream);
    h->launches += 2;
    RSG_CUDA(cudaGetLastError());
    return RSG_OK;
}

// level-space preconditioner application on the handle's own vectors (per-kernel timing)
int rsg_precond_level_probe(rsg_solver* h, int reps) {
    if (!h || !h->haveSetup || h->genActive) return fail(RSG_ESTATE, "precond_apply before setup (nb = 3)");
    for (int r = 0; r < reps; ++r) {
        int rc = precond_apply_dev(h, h->b, h->xout);
        if (rc) return rc;
    }
    return RSG_OK;
}

int rsg_precond_apply(rsg_solver* h, const double* r, double* z) {
    if (!h || !r || !z) return fail(RSG_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    if (!h->haveSetup) return fail(RSG_ESTATE, "precond_apply before setup");
    if (h->genActive) return gen_precond_host(h->gen, r, z);
    const size_t N = size_t(h->plan.n) * NB;
    RSG_CUDA(cudaMemcpyAsync(h->tmp, r, N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    launch_gather_vec(h->dp, h->tmp, h->b, h->stream);
    int rc = precond_apply_dev(h, h->b, h->xout);
    if (rc) return rc;
    launch_scatter_vec(h->dp, h->xout, h->tmp, h->stream);
    h->launches += 2;
    rc = check_device_errors(h);
    if (rc) return rc;
    RSG_CUDA(cudaMemcpyAsync(z, h->tmp, N * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    RSG_CUDA(cudaStreamSynchronize(h->stream));
    return RSG_OK;
}

int rsg_get_factors(rsg_solver* h, double* lu) {
    if (!h || !lu) return fail(RSG_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(h->mu);
    cudaSetDevice(h->device);
    if (h->genActive) return gen_get_factors(h->gen, lu);
    if (!h->haveSetup || (!h->lu && !h->luf)) return fail(RSG_ESTATE, "no BILU0 factors (setup not run, or not a BILU0 / CPR path)");
    std::vector<double> lev(size_t(h->plan.nnzb) * NB2);
    if (h->lu) {
        RSG_CUDA(cudaMemcpyAsync(lev.data(), h->lu, lev.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        RSG_CUDA(cudaStreamSynchronize(h->stream));
    } else {                                     // FP32 factors of the mixed forms, exactly widened
        std::vector<float> f(lev.size());
        RSG_CUDA(cudaMemcpyAsync(f.data(), h->luf, f.size() * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
        RSG_CUDA(cudaStreamSynchronize(h->stream));
        for (size_t e = 0; e < f.size(); ++e) lev[e] = double(f[e]);
    }
    for (size_t p = 0; p < size_t(h->plan.nnzb); ++p)   // back to the caller's block order
        std::memcpy(lu + size_t(h->plan.valSrc[p]) * NB2, lev.data() + p * NB2, sizeof(double) * NB2);
    return RSG_OK;
}

int rsg_tuning(rsg_solver* h, char* buf, int len) {
    if (!h || !buf || len < 1) return fail(RSG_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(h->mu);
    std::snprintf(buf, size_t(len), "%s", h->genActive ? "block-size-generic path: fixed shapes" : h->tune.desc.c_str());
    return RSG_OK;
}

int rsg_get_stats(rsg_solver* h, rsg_stats* st) {
    if (!h || !st) return fail(RSG_EINVAL, "null argument");
    if (h->genActive) {
        gen_stats(h->gen, st);
        st->device_bytes += h->mem.bytes;
        return RSG_OK;
    }
    *st = h->st;
    st->device_bytes = h->mem.bytes + h->pmem.bytes;
    st->kernel_launches = h->launches;
    return RSG_OK;
}

void* rsg_stream(rsg_solver* h) { return h ? (void*)h->stream : nullptr; }

int rsg_wellschur_reduce(int nrows, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw,
                         const double* b, int* nnzb, int* sRowPtr, int* sCol, double* sVal, double* bc) {
    if (!rowPtr || !col || !val || !nnzb) return fail(RSG_EINVAL, "null argument");
    std::string err;
    if (wellschur_reduce(nrows, rowPtr, col, val, na, nv, nw, b, nnzb, sRowPtr, sCol, sVal, bc, err)) return fail(RSG_EINVAL, err);
    return RSG_OK;
}

int rsg_wellschur_recover(int nrows, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw,
                          const double* b, const double* xc, double* x) {
    if (!rowPtr || !col || !val || !b || !xc || !x) return fail(RSG_EINVAL, "null argument");
    std::string err;
    if (wellschur_recover(nrows, rowPtr, col, val, na, nv, nw, b, xc, x, err)) return fail(RSG_EINVAL, err);
    return RSG_OK;
}

}  // extern "C"
