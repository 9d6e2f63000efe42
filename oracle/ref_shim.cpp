// C-ABI shim over the reference's own solver classes (test infrastructure only).
//
// Compiled against the reference engine built from its sources (oracle/Makefile.ref) on the machine
// where the reference tree exists; used by tests/golden/make_golden.py to produce golden vectors and
// by the CPU tests to cross-check the C restatement (oracle/rsg_oracle.c). Never shipped, never part
// of the product path.
//
// Entry points wrap, without changing their arithmetic:
//   BSR::spmv                    engine/src/bsr.cpp:109-126
//   BILU0::factor / apply        engine/src/bsr.cpp:347-596
//   BILU0f::factor / apply       engine/src/bsr.cpp:1087-1121
//   BlockCPR::setup / apply      engine/src/bsr.cpp:993-1084
//   AMG hierarchy                engine/src/amg.cpp:137-337
//   bicgstab / gmres             engine/src/linsolve.cpp:159-273
//   WellSchur build/reduce/recover engine/src/bsr.cpp:733-990
//   CpuFloatBlockSolver, refineWithDevice engine/src/bsr.cpp:1130-1215,1373-1396
//   DeviceCprAmg build / apply   engine/src/bsr.cpp:1217-1371
//   MCBILU0 factor / apply       engine/src/bsr.cpp:599-730
#define private public      // read the factor storage of BILU0 (layout is unchanged by access specifiers)
#include "ressim/bsr.h"
#undef private
#include "ressim/linsolve.h"
#include <cstdlib>
#include <cstring>
#include <vector>

using namespace ressim;

namespace {
BSR makeBsr(int n, int nb, const int* rowPtr, const int* col, const double* val) {
    BSR A; A.n = n; A.nb = nb;
    A.rowPtr.assign(rowPtr, rowPtr + n + 1);
    A.col.assign(col, col + rowPtr[n]);
    A.val.assign(val, val + size_t(rowPtr[n]) * nb * nb);
    A.finalizeDiag();
    return A;
}
void setLevelMode(int mode) {
    // 0 = serial sweeps, 2 = level-ordered contiguous storage (engine/src/bsr.cpp:296-313)
    if (mode == 2) setenv("RESSIM_LEVEL_ILU", "2", 1); else setenv("RESSIM_LEVEL_ILU", "0", 1);
}
}  // namespace

extern "C" {

void ref_set_threads(int n) { setNumThreads(n); }

void ref_bsr_spmv(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* x, double* y) {
    const BSR A = makeBsr(n, nb, rowPtr, col, val);
    A.spmv(x, y);
}

// BILU0 factors in the original numbering: L strictly lower, U_ii^-1 on the diagonal, U upper.
int ref_bilu0_factor(int n, int nb, const int* rowPtr, const int* col, const double* val, double* lu) {
    setLevelMode(0);
    const BSR A = makeBsr(n, nb, rowPtr, col, val);
    BILU0 M; M.factor(A);
    std::memcpy(lu, M.LU_.val.data(), sizeof(double) * M.LU_.val.size());
    return M.regularisedBlocks();
}

int ref_bilu0_apply(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* r, double* z, int levelMode) {
    setLevelMode(levelMode);
    const BSR A = makeBsr(n, nb, rowPtr, col, val);
    BILU0 M; M.factor(A);
    M.apply(r, z);
    return M.regularisedBlocks();
}

void ref_bilu0f_apply(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* r, double* z) {
    const BSR A = makeBsr(n, nb, rowPtr, col, val);
    BILU0f M; M.factor(A);
    M.apply(r, z);
}

// prec: 0 = BILU0, 1 = BlockCPR (AMG + BILU0), acc optional (true-IMPES weights)
static const Preconditioner* makePrec(int prec, const BSR& A, const double* acc, BILU0& ilu, BlockCPR& cpr) {
    if (prec == 1) { cpr.setup(A, acc); return &cpr; }
    ilu.factor(A); return &ilu;
}

int ref_prec_apply(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* acc, int prec, const double* r, double* z) {
    setLevelMode(0);
    const BSR A = makeBsr(n, nb, rowPtr, col, val);
    BILU0 ilu; BlockCPR cpr;
    const Preconditioner* M = makePrec(prec, A, acc, ilu, cpr);
    M->apply(r, z);
    return prec == 1 ? cpr.amg().levels() : 0;
}

// method: 0 = bicgstab, 1 = gmres(restart)
int ref_solve(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* acc, int prec, int method,
              int restart, const double* b, double* x, double tol, int maxIt, int* its, double* relres) {
    setLevelMode(0);
    const BSR A = makeBsr(n, nb, rowPtr, col, val);
    BILU0 ilu; BlockCPR cpr;
    const Preconditioner* M = makePrec(prec, A, acc, ilu, cpr);
    std::vector<double> bv(b, b + size_t(n) * nb), xv;
    BsrOperator op(A);
    const LinResult r = method == 1 ? gmres(op, *M, bv, xv, tol, maxIt, restart) : bicgstab(op, *M, bv, xv, tol, maxIt);
    std::memcpy(x, xv.data(), sizeof(double) * xv.size());
    *its = r.iterations; *relres = r.relResidual;
    return r.converged ? 1 : 0;
}

// CPR weights (n*nb) and the AMG hierarchy summary: sizes[l] = rows, nnz[l] = nonzeros of level l
int ref_cpr_info(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* acc, double* w, int* sizes, int* nnz, int maxLevels) {
    const BSR A = makeBsr(n, nb, rowPtr, col, val);
    BlockCPR cpr; cpr.setup(A, acc);
    std::memcpy(w, cpr.weights().data(), sizeof(double) * cpr.weights().size());
    const auto& H = cpr.amg().hierarchy();
    const int L = int(H.size());
    for (int l = 0; l < L && l < maxLevels; ++l) { sizes[l] = H[size_t(l)].A.n; nnz[l] = int(H[size_t(l)].A.col.size()); }
    return L;
}

// AMG level l: its matrix (CSR) and aggregation (P column of every fine row; -1 on the coarsest level)
int ref_amg_level(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* acc, int l,
                  int* rowPtrOut, int* colOut, double* valOut, int* agg) {
    const BSR A = makeBsr(n, nb, rowPtr, col, val);
    BlockCPR cpr; cpr.setup(A, acc);
    const auto& H = cpr.amg().hierarchy();
    if (l >= int(H.size())) return -1;
    const auto& L = H[size_t(l)];
    std::memcpy(rowPtrOut, L.A.rowPtr.data(), sizeof(int) * L.A.rowPtr.size());
    std::memcpy(colOut, L.A.col.data(), sizeof(int) * L.A.col.size());
    std::memcpy(valOut, L.A.val.data(), sizeof(double) * L.A.val.size());
    if (agg) for (int i = 0; i < L.A.n; ++i) agg[i] = L.pRow.empty() ? -1 : L.pCol[size_t(L.pRow[size_t(i)])];
    return L.A.n;
}

// WellSchur on a scalar CSR with well rows: S (BSR), bc; then recover x from xc
int ref_wellschur(int nrows, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw, const double* b,
                  int* sRowPtr, int* sCol, double* sVal, double* bc, int* nnzbOut) {
    CSR A; A.n = nrows; A.rowPtr.assign(rowPtr, rowPtr + nrows + 1); A.col.assign(col, col + rowPtr[nrows]);
    A.val.assign(val, val + rowPtr[nrows]); A.finalizeDiag();
    WellSchur W;
    if (!W.build(A, na, nv, nw)) return 0;
    const BSR& S = W.reduced();
    *nnzbOut = S.nnzb();
    if (sRowPtr) {
        std::memcpy(sRowPtr, S.rowPtr.data(), sizeof(int) * S.rowPtr.size());
        std::memcpy(sCol, S.col.data(), sizeof(int) * S.col.size());
        std::memcpy(sVal, S.val.data(), sizeof(double) * S.val.size());
        W.reduceRhs(b, bc);
    }
    return 1;
}

int ref_wellschur_recover(int nrows, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw, const double* b,
                          const double* xc, double* x) {
    CSR A; A.n = nrows; A.rowPtr.assign(rowPtr, rowPtr + nrows + 1); A.col.assign(col, col + rowPtr[nrows]);
    A.val.assign(val, val + rowPtr[nrows]); A.finalizeDiag();
    WellSchur W;
    if (!W.build(A, na, nv, nw)) return 0;
    W.recover(b, xc, x);
    return 1;
}

// float32 device algorithm emulation (BILU0f-BiCGSTAB in float) wrapped in double refinement
int ref_refine_float(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* b, double* x, double tol,
                     int maxOuter, int innerIt, int* its, double* relres) {
    const BSR A = makeBsr(n, nb, rowPtr, col, val);
    CpuFloatBlockSolver dev;
    std::vector<double> bv(b, b + size_t(n) * nb), xv;
    const LinResult r = refineWithDevice(dev, A, bv, xv, tol, maxOuter, innerIt);
    std::memcpy(x, xv.data(), sizeof(double) * xv.size());
    *its = r.iterations; *relres = r.relResidual;
    return r.converged ? 1 : 0;
}

// multicolour BILU0 (MCBILU0::factor / apply, engine/src/bsr.cpp:599-730): z = M^-1 r, returns the colours
int ref_mcbilu0_apply(int n, int nb, const int* rowPtr, const int* col, const double* val, const double* r, double* z) {
    const BSR A = makeBsr(n, nb, rowPtr, col, val);
    MCBILU0 M;
    M.factor(A);
    M.apply(r, z);
    return M.colours();
}

// GPU-shaped float CPR-AMG (DeviceCprAmg::build / apply, engine/src/bsr.cpp:1217-1371): z = M^-1 r in float
int ref_devcpr_apply(int n, int nb, const int* rowPtr, const int* col, const double* val, const float* r, float* z) {
    const BSR A = makeBsr(n, nb, rowPtr, col, val);
    DeviceCprAmg D;
    if (!D.build(A)) return 0;
    std::vector<float> Av(A.val.size());
    for (size_t e = 0; e < Av.size(); ++e) Av[e] = float(A.val[e]);
    D.apply(A, Av, r, z);
    return int(D.lv.size());
}

}  // extern "C"

// ---- the reference CPU path over an ensemble (the timed CPU baseline): one BlockCPR per realisation, as one
// simulator per realisation keeps its own (engine/src/simulator.cpp: bcpr_), set up on each new Jacobian with the AMG
// aggregates reused from the first set-up (BlockCPR::setup reuseAmg, engine/src/bsr.cpp:993-1059), then BiCGSTAB
// (engine/src/linsolve.cpp:159-216) from x0 = 0.
#include <atomic>
#include <chrono>
#include <thread>

namespace {
struct RefMember {
    BSR A;
    std::vector<double> b, x;
    BlockCPR cpr;
    bool built = false;
    int its = 0, conv = 0;
    double relres = 0;
};
struct RefEnsemble {
    std::vector<RefMember> m;
};
void solveMember(RefMember& s, double tol, int maxIt) {
    s.cpr.setup(s.A, nullptr, s.built);
    s.built = true;
    BsrOperator op(s.A);
    const LinResult r = bicgstab(op, s.cpr, s.b, s.x, tol, maxIt);
    s.its = r.iterations;
    s.relres = r.relResidual;
    s.conv = r.converged ? 1 : 0;
}
}  // namespace

extern "C" {

int ref_physical_cores() { return physicalCores(); }

void* ref_ens_create(int nsys) {
    auto* e = new RefEnsemble;
    e->m.resize(size_t(nsys));
    return e;
}

void ref_ens_set(void* h, int s, int n, int nb, const int* rowPtr, const int* col, const double* val, const double* b) {
    RefMember& m = static_cast<RefEnsemble*>(h)->m[size_t(s)];
    m.A = makeBsr(n, nb, rowPtr, col, val);
    m.b.assign(b, b + size_t(n) * nb);
    m.built = false;
}

// One step over every member: set-up (AMG refresh after the first) and solve. workers <= 1: one member after another
// with the reference's OpenMP on `threads` threads (<= 0: its default, one per physical core); workers > 1: that many
// members at once, one OpenMP thread each. Returns the wall seconds of the step.
double ref_ens_step(void* h, double tol, int maxIt, int workers, int threads) {
    RefEnsemble& e = *static_cast<RefEnsemble*>(h);
    unsetenv("RESSIM_LEVEL_ILU");   // the engine's own choice of BILU0 sweep (serial / contiguous levels)
    const auto t0 = std::chrono::steady_clock::now();
    if (workers <= 1) {
        setNumThreads(threads);
        for (RefMember& s : e.m) solveMember(s, tol, maxIt);
    } else {
        std::atomic<size_t> next{0};
        std::vector<std::thread> pool;
        for (int w = 0; w < workers; ++w)
            pool.emplace_back([&] {
                setNumThreads(1);
                for (size_t k; (k = next.fetch_add(1)) < e.m.size();) solveMember(e.m[k], tol, maxIt);
            });
        for (auto& t : pool) t.join();
    }
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

int ref_ens_result(void* h, int s, double* x, int* its, double* relres) {
    const RefMember& m = static_cast<RefEnsemble*>(h)->m[size_t(s)];
    if (x) std::memcpy(x, m.x.data(), sizeof(double) * m.x.size());
    if (its) *its = m.its;
    if (relres) *relres = m.relres;
    return m.conv;
}

void ref_ens_free(void* h) { delete static_cast<RefEnsemble*>(h); }

}  // extern "C"
