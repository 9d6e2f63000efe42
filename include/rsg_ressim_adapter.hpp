// Reference-side binding: ResSim Studio's solver hooks implemented over the rsg C ABI (include/rsg.h).
//
// Header-only C++17; compile it inside the reference engine (it includes the engine's own ressim/bsr.h) and
// link librsg.so. Two adapters:
//
//  * rsg::RsgGpuBlockSolver -- a ressim::GpuBlockSolver (engine/include/ressim/bsr.h:143-151). Register it with
//    ressim::setDistributedSolver() for the FP64 path (the Newton loop trusts its result at the linear tolerance,
//    engine/src/simulator.cpp:3358-3367) or with ressim::setGpuBlockSolver() for the mixed-precision path that
//    the engine wraps in its own FP64 refinement (refineWithDevice, engine/src/simulator.cpp:3368-3378).
//    By default it chooses the preconditioner as the engine does (CPR from 500 cells, else BILU0) and its GMRES
//    fallback is GMRES(60), the engine's. solve() returns false on any device error or non-finite result (and, in
//    the FP64 role, on a solve that missed the tolerance), so the engine falls back to its CPU path.
//    The same hook serves the compositional and thermal simulators, whose blocks are nb = nc + 1 / 4-5 wide: those
//    systems go to a third handle on the library's block-size-generic path, solved as those simulators solve them on
//    the CPU (BlockCPR + GMRES, engine/src/compsim.cpp:1443-1449 with GMRES(60), engine/src/thermsim.cpp:1818-1828
//    with GMRES(80): `genericRestart`), in FP64.
//  * rsg::RsgBlockSolver -- the BlockSolver interface that tools/lsbench.cpp:65-81 expects from the (absent)
//    header ressim/blocksolve.h: full scalar CSR with well rows -> well Schur complement -> device solve ->
//    recovery of the BHPs.
#pragma once
#include "rsg.h"
#include "ressim/bsr.h"

#include <chrono>
#include <cmath>
#include <mutex>
#include <vector>

namespace rsg {

class RsgGpuBlockSolver : public ressim::GpuBlockSolver {
public:
    // Preconditioner choice of the engine itself: CPR from 500 cells, BILU0 below (linearSolver 2,
    // engine/src/simulator.cpp:224)
    static constexpr int kEngineChoice = -1;
    // Distributed: registered with setDistributedSolver, the result must meet the tolerance (false otherwise, and the
    // engine solves the system on its CPU path). Refinement: registered with setGpuBlockSolver, the inner solve of
    // the engine's FP64 defect correction (refineWithDevice, engine/src/bsr.cpp:1373-1396): an iterate that stopped at
    // the iteration limit still corrects x, so only device errors and non-finite results return false.
    enum class Role { Distributed, Refinement };

    explicit RsgGpuBlockSolver(int precision = RSG_FP64, int precond = kEngineChoice, int krylov = RSG_KRYLOV_BICGSTAB,
                               Role role = Role::Distributed, int genericRestart = 60)
        : precond_(precond), role_(role), genericRestart_(genericRestart) {
        rsg_options o;
        rsg_default_options(&o);
        o.precision = precision;
        o.precond = precond == kEngineChoice ? RSG_PREC_CPR : precond;
        o.krylov = krylov;
        o.restart = 60;   // the engine's GMRES fallback is GMRES(60) (engine/src/simulator.cpp:3390)
        o.gmres_fallback = role == Role::Distributed ? 1 : 0;   // try it on the device before handing back to the CPU
        ok_ = rsg_create(&cpr_, &o) == RSG_OK;
        if (ok_ && precond == kEngineChoice) {
            o.precond = RSG_PREC_BILU0;
            ok_ = rsg_create(&ilu_, &o) == RSG_OK;
        }
    }
    ~RsgGpuBlockSolver() override {
        if (cpr_) rsg_destroy(cpr_);
        if (ilu_) rsg_destroy(ilu_);
        if (gen_) rsg_destroy(gen_);
    }
    bool ok() const { return ok_; }
    const char* name() const override { return rsg_version(); }
    bool solve(const ressim::BSR& A, const std::vector<double>& b, std::vector<double>& x, double tol, int maxIt,
               int& iterations) override {
        std::lock_guard<std::mutex> lk(mu_);   // studies run several simulators at once: one solve per handle at a time
        iterations = 0;
        if (!ok_) return false;
        rsg_solver* h = (precond_ == kEngineChoice && A.n < 500) ? ilu_ : cpr_;
        if (A.nb != 3) {                        // compositional / thermal blocks: CPR + GMRES in FP64
            if (!gen_) {
                rsg_options o;
                rsg_default_options(&o);
                o.precision = RSG_FP64;
                o.precond = precond_ == kEngineChoice ? RSG_PREC_CPR : precond_;
                o.krylov = RSG_KRYLOV_GMRES;
                o.restart = genericRestart_;
                o.gmres_fallback = 0;
                if (rsg_create(&gen_, &o) != RSG_OK) return false;
            }
            h = gen_;
        }
        if (rsg_set_matrix(h, A.n, A.nb, A.rowPtr.data(), A.col.data(), A.val.data()) != RSG_OK) return false;
        if (rsg_setup(h, nullptr) != RSG_OK) return false;
        x.assign(size_t(A.size()), 0.0);
        double rr = 0;
        const int rc = rsg_solve(h, b.data(), x.data(), tol, maxIt, &iterations, &rr);
        rsg_stats st;
        if (rsg_get_stats(h, &st) == RSG_OK) seconds_ += 1e-3 * (st.setup_ms + st.solve_ms);
        if (rc < 0 || (rc == RSG_ENOTCONV && role_ == Role::Distributed)) return false;
        for (double v : x)
            if (!std::isfinite(v)) return false;
        return true;
    }
    double deviceSeconds() const override { return seconds_; }

private:
    rsg_solver* cpr_ = nullptr;
    rsg_solver* ilu_ = nullptr;
    rsg_solver* gen_ = nullptr;   // blocks other than 3 x 3
    int precond_;
    Role role_;
    int genericRestart_;
    bool ok_ = false;
    double seconds_ = 0;
    std::mutex mu_;
};

// ---- the API tools/lsbench.cpp:65-81 uses (ressim/blocksolve.h is not in the reference tree)
struct BlockSolverOptions {
    double tol = 1e-4;
    int maxIt = 200;
    bool wellsInPressure = true;   // accepted for source compatibility; wells are always Schur-eliminated here
    bool cpr = true;
    bool accelerator = false;
};
struct BlockSolverStats {
    double setupSec = 0, solveSec = 0;
    int iterations = 0;
    double relResidual = 0;
    bool converged = false;
    int amgLevels = 0;
};

class RsgBlockSolver {
public:
    BlockSolverStats solve(const ressim::CSR& A, int na, int nv, int nw, const double* acc, const std::vector<double>& b,
                           std::vector<double>& x, const BlockSolverOptions& o) {
        BlockSolverStats st;
        const auto t0 = std::chrono::steady_clock::now();
        int nnzb = 0;
        if (rsg_wellschur_reduce(A.n, A.rowPtr.data(), A.col.data(), A.val.data(), na, nv, nw, b.data(), &nnzb, nullptr, nullptr,
                                 nullptr, nullptr) != RSG_OK)
            return st;
        std::vector<int> rp(size_t(na) + 1), ci(static_cast<size_t>(nnzb));
        std::vector<double> sv(size_t(nnzb) * nv * nv), bc(size_t(na) * nv);
        rsg_wellschur_reduce(A.n, A.rowPtr.data(), A.col.data(), A.val.data(), na, nv, nw, b.data(), &nnzb, rp.data(), ci.data(),
                             sv.data(), bc.data());
        rsg_options opt;
        rsg_default_options(&opt);
        opt.precond = o.cpr ? RSG_PREC_CPR : RSG_PREC_BILU0;
        rsg_solver* h = nullptr;
        if (rsg_create(&h, &opt) != RSG_OK) return st;
        std::vector<double> xc(bc.size());
        double rr = 0;
        int its = 0;
        int rc = rsg_set_matrix(h, na, nv, rp.data(), ci.data(), sv.data());
        if (rc == RSG_OK) rc = rsg_setup(h, acc);
        const auto t1 = std::chrono::steady_clock::now();
        if (rc == RSG_OK) rc = rsg_solve(h, bc.data(), xc.data(), o.tol, o.maxIt, &its, &rr);
        rsg_stats s{};
        rsg_get_stats(h, &s);
        rsg_destroy(h);
        x.assign(size_t(A.n), 0.0);
        rsg_wellschur_recover(A.n, A.rowPtr.data(), A.col.data(), A.val.data(), na, nv, nw, b.data(), xc.data(), x.data());
        const auto t2 = std::chrono::steady_clock::now();
        st.setupSec = std::chrono::duration<double>(t1 - t0).count();
        st.solveSec = std::chrono::duration<double>(t2 - t1).count();
        st.iterations = its;
        st.relResidual = s.true_rel_residual >= 0 ? s.true_rel_residual : rr;
        st.converged = rc == RSG_OK;
        st.amgLevels = s.amg_levels;
        return st;
    }
};

}  // namespace rsg
