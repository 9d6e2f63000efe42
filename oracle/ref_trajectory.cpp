// Newton-trajectory harness (test infrastructure): the reference black-oil simulator on the 20x20x4 waterflood
// (oracle/ref_case.hpp), either stock or with this repository's GPU solver in the engine's own solver hooks.
//
//   ref_trajectory MODE LINEAR_SOLVER NSTEPS STEP_DAYS [qimpes]
//
// qimpes: CPR with quasi-IMPES weights (tuning.cprWeights = 0) instead of the engine's default true-IMPES weights,
// which need the accumulation blocks that the GpuBlockSolver hook does not pass on (engine/include/ressim/bsr.h:147).
//
// MODE
//   cpu      the stock run: the engine's own CPU solver (ILU(0)- or CPR-BiCGSTAB, GMRES(60) fallback)
//   gpu      rsg::RsgGpuBlockSolver (FP64) registered with ressim::setDistributedSolver: the Newton loop trusts its
//            result at the linear tolerance (engine/src/simulator.cpp:3358-3367). Its preconditioner follows the
//            engine's choice for the case (LINEAR_SOLVER 0: BILU0; 1: CPR; 2: CPR from 500 cells,
//            engine/src/simulator.cpp:224)
//   refine   the precision form registered with ressim::setGpuBlockSolver and tuning.gpu = 1: the engine wraps it in
//            its own FP64 defect correction (refineWithDevice, engine/src/simulator.cpp:3368-3378)
//
// Output (stdout), one line per accepted time step (onTimestep, engine/include/ressim/simulator.h:332):
//   ts K time T dt DT newton N linear L fopr .. fwpr .. fwir .. fopt .. fwpt .. fwit .. fpr ..
// then "run newton N linear L gpu_solves G gpu_fallbacks F dd_solves D dd_fallbacks E".
// With RESSIM_DEBUG set the engine itself prints each Newton iteration's CNV and material-balance residuals to
// stderr ("it I cnv C mb M ...", engine/src/simulator.cpp:3207-3215).
#include "ref_case.hpp"
#include "rsg_ressim_adapter.hpp"
#include "ressim/bsr.h"
#include "ressim/simulator.h"
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>

using namespace ressim;

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: ref_trajectory cpu|gpu|refine LINEAR_SOLVER NSTEPS STEP_DAYS [qimpes]\n");
        return 1;
    }
    const std::string mode = argv[1];
    const int linearSolver = std::atoi(argv[2]), nsteps = std::atoi(argv[3]);
    const double stepDays = std::atof(argv[4]);
    Case c = rsgref::waterfloodCase(nsteps, stepDays, linearSolver);
    if (argc > 5 && std::strcmp(argv[5], "qimpes") == 0) c.tuning.cprWeights = 0;

    std::unique_ptr<rsg::RsgGpuBlockSolver> dev;
    if (mode == "gpu") {
        const int prec = linearSolver == 0 ? RSG_PREC_BILU0 : linearSolver == 1 ? RSG_PREC_CPR : rsg::RsgGpuBlockSolver::kEngineChoice;
        dev.reset(new rsg::RsgGpuBlockSolver(RSG_FP64, prec));
        setDistributedSolver(dev.get());
    } else if (mode == "refine") {
        dev.reset(new rsg::RsgGpuBlockSolver(RSG_MIXED_F32, rsg::RsgGpuBlockSolver::kEngineChoice, RSG_KRYLOV_BICGSTAB,
                                             rsg::RsgGpuBlockSolver::Role::Refinement));
        setGpuBlockSolver(dev.get());
        c.tuning.gpu = 1;
    } else if (mode != "cpu") {
        std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
        return 1;
    }
    if (dev && !dev->ok()) {
        std::fprintf(stderr, "GPU solver unavailable: %s\n", rsg_last_error());
        return 3;
    }

    Simulator sim;
    int k = 0;
    sim.onTimestep = [&](const SummaryPoint& s) {
        std::printf("ts %d time %.17g dt %.17g newton %d linear %d fopr %.17g fwpr %.17g fwir %.17g fopt %.17g fwpt %.17g fwit %.17g "
                    "fpr %.17g\n", ++k, s.time, s.dt, s.newton, s.linear, s.fopr, s.fwpr, s.fwir, s.fopt, s.fwpt, s.fwit, s.fpr);
        std::fflush(stdout);
    };
    sim.setup(c);
    sim.initialize();
    while (sim.runReportStep()) {
    }
    const RunStats& st = sim.stats();
    std::printf("run newton %d linear %d gpu_solves %d gpu_fallbacks %d dd_solves %d dd_fallbacks %d\n", st.newton, st.linear,
                st.gpuSolves, st.gpuFallbacks, st.ddSolves, st.ddFallbacks);
    setDistributedSolver(nullptr);
    setGpuBlockSolver(nullptr);
    return 0;
}
