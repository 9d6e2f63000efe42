// Whole-run check of the block-size-generic path inside the reference's compositional and thermal simulators (test
// infrastructure; the reference engine is compiled from its staged sources by oracle/Makefile.ref).
//
// Runs an example deck with the compositional simulator (comp::runDeckModel) or the thermal one
// (thermal::runDeckModel) either stock ("cpu": the engine's own BlockCPR + GMRES) or with this repository's GPU solver
// registered in the engine's distributed-solver hook ("gpu": rsg::RsgGpuBlockSolver of include/rsg_ressim_adapter.hpp,
// which the compositional (engine/src/compsim.cpp:1443-1449) and thermal (engine/src/thermsim.cpp:1818-1828) Newton
// loops call with every system before their CPU path), and prints one line per report step and the run's Newton and
// linear iteration counts and hook statistics.
//
//   ref_run_nb comp|thermal DECK REPORT_STEPS cpu|gpu
#include "rsg_ressim_adapter.hpp"
#include "ressim/bsr.h"
#include "ressim/comp_deck.h"
#include "ressim/therm_deck.h"
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>
#include <vector>

using namespace ressim;

namespace {
// counts the hook's calls and how many returned a solution
struct Counting : GpuBlockSolver {
    GpuBlockSolver* inner;
    int calls = 0, solved = 0;
    explicit Counting(GpuBlockSolver* s) : inner(s) {}
    const char* name() const override { return inner->name(); }
    bool solve(const BSR& A, const std::vector<double>& b, std::vector<double>& x, double tol, int maxIt, int& its) override {
        ++calls;
        const bool ok = inner->solve(A, b, x, tol, maxIt, its);
        solved += ok ? 1 : 0;
        return ok;
    }
    double deviceSeconds() const override { return inner->deviceSeconds(); }
};
}  // namespace

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: ref_run_nb comp|thermal DECK REPORT_STEPS cpu|gpu\n");
        return 1;
    }
    const std::string kind = argv[1], deckPath = argv[2], mode = argv[4];
    const int steps = std::atoi(argv[3]);
    // the thermal simulator solves with GMRES(80), the compositional one with GMRES(60)
    std::unique_ptr<rsg::RsgGpuBlockSolver> gpu;
    std::unique_ptr<Counting> hook;
    if (mode == "gpu") {
        gpu.reset(new rsg::RsgGpuBlockSolver(RSG_FP64, rsg::RsgGpuBlockSolver::kEngineChoice, RSG_KRYLOV_BICGSTAB,
                                             rsg::RsgGpuBlockSolver::Role::Distributed, kind == "thermal" ? 80 : 60));
        if (!gpu->ok()) { std::fprintf(stderr, "rsg: %s\n", rsg_last_error()); return 2; }
        hook.reset(new Counting(gpu.get()));
        setDistributedSolver(hook.get());
    }
    std::string err;
    bool ok = false;
    if (kind == "comp") {
        comp::DeckModel m;
        if (!comp::deckModelFromFile(deckPath, m, &err)) { std::fprintf(stderr, "deck: %s\n", err.c_str()); return 2; }
        std::vector<comp::CompSummary> out;
        comp::CompStats st;
        ok = comp::runDeckModel(m, out, {}, &err, steps, &st);
        for (const auto& s : out)
            std::printf("ts time %.17g fopt %.17g fgpt %.17g fwpt %.17g fpr %.17g foip %.17g end\n", s.time, s.fopt, s.fgpt, s.fwpt, s.fpr,
                        s.foip);
        std::printf("run steps %d newton %d linear %d cuts %d", st.steps, st.newton, st.linear, st.cuts);
    } else {
        thermal::DeckModel m;
        if (!thermal::deckModelFromFile(deckPath, m, &err)) { std::fprintf(stderr, "deck: %s\n", err.c_str()); return 2; }
        std::vector<thermal::Summary> out;
        thermal::Stats st;
        ok = thermal::runDeckModel(m, out, {}, &err, steps, &st);
        for (const auto& s : out)
            std::printf("ts time %.17g fopt %.17g fwpt %.17g fgpt %.17g fpr %.17g favgT %.17g end\n", s.time, s.fopt, s.fwpt, s.fgpt, s.fpr,
                        s.favgT);
        std::printf("run steps %d newton %d linear %d cuts %d", st.steps, st.newton, st.linear, st.cuts);
    }
    std::printf(" hook_calls %d hook_solved %d end\n", hook ? hook->calls : 0, hook ? hook->solved : 0);
    setDistributedSolver(nullptr);
    if (!ok) { std::fprintf(stderr, "run: %s\n", err.c_str()); return 3; }
    return 0;
}
