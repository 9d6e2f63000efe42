// Golden-system capture harness (test infrastructure; runs only where the reference tree exists).
//
// Builds the 20x20x4 three-phase waterflood from the reference's own input generators (oracle/ref_case.hpp),
// runs the reference black-oil simulator, and records every
// Schur-reduced Newton system (S, b) that the Newton loop hands to the double-precision solver
// hook (engine/src/simulator.cpp:3358-3367, hook declared at engine/include/ressim/bsr.h:153-157).
// The hook returns false, so the engine falls back to its own CPU solver and the run is the
// stock reference run. The first full Jacobian is also written by the engine's own RESSIM_DUMP
// (engine/src/simulator.cpp:3252-3263) when requested.
//
//   ref_capture OUTDIR LINEAR_SOLVER NSTEPS STEP_DAYS [NX NY NZ SIGMA SEED]
//
// Output: OUTDIR/sys_NNN.bin (format below), OUTDIR/trajectory.txt (one line per report step).
// System file format (little endian): int32 magic 0x42475352 ("RSGB"), int32 version 1, int32 n,
// int32 nb, int32 nnzb, int32 maxIt, float64 tol, int32 rowPtr[n+1], int32 col[nnzb],
// float64 val[nnzb*nb*nb], float64 b[n*nb].
#include "ref_case.hpp"
#include "ressim/bsr.h"
#include "ressim/simulator.h"
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

using namespace ressim;

namespace {
struct Capture : GpuBlockSolver {
    std::string dir;
    int count = 0;
    const char* name() const override { return "capture"; }
    bool solve(const BSR& A, const std::vector<double>& b, std::vector<double>& x, double tol, int maxIt, int& its) override {
        char path[512];
        std::snprintf(path, sizeof(path), "%s/sys_%03d.bin", dir.c_str(), count++);
        if (FILE* f = std::fopen(path, "wb")) {
            const int hdr[6] = {0x42475352, 1, A.n, A.nb, A.nnzb(), maxIt};
            std::fwrite(hdr, 4, 6, f);
            std::fwrite(&tol, 8, 1, f);
            std::fwrite(A.rowPtr.data(), 4, size_t(A.n) + 1, f);
            std::fwrite(A.col.data(), 4, size_t(A.nnzb()), f);
            std::fwrite(A.val.data(), 8, A.val.size(), f);
            std::fwrite(b.data(), 8, b.size(), f);
            std::fclose(f);
        }
        x.clear(); its = 0;
        return false;   // the engine solves the system itself (stock CPU path)
    }
};
}  // namespace

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: ref_capture OUTDIR LINEAR_SOLVER NSTEPS STEP_DAYS [NX NY NZ SIGMA SEED]\n");
        return 1;
    }
    const std::string dir = argv[1];
    const int linearSolver = std::atoi(argv[2]), nsteps = std::atoi(argv[3]);
    const double stepDays = std::atof(argv[4]);
    const int nx = argc > 5 ? std::atoi(argv[5]) : 20, ny = argc > 6 ? std::atoi(argv[6]) : 20, nz = argc > 7 ? std::atoi(argv[7]) : 4;
    const double sigma = argc > 8 ? std::atof(argv[8]) : 1.0;
    const unsigned seed = argc > 9 ? unsigned(std::atoi(argv[9])) : 0u;

    const Case c = rsgref::waterfloodCase(nsteps, stepDays, linearSolver, nx, ny, nz, sigma, seed);

    Capture cap; cap.dir = dir;
    setDistributedSolver(&cap);
    Simulator sim;
    sim.setup(c);
    sim.initialize();
    std::string traj;
    int step = 0;
    while (sim.runReportStep()) {
        const auto& s = sim.summary().back();
        const auto& st = sim.stats();
        char line[256];
        std::snprintf(line, sizeof(line), "step %d newton %d linear %d fopt %.9g fpr %.9g systems %d\n", ++step, st.newton, st.linear, s.fopt, s.fpr, cap.count);
        traj += line;
    }
    setDistributedSolver(nullptr);
    if (FILE* f = std::fopen((dir + "/trajectory.txt").c_str(), "w")) { std::fputs(traj.c_str(), f); std::fclose(f); }
    std::printf("%s", traj.c_str());
    std::printf("captured %d systems\n", cap.count);
    return 0;
}
