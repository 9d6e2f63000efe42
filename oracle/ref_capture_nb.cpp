// Golden-system capture of the engine's other callers of the block solver (test infrastructure; runs only where the
// reference tree exists).
//
// Runs one of the reference's example decks with its compositional simulator (comp::deckModelFromFile /
// comp::runDeckModel; engine/src/compsim.cpp:1443-1449 hands every Newton system to the distributed-solver hook with
// tol = linTol, maxIt = 300) or its thermal simulator (thermal::deckModelFromFile / thermal::runDeckModel;
// engine/src/thermsim.cpp:1818-1823, tol = 1e-6, maxIt = 400), and records the first MAXSYS systems in the format of
// ref_capture (blocks nb = the simulator's unknowns per cell). The hook returns false, so the engine solves every
// system itself and the run is the stock run.
//
//   ref_capture_nb comp|thermal DECK OUTDIR MAXSYS [REPORT_STEPS]
#include "ressim/bsr.h"
#include "ressim/comp_deck.h"
#include "ressim/therm_deck.h"
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

using namespace ressim;

namespace {
struct Capture : GpuBlockSolver {
    std::string dir;
    int count = 0, maxSys = 0;
    const char* name() const override { return "capture"; }
    bool solve(const BSR& A, const std::vector<double>& b, std::vector<double>& x, double tol, int maxIt, int& its) override {
        if (count < maxSys) {
            char path[512];
            std::snprintf(path, sizeof(path), "%s/sys_%03d.bin", dir.c_str(), count);
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
        }
        ++count;
        x.clear();
        its = 0;
        return false;
    }
};
}  // namespace

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: ref_capture_nb comp|thermal DECK OUTDIR MAXSYS [REPORT_STEPS]\n");
        return 1;
    }
    const std::string kind = argv[1], deckPath = argv[2];
    Capture cap;
    cap.dir = argv[3];
    cap.maxSys = std::atoi(argv[4]);
    const int steps = argc > 5 ? std::atoi(argv[5]) : 1;
    setDistributedSolver(&cap);
    std::string err;
    bool ok = false;
    if (kind == "comp") {
        comp::DeckModel m;
        if (!comp::deckModelFromFile(deckPath, m, &err)) { std::fprintf(stderr, "deck: %s\n", err.c_str()); return 2; }
        std::vector<comp::CompSummary> out;
        ok = comp::runDeckModel(m, out, {}, &err, steps);
    } else {
        thermal::DeckModel m;
        if (!thermal::deckModelFromFile(deckPath, m, &err)) { std::fprintf(stderr, "deck: %s\n", err.c_str()); return 2; }
        std::vector<thermal::Summary> out;
        ok = thermal::runDeckModel(m, out, {}, &err, steps);
    }
    setDistributedSolver(nullptr);
    std::printf("run %s, captured %d of %d systems\n", ok ? "ok" : err.c_str(), std::min(cap.count, cap.maxSys), cap.count);
    return cap.count > 0 ? 0 : 3;
}
