// Assembly golden capture (test infrastructure; runs only where the reference tree exists).
//
// Runs the reference black-oil simulator on the 20x20x4 waterflood (oracle/ref_case.hpp) with the engine's scalar
// Jacobian (RESSIM_SCALAR_JAC) and, at chosen calls of the double-precision solver hook (engine/src/simulator.cpp:
// 3358-3367), records the simulator's state and three assemblies at that state with a fixed time step dt:
//   full  -- Simulator::assemble (engine/src/simulator.cpp:2500-3033) as the engine runs it: cell accumulation and
//            TPFA fluxes, wells, row scaling dt / PV;
//   cell  -- the same with every well shut, so the cell rows hold the reservoir terms alone (then scaled);
//   well  -- the well terms alone, unscaled and exact: cell properties zeroed (so the reservoir terms add exact
//            zeros), old accumulations zeroed and every pore volume set to dt (row scale dt / PV = 1).
// It also records the fluid and saturation tables the cell properties are interpolated from (ressim::FluidModel /
// SatFunctions after setup, engine/include/ressim/fluid.h), the grid connections and the Jacobian pattern. The first
// capture is repeated on a perturbed state in which some cells carry free gas (state 1, x = Sg) or no oil (state 2,
// x = Rv), so that every branch of the cell evaluation is exercised.
//
// The simulator's state lives in private members; this harness reads them by compiling the reference header with
// `private` defined as `public` (no reference source is changed; access does not affect the class layout).
//
//   ref_asm_capture OUTDIR DT CALL [CALL ...]
//   ref_asm_capture --time NX NY NZ REPS     (CPU timing of the engine's own evalAll + assemble at the first Newton
//                                             state of an NX x NY x NZ waterflood, the engine's default block assembly,
//                                             OMP_NUM_THREADS threads; prints one JSON line)
//
// Output: OUTDIR/asm_CCC.bin and OUTDIR/asm_CCC_perturbed.bin, sequences of records
// {char name[32], int32 kind (0 f64, 1 i32, 2 u8), int64 count, data}.
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <utility>
#include <vector>
#include "ressim/bsr.h"
#define private public
#define protected public
#include "ressim/simulator.h"
#undef private
#undef protected
#include "ref_case.hpp"

using namespace ressim;

namespace {

struct Out {
    FILE* f = nullptr;
    void rec(const char* name, int kind, int64_t count, const void* data, size_t esz) {
        char nm[32] = {0};
        std::strncpy(nm, name, 31);
        std::fwrite(nm, 1, 32, f);
        std::fwrite(&kind, 4, 1, f);
        std::fwrite(&count, 8, 1, f);
        if (count) std::fwrite(data, esz, size_t(count), f);
    }
    void f64(const char* n, const std::vector<double>& v) { rec(n, 0, int64_t(v.size()), v.data(), 8); }
    void i32(const char* n, const std::vector<int>& v) { rec(n, 1, int64_t(v.size()), v.data(), 4); }
    void u8(const char* n, const std::vector<uint8_t>& v) { rec(n, 2, int64_t(v.size()), v.data(), 1); }
    void f64s(const char* n, double v) { f64(n, std::vector<double>{v}); }
    void i32s(const char* n, int v) { i32(n, std::vector<int>{v}); }
    void table(const std::string& n, const Table1D& t) {
        f64((n + "_x").c_str(), t.x);
        f64((n + "_y").c_str(), t.y);
        i32s((n + "_clamp").c_str(), t.clampEnds ? 1 : 0);
    }
    // a list of tables: x and y concatenated, with offsets
    void tables(const std::string& n, const std::vector<Table1D>& ts) {
        std::vector<double> x, y;
        std::vector<int> off{0}, clamp;
        for (const Table1D& t : ts) {
            x.insert(x.end(), t.x.begin(), t.x.end());
            y.insert(y.end(), t.y.begin(), t.y.end());
            off.push_back(int(x.size()));
            clamp.push_back(t.clampEnds ? 1 : 0);
        }
        f64((n + "_x").c_str(), x);
        f64((n + "_y").c_str(), y);
        i32((n + "_off").c_str(), off);
        i32((n + "_clamp").c_str(), clamp);
    }
};

Simulator* g_sim = nullptr;

bool supported(const Simulator& s) {
    bool ok = s.fluids_.size() == 1 && s.sats_.size() == 1 && s.eps_.empty() && !s.hyst_ && !s.hystWetImb_ && !s.solv_ &&
              !s.poly_ && !s.rockOn_ && !s.rockTm_ && s.thp_.empty() && s.sGam_.empty() && s.langK_.empty() && !s.gravdr_ &&
              !s.dirKr_ && s.pcScale_.empty() && s.chPcMul_.empty() && s.chWmul_.empty() && s.chGmul_.empty() &&
              s.chMisc_.empty() && s.fRs_.empty() && s.fRv_.empty() && s.rsLim_.empty() && s.pcZw_.empty() && !s.vap_ &&
              s.aquifers_.empty() && s.saltEvap_.empty() && !s.blkAsm_;
    return ok;
}

void writeState(Simulator& s, const std::string& path, double dt) {
    Out o;
    o.f = std::fopen(path.c_str(), "wb");
    if (!o.f) { std::fprintf(stderr, "cannot write %s\n", path.c_str()); std::exit(2); }
    const int na = s.grid_.numActive(), nv = s.nv_, nw = int(s.wells_.size());
    o.i32s("na", na); o.i32s("nv", nv); o.i32s("nw", nw);
    o.i32("adjStart", s.grid_.adjStart); o.i32("adjNbr", s.grid_.adjNbr); o.i32("adjConn", s.grid_.adjConn);
    std::vector<int> ca, cb;
    std::vector<double> tr, dd;
    for (const Connection& c : s.grid_.conns) { ca.push_back(c.a); cb.push_back(c.b); tr.push_back(c.trans); dd.push_back(c.dDepth); }
    o.i32("conn_a", ca); o.i32("conn_b", cb); o.f64("conn_trans", tr); o.f64("conn_dDepth", dd);
    o.f64("poreVolRef", s.grid_.poreVolRef);
    o.i32("blkStart", s.blkStart_); o.i32("blkCells", s.blkCells_); o.i32("selfPos", s.selfPos_); o.i32("adjPos", s.adjPos_);
    o.i32("J_rowPtr", s.J_.rowPtr); o.i32("J_col", s.J_.col);
    o.u8("phases", std::vector<uint8_t>{uint8_t(s.W_), uint8_t(s.O_), uint8_t(s.G_), uint8_t(s.live_), uint8_t(s.vap_)});
    o.i32("vars", std::vector<int>{s.iSw_, s.iX_, s.eq_[0], s.eq_[1], s.eq_[2]});
    o.f64s("gravity", s.U_.gravity);
    const FluidModel& F = s.fluids_[0];
    o.f64("pvtw", std::vector<double>{F.pvtw_.pref, F.pvtw_.bw, F.pvtw_.cw, F.pvtw_.visc, F.pvtw_.cv});
    o.f64("rock", std::vector<double>{F.rock_.pref, F.rock_.cr});
    o.f64("rhoSC", std::vector<double>{F.rho_.oil, F.rho_.water, F.rho_.gas});
    o.f64s("gasFactor", F.gasFactor_);
    o.u8("fluid_flags", std::vector<uint8_t>{uint8_t(F.live_), uint8_t(F.vap_)});
    o.table("rsOfP", F.rsOfP_); o.table("pbOfRs", F.pbOfRs_);
    o.f64("liveRs", F.rs_); o.f64("livePb", F.pb_); o.f64("bSat", F.bSat_); o.f64("bmuSat", F.bmuSat_);
    o.tables("uB", F.uB_); o.tables("uBMu", F.uBMu_);
    o.table("deadB", F.deadB_); o.table("deadBMu", F.deadBMu_); o.table("gasB", F.gasB_); o.table("gasBMu", F.gasBMu_);
    const SatFunctions& S = s.sats_[0];
    o.table("krw", S.krw_); o.table("krow", S.krow_); o.table("pcow", S.pcow_);
    o.table("krg", S.krg_); o.table("krog", S.krog_); o.table("pcog", S.pcog_);
    o.f64s("swco", S.swco_); o.i32s("kroModel", S.kroModel_);
    o.u8("sat_flags", std::vector<uint8_t>{uint8_t(S.water_), uint8_t(S.gas_), uint8_t(S.threePt_)});
    o.f64("p", s.p_); o.f64("sw", s.sw_); o.f64("x", s.x_); o.u8("hasGas", s.hasGas_); o.f64("accOld", s.accOld_);
    o.f64s("dt", dt);

    const std::vector<Simulator::WellRT> wsave = s.wells_;
    // full assembly at this state
    s.assemble(dt);
    o.f64("J_full", s.J_.val); o.f64("R_full", s.R_);
    s.wells_ = wsave;
    // reservoir terms alone: every well shut
    for (Simulator::WellRT& W : s.wells_) W.open = false;
    s.assemble(dt);
    o.f64("J_cell", s.J_.val); o.f64("R_cell", s.R_);
    s.wells_ = wsave;
    // well terms alone, unscaled: zero cell properties and old accumulations, pore volumes = dt
    const std::vector<Simulator::CellFlux> cfSave = s.cf_;
    const std::vector<double> accSave = s.accOld_, pvSave = s.grid_.poreVolRef;
    for (auto& c : s.cf_) c = Simulator::CellFlux{};
    std::fill(s.accOld_.begin(), s.accOld_.end(), 0.0);
    std::fill(s.grid_.poreVolRef.begin(), s.grid_.poreVolRef.end(), dt);
    s.assemble(dt);
    o.f64("J_well", s.J_.val); o.f64("R_well", s.R_);
    s.cf_ = cfSave; s.accOld_ = accSave; s.grid_.poreVolRef = pvSave;
    s.wells_ = wsave;
    std::fclose(o.f);
}

struct Timer : GpuBlockSolver {
    int reps = 5, count = 0;
    double dt = 3.7;
    const char* name() const override { return "asm-timer"; }
    bool solve(const BSR&, const std::vector<double>&, std::vector<double>& x, double, int, int& its) override {
        x.clear(); its = 0;
        if (count++ != 0) return false;
        Simulator& s = *g_sim;
        const std::vector<Simulator::WellRT> wsave = s.wells_;
        s.evalAll(false);
        s.assemble(dt);   // warm-up
        s.wells_ = wsave;
        std::vector<double> t;
        for (int r = 0; r < reps; ++r) {
            const auto t0 = std::chrono::steady_clock::now();
            s.evalAll(false);
            s.assemble(dt);
            t.push_back(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
            s.wells_ = wsave;
        }
        std::sort(t.begin(), t.end());
        const char* th = std::getenv("OMP_NUM_THREADS");
        std::printf("{\"cells\": %d, \"block_assembly\": %d, \"reps\": %d, \"median_ms\": %.4f, \"min_ms\": %.4f, \"threads\": \"%s\"}\n",
                    s.grid_.numActive(), int(s.blkAsm_), reps, 1e3 * t[t.size() / 2], 1e3 * t[0], th ? th : "default");
        std::fflush(stdout);
        std::exit(0);
    }
};

struct Hook : GpuBlockSolver {
    std::string dir;
    double dt = 1.0;
    std::set<int> calls;
    int count = 0, written = 0;
    const char* name() const override { return "asm-capture"; }
    bool solve(const BSR&, const std::vector<double>&, std::vector<double>& x, double, int, int& its) override {
        const int call = count++;
        x.clear(); its = 0;
        if (!calls.count(call)) return false;
        Simulator& s = *g_sim;
        if (!supported(s)) { std::fprintf(stderr, "case uses features outside the captured subset\n"); std::exit(3); }
        char path[512];
        std::snprintf(path, sizeof(path), "%s/asm_%03d.bin", dir.c_str(), call);
        writeState(s, path, dt);
        if (written++ == 0) {
            // perturbed state: free gas in every fifth cell, no oil in every 23rd (when the case has gas)
            const std::vector<double> p0 = s.p_, sw0 = s.sw_, x0 = s.x_;
            const std::vector<uint8_t> g0 = s.hasGas_;
            const int na = s.grid_.numActive();
            if (s.G_) {
                for (int a = 0; a < na; ++a) {
                    if (a % 5 == 1) {
                        s.hasGas_[size_t(a)] = 1;
                        s.x_[size_t(a)] = 0.02 + 0.25 * double((a * 7) % 13) / 13.0;
                        s.sw_[size_t(a)] = std::min(s.sw_[size_t(a)], 0.95 - s.x_[size_t(a)]);
                    } else if (a % 23 == 4) {
                        s.hasGas_[size_t(a)] = 2;
                        s.x_[size_t(a)] = 0.0;
                        s.sw_[size_t(a)] = 0.3 + 0.4 * double((a * 3) % 11) / 11.0;
                    }
                    s.p_[size_t(a)] *= 1.0 - 0.35 * double((a * 5) % 17) / 17.0;   // some cells well below the bubble point
                }
            }
            s.evalAll(false);
            std::snprintf(path, sizeof(path), "%s/asm_%03d_perturbed.bin", dir.c_str(), call);
            writeState(s, path, dt);
            s.p_ = p0; s.sw_ = sw0; s.x_ = x0; s.hasGas_ = g0;
            s.evalAll(false);
        }
        return false;   // the engine solves the system itself
    }
};

}  // namespace

int main(int argc, char** argv) {
    if (argc >= 6 && std::string(argv[1]) == "--time") {
        Timer tm;
        tm.reps = std::atoi(argv[5]);
        const Case c = rsgref::waterfloodCase(1, 1.0, 0, std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4]));
        setDistributedSolver(&tm);
        Simulator sim;
        g_sim = &sim;
        sim.setup(c);
        sim.initialize();
        while (sim.runReportStep()) {}
        std::fprintf(stderr, "no Newton system reached the solver hook\n");
        return 5;
    }
    if (argc < 4) {
        std::fprintf(stderr, "usage: ref_asm_capture OUTDIR DT CALL [CALL ...]\n");
        return 1;
    }
    setenv("RESSIM_SCALAR_JAC", "1", 1);
    Hook hook;
    hook.dir = argv[1];
    hook.dt = std::atof(argv[2]);
    for (int i = 3; i < argc; ++i) hook.calls.insert(std::atoi(argv[i]));
    const Case c = rsgref::waterfloodCase(6, 30.0, 0);
    setDistributedSolver(&hook);
    Simulator sim;
    g_sim = &sim;
    sim.setup(c);
    sim.initialize();
    while (sim.runReportStep()) {}
    setDistributedSolver(nullptr);
    std::printf("hook calls %d, captured %d\n", hook.count, hook.written);
    return hook.written == int(hook.calls.size()) ? 0 : 4;
}
