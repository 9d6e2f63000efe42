// Whole-run check of the device Jacobian assembly (test infrastructure; links the reference engine and librsg.so).
//
// Runs the reference black-oil simulator on the 20x20x4 waterflood (oracle/ref_case.hpp, 6 report steps of 30 days,
// the engine's scalar Jacobian) and, at every Newton iteration that reaches the engine's solver hook
// (engine/src/simulator.cpp:3358-3367), assembles the same Jacobian on the device from the simulator's state:
//   - the engine's own J and R of this iteration are kept (Simulator::assemble at the step's dt, headDt_);
//   - the engine's well terms at this state are taken from one more engine assembly with the reservoir terms
//     zeroed (cell properties and old accumulations zero, pore volumes = dt so that the row scaling is 1), so they are
//     exact;
//   - rsg_bo_assemble_host assembles from the state (p, Sw, x, cell states, old accumulations) with those terms;
//   - J and R are compared bit for bit with the engine's, which are then put back.
// The hook returns false: the engine solves every system itself, so the run is the stock one. Prints one JSON line
// with the number of iterations compared and of mismatching values.
//
// The simulator's state lives in private members; this harness reads them by compiling the reference header with
// `private` defined as `public` (no reference source is changed; access does not affect the class layout).
//
//   ref_asm_run [NSTEPS STEP_DAYS]
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
#include "rsg.h"

using namespace ressim;

namespace {

Simulator* g_sim = nullptr;

rsg_table tab(const Table1D& t) { return rsg_table{int(t.x.size()), t.x.data(), t.y.data(), t.clampEnds ? 1 : 0}; }

struct Checker : GpuBlockSolver {
    rsg_bo_assembler* asmb = nullptr;
    std::vector<int> connA;
    std::vector<double> trans, dDepth;
    std::vector<rsg_table> ub, ubmu;
    int calls = 0, compared = 0, badCalls = 0;
    long long badJ = 0, badR = 0, values = 0;
    double maxRel = 0;
    std::string error;
    const char* name() const override { return "asm-check"; }

    bool create(Simulator& s) {
        const int na = s.grid_.numActive();
        for (const Connection& c : s.grid_.conns) { connA.push_back(c.a); trans.push_back(c.trans); dDepth.push_back(c.dDepth); }
        rsg_bo_grid g{};
        g.na = na; g.nv = s.nv_; g.nconn = int(s.grid_.conns.size());
        g.adj_start = s.grid_.adjStart.data(); g.adj_nbr = s.grid_.adjNbr.data(); g.adj_conn = s.grid_.adjConn.data();
        g.conn_a = connA.data(); g.conn_trans = trans.data(); g.conn_ddepth = dDepth.data(); g.pore_vol = s.grid_.poreVolRef.data();
        g.gravity = s.U_.gravity; g.i_sw = s.iSw_; g.i_x = s.iX_;
        for (int p = 0; p < 3; ++p) g.eq[p] = s.eq_[p];
        const FluidModel& F = s.fluids_[0];
        rsg_bo_fluid f{};
        f.water = s.W_; f.oil = s.O_; f.gas = s.G_; f.live = F.live_; f.vap = F.vap_;
        const double pw[5] = {F.pvtw_.pref, F.pvtw_.bw, F.pvtw_.cw, F.pvtw_.visc, F.pvtw_.cv};
        std::copy(pw, pw + 5, f.pvtw);
        f.rock[0] = F.rock_.pref; f.rock[1] = F.rock_.cr;
        f.rho_sc[0] = F.rho_.oil; f.rho_sc[1] = F.rho_.water; f.rho_sc[2] = F.rho_.gas;
        f.gas_factor = F.gasFactor_;
        f.rs_of_p = tab(F.rsOfP_); f.pb_of_rs = tab(F.pbOfRs_); f.dead_b = tab(F.deadB_); f.dead_bmu = tab(F.deadBMu_);
        f.gas_b = tab(F.gasB_); f.gas_bmu = tab(F.gasBMu_);
        f.nsat = int(F.rs_.size()); f.sat_rs = F.rs_.data(); f.sat_b = F.bSat_.data(); f.sat_bmu = F.bmuSat_.data();
        for (const Table1D& t : F.uB_) ub.push_back(tab(t));
        for (const Table1D& t : F.uBMu_) ubmu.push_back(tab(t));
        f.under_b = ub.data(); f.under_bmu = ubmu.data();
        const SatFunctions& S = s.sats_[0];
        rsg_bo_satfun sf{};
        sf.krw = tab(S.krw_); sf.krow = tab(S.krow_); sf.pcow = tab(S.pcow_);
        sf.krg = tab(S.krg_); sf.krog = tab(S.krog_); sf.pcog = tab(S.pcog_);
        sf.swco = S.swco_; sf.kro_model = S.kroModel_; sf.water = S.water_; sf.gas = S.gas_; sf.three_point = S.threePt_;
        if (rsg_bo_create(&asmb, &g, &f, &sf, s.J_.n, int(s.wells_.size()), s.J_.rowPtr.data(), s.J_.col.data(), 0) != RSG_OK) {
            error = std::string("rsg_bo_create: ") + rsg_last_error();
            return false;
        }
        return true;
    }

    bool solve(const BSR&, const std::vector<double>&, std::vector<double>& x, double, int, int& its) override {
        x.clear(); its = 0;
        ++calls;
        if (!error.empty()) return false;
        Simulator& s = *g_sim;
        if (!asmb && !create(s)) return false;
        const double dt = s.headDt_;
        const std::vector<double> J0 = s.J_.val, R0 = s.R_;   // the engine's own assembly of this iteration
        // the engine's well terms at this state, exact: reservoir terms zeroed, row scale dt / PV = 1
        const std::vector<Simulator::WellRT> wsave = s.wells_;
        const std::vector<Simulator::CellFlux> cfSave = s.cf_;
        const std::vector<double> accSave = s.accOld_, pvSave = s.grid_.poreVolRef;
        for (auto& c : s.cf_) c = Simulator::CellFlux{};
        std::fill(s.accOld_.begin(), s.accOld_.end(), 0.0);
        std::fill(s.grid_.poreVolRef.begin(), s.grid_.poreVolRef.end(), dt);
        s.assemble(dt);
        std::vector<long long> ap;
        std::vector<double> av, rv;
        std::vector<int> rp;
        for (size_t k = 0; k < s.J_.val.size(); ++k)
            if (s.J_.val[k] != 0.0) { ap.push_back((long long)k); av.push_back(s.J_.val[k]); }
        for (size_t r = 0; r < s.R_.size(); ++r)
            if (s.R_[r] != 0.0) { rp.push_back(int(r)); rv.push_back(s.R_[r]); }
        s.cf_ = cfSave; s.accOld_ = accSave; s.grid_.poreVolRef = pvSave; s.wells_ = wsave;
        s.J_.val = J0; s.R_ = R0;
        // the device assembly from the state
        std::vector<double> Jd(J0.size()), Rd(R0.size());
        const int rc = rsg_bo_assemble_host(asmb, s.p_.data(), s.sw_.data(), s.x_.data(), s.hasGas_.data(), s.accOld_.data(), dt, int(ap.size()),
                                            ap.data(), av.data(), int(rp.size()), rp.data(), rv.data(), Jd.data(), Rd.data());
        if (rc != RSG_OK) { error = std::string("rsg_bo_assemble_host: ") + rsg_last_error(); return false; }
        ++compared;
        long long bj = 0, br = 0;
        for (size_t k = 0; k < J0.size(); ++k)
            if (!(Jd[k] == J0[k])) {
                ++bj;
                maxRel = std::max(maxRel, std::fabs(Jd[k] - J0[k]) / std::max(std::fabs(J0[k]), 1e-300));
            }
        for (size_t r = 0; r < R0.size(); ++r)
            if (!(Rd[r] == R0[r])) {
                ++br;
                maxRel = std::max(maxRel, std::fabs(Rd[r] - R0[r]) / std::max(std::fabs(R0[r]), 1e-300));
            }
        values += (long long)(J0.size() + R0.size());
        badJ += bj; badR += br;
        if (bj || br) ++badCalls;
        return false;   // the engine solves the system itself: the stock run
    }
};

}  // namespace

int main(int argc, char** argv) {
    const int nsteps = argc > 1 ? std::atoi(argv[1]) : 6;
    const double days = argc > 2 ? std::atof(argv[2]) : 30.0;
    setenv("RESSIM_SCALAR_JAC", "1", 1);
    Checker chk;
    const Case c = rsgref::waterfloodCase(nsteps, days, 0);
    setDistributedSolver(&chk);
    Simulator sim;
    g_sim = &sim;
    sim.setup(c);
    sim.initialize();
    int steps = 0;
    while (sim.runReportStep()) ++steps;
    setDistributedSolver(nullptr);
    const auto& st = sim.stats();
    std::printf("{\"report_steps\": %d, \"newton\": %d, \"hook_calls\": %d, \"compared\": %d, \"values\": %lld, \"mismatching_calls\": %d, "
                "\"mismatching_J\": %lld, \"mismatching_R\": %lld, \"max_rel_diff\": %.3e, \"error\": \"%s\"}\n",
                steps, st.newton, chk.calls, chk.compared, chk.values, chk.badCalls, chk.badJ, chk.badR, chk.maxRel, chk.error.c_str());
    if (chk.asmb) rsg_bo_destroy(chk.asmb);
    return chk.error.empty() && chk.compared > 0 && chk.badCalls == 0 ? 0 : 1;
}
