// Black-oil Newton Jacobian assembly on the device: the reservoir part of the engine's fully implicit system.
//
// Replaces, for the standard three-phase black-oil model, Simulator::evalAll / evalCell (engine/src/simulator.cpp:
// 2133-2276, 2429-2459), the cell loop of Simulator::assemble (:2500-2686) and its row scaling (:3010-3032). The
// model: water (PVTW formulas), live oil (saturated nodes with undersaturated ratio tables, pressure and Rs derivatives
// by central differences as ressim::FluidModel::liveOilAD, engine/src/fluid.cpp:257-280), dry gas (tables), rock
// compressibility, SWOF / SGOF tables without end-point scaling and the ECLIPSE default three-phase oil relative
// permeability (engine/src/fluid.cpp:445-460), TPFA fluxes upwinded per phase on the potential with gravity, the
// dissolved gas carried by the oil flux. Cell states follow the engine's variable switching: 0 = no free gas (x = Rs),
// 1 = oil + gas (x = Sg), 2 = no oil (x = Rv).
//
// The wells stay with the caller (the engine's well model runs on its host, engine/src/simulator.cpp:2692-2954): their
// terms come in as addends to entries of J and R, applied after the reservoir terms and before the row scaling, in
// the caller's order -- the order in which the engine adds them. Every addition, product and quotient is the
// reference's, in the reference's order (this file is compiled without contraction into fused multiply-adds), so the
// Jacobian and residual are the engine's bit for bit.
//
// Three kernels per assembly (four with well terms): k_bo_props evaluates every cell's properties with their
// derivatives, one thread per cell (13 dual numbers, stored component-major so that neighbouring threads read
// neighbouring words); k_bo_conn forms each connection's phase fluxes once, one thread per connection; k_bo_cells forms
// the accumulation of a cell's three rows, adds its connections' fluxes (negated, with the two cells' derivative slots
// exchanged, on a connection's second cell) and writes the rows once; k_bo_addends finishes the few rows that take
// well terms.
#include "rsg.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

namespace rsg {
void set_last_error(const std::string& msg);
}

namespace {

constexpr int kThreads = 128;
constexpr int kRec = 13;               // dual numbers per cell record: P[3], mob[3], rho[3], mobRs, acc[3]
constexpr int kRecWords = kRec * 4;    // value + 3 derivatives each
constexpr int PW = 0, PO = 1, PG = 2;

// ---------------------------------------------------------------------------------------------------------------
// Dual numbers with three derivatives (the cell's own unknowns). The rounding of every rule is that of the engine's
// forward-mode type (engine/include/ressim/ad.h): a product's derivative is d_a b + a d_b, a quotient's is
// (d_a b - a d_b) inv inv with the value a inv, and division by a constant multiplies by its reciprocal.
struct D3 {
    double v, d0, d1, d2;
};

__device__ __forceinline__ D3 dconst(double v) { return D3{v, 0.0, 0.0, 0.0}; }
__device__ __forceinline__ D3 dvar(double v, int slot) {
    return D3{v, slot == 0 ? 1.0 : 0.0, slot == 1 ? 1.0 : 0.0, slot == 2 ? 1.0 : 0.0};
}
__device__ __forceinline__ D3 add(D3 a, D3 b) { return D3{a.v + b.v, a.d0 + b.d0, a.d1 + b.d1, a.d2 + b.d2}; }
__device__ __forceinline__ D3 sub(D3 a, D3 b) { return D3{a.v - b.v, a.d0 - b.d0, a.d1 - b.d1, a.d2 - b.d2}; }
__device__ __forceinline__ D3 addc(D3 a, double c) { a.v = a.v + c; return a; }      // a + c and c + a
__device__ __forceinline__ D3 subc(D3 a, double c) { a.v = a.v - c; return a; }      // a - c
__device__ __forceinline__ D3 csub(double c, D3 a) { return D3{-a.v + c, -a.d0, -a.d1, -a.d2}; }   // c - a
__device__ __forceinline__ D3 mulc(D3 a, double c) { return D3{a.v * c, a.d0 * c, a.d1 * c, a.d2 * c}; }
__device__ __forceinline__ D3 mul(D3 a, D3 b) {
    return D3{a.v * b.v, a.d0 * b.v + a.v * b.d0, a.d1 * b.v + a.v * b.d1, a.d2 * b.v + a.v * b.d2};
}
__device__ __forceinline__ D3 dvd(D3 a, D3 b) {
    const double inv = 1.0 / b.v;
    return D3{a.v * inv, (a.d0 * b.v - a.v * b.d0) * inv * inv, (a.d1 * b.v - a.v * b.d1) * inv * inv,
              (a.d2 * b.v - a.v * b.d2) * inv * inv};
}
__device__ __forceinline__ D3 chain(D3 x, double f, double dfdx) { return D3{f, dfdx * x.d0, dfdx * x.d1, dfdx * x.d2}; }
__device__ __forceinline__ D3 chain2(D3 x, D3 y, double f, double fx, double fy) {
    return D3{f, fx * x.d0 + fy * y.d0, fx * x.d1 + fy * y.d1, fx * x.d2 + fy * y.d2};
}

// ---------------------------------------------------------------------------------------------------------------
// Tables (ressim::Table1D, engine/include/ressim/fluid.h:10-17): piecewise linear, extrapolated linearly beyond the
// ends unless clamped, the segment found as upper_bound - 1 within [0, n - 2]. The slope of every segment,
// (y[i+1] - y[i]) / (x[i+1] - x[i]) (0 for a zero-width segment), is computed once on the host -- the same IEEE
// operations the engine performs at each evaluation, so the same value -- and the evaluation is y[i] + s (xv - x[i]).
struct Tab {
    int x, y, s, k, n, clamp;   // offsets of x, y, the slopes and the order keys in the table buffer, length, clamp flag
};

// Order key of a double: a 64-bit integer that compares as the IEEE value does (-0 taken as +0; no NaN in the
// tables), so that table searches run on the integer pipe and leave the FP64 pipe, the binding unit of the assembly,
// to the arithmetic. The keys of the tables' abscissae are formed on the host.
__device__ __forceinline__ long long okey(double v) {
    long long b = __double_as_longlong(v);
    b = b == (long long)0x8000000000000000ULL ? 0 : b;
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

// upper_bound - 1 of xk among the n keys K, within [0, n - 2], with the engine's guards for the first and last segment
__device__ __forceinline__ int seg_of(const long long* __restrict__ K, int n, long long xk) {
    if (xk <= K[1]) return 0;
    if (xk >= K[n - 2]) return n - 2;
    int lo = 0, cnt = n;
    while (cnt > 0) {
        const int step = cnt >> 1;
        if (!(xk < K[lo + step])) { lo += step + 1; cnt -= step + 1; }
        else cnt = step;
    }
    return min(max(lo - 1, 0), n - 2);
}

__device__ double tab_eval(const double* __restrict__ T, Tab t, double xv, double& s) {
    const int n = t.n;
    if (n == 0) { s = 0.0; return 0.0; }
    const double* x = T + t.x;
    const double* y = T + t.y;
    if (n == 1) { s = 0.0; return y[0]; }
    const long long* K = reinterpret_cast<const long long*>(T + t.k);
    const long long xk = okey(xv);
    if (t.clamp) {
        if (xk <= K[0]) { s = 0.0; return y[0]; }
        if (xk >= K[n - 1]) { s = 0.0; return y[n - 1]; }
    }
    const int i = seg_of(K, n, xk);
    s = T[t.s + i];
    return y[i] + s * (xv - x[i]);
}
__device__ __forceinline__ D3 tab_ad(const double* __restrict__ T, Tab t, D3 xv) {
    double s;
    const double f = tab_eval(T, t, xv.v, s);
    return chain(xv, f, s);
}

struct Model {
    // phases and unknowns
    int water, oil, gas, live;
    int iSw, iX, eq[3];
    double gravity;
    // water, rock, densities
    double pw_ref, pw_bw, pw_cw, pw_visc, pw_cv;
    double rock_ref, rock_cr;
    double rho_oil, rho_water, rho_gas, gas_factor;
    // constants of the engine's expressions, formed once with the same IEEE operations: 1 / Bw, 1 / (Bw mu_w),
    // cw - cv, rho_gas * gasFactor
    double inv_bw, inv_bwvisc, pw_cwv, rho_gfac;
    // tables
    Tab rsOfP, pbOfRs, deadB, deadBMu, gasB, gasBMu;
    Tab krw, krow, pcow, krg, krog, pcog;
    double swco;
    int sat_water, sat_gas;
    // live oil: nsat saturated nodes (Rs, 1/Bo, 1/(Bo mu)) at rs, bsat, bmusat; under tables at utab[2 k] (1/Bo
    // ratio) and utab[2 k + 1] (1/(Bo mu) ratio) of the descriptor array
    int nsat, rs, rsk, bsat, bmusat;   // rsk: order keys of the nodes' Rs
};

// FluidModel::liveOil (engine/src/fluid.cpp:257-271): interpolation between the saturated nodes bracketing rs of
// the undersaturated ratio at p - pb(rs). Split in two: the segment of rs (node k, pb(rs), weight w), then both
// quantities (1/Bo and 1/(Bo mu)) at one p, so that evaluations at the same rs share the segment.
struct LiveSeg {
    int k;
    double pb, w;
};

__device__ LiveSeg live_seg(const double* __restrict__ T, const Model& m, double rs) {
    const double* R = T + m.rs;
    const int k = seg_of(reinterpret_cast<const long long*>(T + m.rsk), m.nsat, okey(rs));
    double s;
    LiveSeg g;
    g.k = k;
    g.pb = tab_eval(T, m.pbOfRs, rs, s);
    g.w = (rs - R[k]) / (R[k + 1] - R[k]);
    return g;
}

__device__ __forceinline__ void live_pair(const double* __restrict__ T, const Tab* __restrict__ U, const Model& m, LiveSeg g,
                                          double p, double& b, double& bmu) {
    const double dp = p - g.pb;
    const int k = g.k;
    double s;
    const double* sb = T + m.bsat;
    const double* sm = T + m.bmusat;
    const double b0 = sb[k] * tab_eval(T, U[2 * k], dp, s);
    const double b1 = sb[k + 1] * tab_eval(T, U[2 * (k + 1)], dp, s);
    b = b0 + g.w * (b1 - b0);
    const double m0 = sm[k] * tab_eval(T, U[2 * k + 1], dp, s);
    const double m1 = sm[k + 1] * tab_eval(T, U[2 * (k + 1) + 1], dp, s);
    bmu = m0 + g.w * (m1 - m0);
}

// FluidModel::liveOilAD (engine/src/fluid.cpp:273-280) for 1/Bo and 1/(Bo mu) at once: the values and central
// differences in p (at rs's segment) and in rs (at the segments of rs +- hr)
__device__ void live_oil_ad2(const double* __restrict__ T, const Tab* __restrict__ U, const Model& m, D3 p, D3 rs, D3& bo, D3& bomu) {
    const LiveSeg g0 = live_seg(T, m, rs.v);
    const double hp = 1e-4 * fmax(1.0, fabs(p.v));
    const double hr = 1e-5 * fmax(1e-2, fabs(rs.v));
    double fb, fm, pbp, pmp, pbm, pmm, rbp, rmp, rbm, rmm;
    live_pair(T, U, m, g0, p.v, fb, fm);
    live_pair(T, U, m, g0, p.v + hp, pbp, pmp);
    live_pair(T, U, m, g0, p.v - hp, pbm, pmm);
    live_pair(T, U, m, live_seg(T, m, rs.v + hr), p.v, rbp, rmp);
    live_pair(T, U, m, live_seg(T, m, rs.v - hr), p.v, rbm, rmm);
    bo = chain2(p, rs, fb, (pbp - pbm) / (2 * hp), (rbp - rbm) / (2 * hr));
    bomu = chain2(p, rs, fm, (pmp - pmm) / (2 * hp), (rmp - rmm) / (2 * hr));
}

__device__ __forceinline__ D3 rs_sat(const double* T, const Model& m, D3 p) {   // FluidModel::rsSat (fluid.cpp:248-254)
    if (!m.live) return dconst(0.0);
    double d;
    double r = tab_eval(T, m.rsOfP, p.v, d);
    if (r < 0) { r = 0; d = 0; }
    return chain(p, r, d);
}

// SatFunctions::kro without end-point scaling (engine/src/fluid.cpp:445-460), ECLIPSE default model
__device__ D3 kro3(const double* T, const Model& m, D3 sw, D3 sg) {
    if (m.sat_water && !m.sat_gas) return tab_ad(T, m.krow, sw);
    if (!m.sat_water && m.sat_gas) return tab_ad(T, m.krog, sg);
    if (!m.sat_water && !m.sat_gas) return dconst(1.0);
    D3 dw = subc(sw, m.swco);
    if (dw.v < 0) dw = dconst(0.0);
    const D3 swEff = add(sw, sg);
    const D3 sgEff = subc(add(sw, sg), m.swco);
    const D3 den = add(sg, dw);
    if (den.v < 1e-9) return tab_ad(T, m.krow, swEff);
    return dvd(add(mul(sg, tab_ad(T, m.krog, sgEff)), mul(dw, tab_ad(T, m.krow, swEff))), den);
}

// ---------------------------------------------------------------------------------------------------------------
// Cell properties (Simulator::evalCell, engine/src/simulator.cpp:2133-2276, for this model): record layout
// P[0..2] mob[3..5] rho[6..8] mobRs[9] acc[10..12], word j of field f of cell c at rec[(4 f + j) na + c].
__global__ void __launch_bounds__(kThreads) k_bo_props(int na, Model m, const double* __restrict__ T, const Tab* __restrict__ U,
                                                       const double* __restrict__ pv0, const double* __restrict__ pres,
                                                       const double* __restrict__ swv, const double* __restrict__ xv,
                                                       const unsigned char* __restrict__ state, double* __restrict__ rec) {
    const int c = blockIdx.x * kThreads + threadIdx.x;
    if (c >= na) return;
    const D3 P = dvar(__ldg(pres + c), 0);
    D3 Sw = dconst(m.water && !m.oil ? 1.0 : 0.0), Sg = dconst(0.0), rs = dconst(0.0);
    if (m.iSw >= 0) Sw = dvar(__ldg(swv + c), m.iSw);
    const int st = __ldg(state + c);
    if (m.gas) {
        if (st == 1) {
            Sg = dvar(__ldg(xv + c), m.iX);
            if (m.live) rs = rs_sat(T, m, P);
        } else if (st == 0) {
            rs = dvar(__ldg(xv + c), m.iX);
        } else {
            Sg = csub(1.0, Sw);
            if (m.live) rs = rs_sat(T, m, P);
        }
    }
    const D3 So = (m.oil && !(m.gas && st == 2)) ? sub(csub(1.0, Sw), Sg) : dconst(0.0);
    // pore volume: FluidModel::pvMult (fluid.cpp:199-202) times the reference pore volume
    D3 pv;
    {
        const D3 X = mulc(subc(P, m.rock_ref), m.rock_cr);
        pv = mulc(add(addc(X, 1.0), mulc(mul(X, X), 0.5)), __ldg(pv0 + c));
    }
    D3 Pp[3] = {dconst(0.0), dconst(0.0), dconst(0.0)}, mob[3] = {dconst(0.0), dconst(0.0), dconst(0.0)};
    D3 rho[3] = {dconst(0.0), dconst(0.0), dconst(0.0)}, acc[3] = {dconst(0.0), dconst(0.0), dconst(0.0)};
    D3 mobRs = dconst(0.0), bo = dconst(0.0);
    if (m.water) {
        Pp[PW] = m.oil ? sub(P, mulc(mulc(tab_ad(T, m.pcow, Sw), 1.0), 1.0)) : P;
        // FluidModel::bw / bwMu (fluid.cpp:191-198)
        const D3 X = mulc(subc(Pp[PW], m.pw_ref), m.pw_cw);
        const D3 bw = mulc(add(addc(X, 1.0), mulc(mul(X, X), 0.5)), m.inv_bw);
        const D3 Y = mulc(subc(Pp[PW], m.pw_ref), m.pw_cwv);
        const D3 bwmu = mulc(add(addc(Y, 1.0), mulc(mul(Y, Y), 0.5)), m.inv_bwvisc);
        const D3 kr = !m.oil ? dconst(1.0) : tab_ad(T, m.krw, Sw);
        mob[PW] = mul(bwmu, kr);
        rho[PW] = mulc(bw, m.rho_water);
        acc[PW] = mul(mul(pv, bw), Sw);
    }
    if (m.oil) {
        Pp[PO] = P;
        D3 bomu;
        if (m.live) live_oil_ad2(T, U, m, P, rs, bo, bomu);
        else { bo = tab_ad(T, m.deadB, P); bomu = tab_ad(T, m.deadBMu, P); }
        D3 kr = dconst(1.0);
        if (m.water || m.gas) kr = kro3(T, m, Sw, Sg);
        mob[PO] = mul(bomu, kr);
        rho[PO] = mul(bo, addc(mulc(rs, m.rho_gfac), m.rho_oil));
        acc[PO] = mul(mul(pv, bo), So);
        mobRs = mul(mob[PO], rs);
    }
    if (m.gas) {
        Pp[PG] = add(P, tab_ad(T, m.pcog, Sg));
        const D3 krg = tab_ad(T, m.krg, Sg);
        const D3 bg = tab_ad(T, m.gasB, Pp[PG]);
        mob[PG] = mul(tab_ad(T, m.gasBMu, Pp[PG]), krg);
        rho[PG] = mulc(bg, m.rho_gfac);
        acc[PG] = mul(pv, add(mul(bg, Sg), m.oil ? mul(mul(rs, bo), So) : dconst(0.0)));
    }
    const D3 f[kRec] = {Pp[0], Pp[1], Pp[2], mob[0], mob[1], mob[2], rho[0], rho[1], rho[2], mobRs, acc[0], acc[1], acc[2]};
    const size_t N = size_t(na);
#pragma unroll
    for (int k = 0; k < kRec; ++k) {
        rec[(4 * k + 0) * N + c] = f[k].v;
        rec[(4 * k + 1) * N + c] = f[k].d0;
        rec[(4 * k + 2) * N + c] = f[k].d1;
        rec[(4 * k + 3) * N + c] = f[k].d2;
    }
}

__device__ __forceinline__ D3 ld3(const double* __restrict__ rec, size_t N, int field, int c) {
    return D3{__ldg(rec + (4 * field + 0) * N + c), __ldg(rec + (4 * field + 1) * N + c), __ldg(rec + (4 * field + 2) * N + c),
              __ldg(rec + (4 * field + 3) * N + c)};
}

// ---------------------------------------------------------------------------------------------------------------
// Phase flux over a connection, in the perspective of its cell a (Simulator::assemble, engine/src/simulator.cpp:
// 2567-2620): dphi = P_a - P_b + rho g dD with rho = (rho_a + rho_b) / 2, F = mob_upstream dphi T. The dual numbers
// carry a's derivatives (fa) and b's (fb); the slots a lifted operand does not have are exact zeros, so their
// products and sums are left out (x + 0 and 0 * y change no value), and so is the gravity term of a connection
// without depth difference.
struct Dphi {
    double v, da[3], db[3];
};

__device__ __forceinline__ Dphi dphi_of(const double* __restrict__ rec, size_t N, int p, int b, const D3& PA, const D3& RA, double gd) {
    const D3 PB = ld3(rec, N, p, b);
    Dphi d{PA.v - PB.v, {PA.d0, PA.d1, PA.d2}, {-PB.d0, -PB.d1, -PB.d2}};
    if (gd != 0.0) {
        const D3 RB = ld3(rec, N, 6 + p, b);
        d.v = d.v + ((RA.v + RB.v) * 0.5) * gd;
        d.da[0] = d.da[0] + (RA.d0 * 0.5) * gd;
        d.da[1] = d.da[1] + (RA.d1 * 0.5) * gd;
        d.da[2] = d.da[2] + (RA.d2 * 0.5) * gd;
        d.db[0] = d.db[0] + (RB.d0 * 0.5) * gd;
        d.db[1] = d.db[1] + (RB.d1 * 0.5) * gd;
        d.db[2] = d.db[2] + (RB.d2 * 0.5) * gd;
    }
    return d;
}

struct Flux {
    double v, fa[3], fb[3];
};

// F = mob dphi T with the upstream cell's mobility `mo` (its own derivatives in the first or the second slots)
__device__ __forceinline__ Flux flux_of(const D3& mo, bool upA, const Dphi& d, double tr) {
    Flux F;
    const double mu[3] = {mo.d0, mo.d1, mo.d2};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        F.fa[i] = (upA ? mu[i] * d.v + mo.v * d.da[i] : mo.v * d.da[i]) * tr;
        F.fb[i] = (upA ? mo.v * d.db[i] : mu[i] * d.v + mo.v * d.db[i]) * tr;
    }
    F.v = (mo.v * d.v) * tr;
    return F;
}

constexpr int kFluxKinds = 4;                 // per connection: water, oil, dissolved gas (with the oil), gas
constexpr int kFluxWords = kFluxKinds * 7;    // value, the first cell's 3 derivatives, the second's 3

// The fluxes of every connection, once, in the perspective of its first cell a (conn_a). Seen from its second cell b
// the engine's flux is the exact negative with the slots exchanged -- -(x) + -(y) = -(x + y) and (-x) y = -(x y) in
// IEEE arithmetic, and b takes the same cell as upstream -- except where the potential difference is exactly zero
// (then each side takes itself as upstream) or not a number: those phases are flagged and their two cells form them
// themselves. Record layout: word j of term k of connection c at flux[(7 k + j) nconn + c].
__global__ void __launch_bounds__(kThreads) k_bo_conn(int nconn, int na, Model m, const double* __restrict__ rec,
                                                      const int* __restrict__ connA, const int* __restrict__ connB,
                                                      const double* __restrict__ trans, const double* __restrict__ dDepth,
                                                      double* __restrict__ flux, unsigned char* __restrict__ flag) {
    const int c = blockIdx.x * kThreads + threadIdx.x;
    if (c >= nconn) return;
    const size_t N = size_t(na), NC = size_t(nconn);
    const int a = __ldg(connA + c), b = __ldg(connB + c);
    const double tr = __ldg(trans + c);
    const double gd = m.gravity * __ldg(dDepth + c);
    unsigned fl = 0;
    auto put = [&](int k, const Flux& F) {
        flux[(7 * k + 0) * NC + c] = F.v;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            flux[(7 * k + 1 + i) * NC + c] = F.fa[i];
            flux[(7 * k + 4 + i) * NC + c] = F.fb[i];
        }
    };
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        const Dphi d = dphi_of(rec, N, p, b, ld3(rec, N, p, a), ld3(rec, N, 6 + p, a), gd);
        if (!(d.v > 0 || d.v < 0)) { fl |= 1u << p; continue; }
        const bool upA = d.v >= 0;
        const int up = upA ? a : b;
        put(p == PG ? 3 : p, flux_of(ld3(rec, N, 3 + p, up), upA, d, tr));
        if (p == PO) put(2, flux_of(ld3(rec, N, 9, up), upA, d, tr));
    }
    flag[c] = static_cast<unsigned char>(fl);
}

// Accumulation and TPFA flux terms of cell a's rows (Simulator::assemble cell loop, engine/src/simulator.cpp:2511-2686,
// without the features this model leaves out), then the row scaling dt / PV (:3010-3032). The flux terms come from
// k_bo_conn (negated and exchanged for the connections whose second cell a is), except for flagged phases, which
// the cell forms itself. Rows that take well terms (cells listed in acell) are written unscaled and finished by
// k_bo_addends.
__global__ void __launch_bounds__(kThreads) k_bo_cells(int na, int nv, int nconn, Model m, double dt, const double* __restrict__ rec,
                                                       const double* __restrict__ flux, const unsigned char* __restrict__ flag,
                                                       const double* __restrict__ accOld, const double* __restrict__ pv0,
                                                       const int* __restrict__ adjStart, const int* __restrict__ adjNbr,
                                                       const int* __restrict__ adjConn, const int* __restrict__ adjPos,
                                                       const int* __restrict__ connA, const double* __restrict__ trans,
                                                       const double* __restrict__ dDepth, const int* __restrict__ blkStart,
                                                       const int* __restrict__ selfPos, const int* __restrict__ Jrow,
                                                       const int* __restrict__ acell, int nacell, double* __restrict__ J,
                                                       double* __restrict__ R) {
    const int a = blockIdx.x * kThreads + threadIdx.x;
    if (a >= na) return;
    const size_t N = size_t(na), NC = size_t(nconn);
    const double invDt = 1.0 / dt;
    // Accumulators per phase balance (the equation row of phase p is m.eq[p]): the cell's own block and residual.
    // The model has all three phases and dissolved gas (checked at creation), so the order of the terms is fixed: a
    // balance's first term is assigned rather than added to zero (the same value).
    double sj[3][3], sr[3];
    // does the cell take well terms (then its rows are finished by k_bo_addends)?
    bool finish = false;
    {
        int lo = 0, hi = nacell;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            const int v = __ldg(acell + mid);
            if (v < a) lo = mid + 1;
            else hi = mid;
        }
        finish = lo < nacell && __ldg(acell + lo) == a;
    }
    const double s = finish ? 1.0 : dt / __ldg(pv0 + a);
    // accumulation (acc - accOld) / dt
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        D3 acc = ld3(rec, N, 10 + p, a);
        acc.v = acc.v - __ldg(accOld + size_t(a) * 3 + p);
        sr[p] = acc.v * invDt;
        sj[p][0] = acc.d0 * invDt;
        sj[p][1] = acc.d1 * invDt;
        sj[p][2] = acc.d2 * invDt;
    }
    const int r0 = a * nv;
    int rowp[3];
#pragma unroll
    for (int p = 0; p < 3; ++p) rowp[p] = __ldg(Jrow + r0 + m.eq[p]);
    const int nblk = __ldg(blkStart + a + 1) - __ldg(blkStart + a);
    const int e1 = __ldg(adjStart + a + 1);
    for (int q = __ldg(adjStart + a); q < e1; ++q) {
        const int cn = __ldg(adjConn + q);
        const bool first = __ldg(connA + cn) == a;            // the connection's first cell: its fluxes as stored
        const unsigned fl = __ldg(flag + cn);
        double nbk[3][3];   // the neighbour's block of this connection
        // add one flux term to balance `bal`; `lead`: the connection's first term of that balance in nbk
        auto add = [&](int bal, bool lead, double v, const double* own, const double* nb) {
            sr[bal] += v;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                sj[bal][k] += own[k];
                nbk[bal][k] = lead ? nb[k] : nbk[bal][k] + nb[k];
            }
        };
        auto stored = [&](int kind, int bal, bool lead) {
            double w[7];
#pragma unroll
            for (int j = 0; j < 7; ++j) w[j] = __ldg(flux + (7 * kind + j) * NC + cn);
            if (first) add(bal, lead, w[0], w + 1, w + 4);
            else {
                const double own[3] = {-w[4], -w[5], -w[6]}, nb[3] = {-w[1], -w[2], -w[3]};
                add(bal, lead, -w[0], own, nb);
            }
        };
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            if (!((fl >> p) & 1u)) {
                stored(p == PG ? 3 : p, p, p != PG);
                if (p == PO) stored(2, PG, true);
                continue;
            }
            // a zero (or undefined) potential difference: the cell forms the phase's terms itself
            const int b = __ldg(adjNbr + q);
            const double dD = first ? __ldg(dDepth + cn) : -__ldg(dDepth + cn);
            const double tr = __ldg(trans + cn);
            const Dphi d = dphi_of(rec, N, p, b, ld3(rec, N, p, a), ld3(rec, N, 6 + p, a), m.gravity * dD);
            const bool upA = d.v >= 0;
            const int up = upA ? a : b;
            const Flux F = flux_of(ld3(rec, N, 3 + p, up), upA, d, tr);
            add(p, p != PG, F.v, F.fa, F.fb);
            if (p == PO) {
                const Flux Fd = flux_of(ld3(rec, N, 9, up), upA, d, tr);
                add(PG, true, Fd.v, Fd.fa, Fd.fb);
            }
        }
        const int pos = __ldg(adjPos + q);
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            double* row = J + rowp[p] + pos * 3;
            row[0] = nbk[p][0] * s;
            row[1] = nbk[p][1] * s;
            row[2] = nbk[p][2] * s;
        }
    }
    const int sp = __ldg(selfPos + a);
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        const int e = m.eq[p];
        double* row = J + rowp[p];
        row[sp * 3 + 0] = sj[p][0] * s;
        row[sp * 3 + 1] = sj[p][1] * s;
        row[sp * 3 + 2] = sj[p][2] * s;
        const int re = __ldg(Jrow + r0 + e + 1);
        for (int k = rowp[p] + nblk * 3; k < re; ++k) J[k] = 0.0;   // well columns: the caller's terms only
        R[r0 + e] = sr[p] * s;
    }
}

// Rows that take well terms: the caller's addends in their order, then (cell rows) the row scaling dt / PV. Entry i of
// the list is a cell (0 <= id < na: its nv rows) or a well row (id = na + w, row na nv + w, zeroed first, unscaled).
__global__ void k_bo_addends(int na, int nv, int nrows, double dt, const int* __restrict__ acell, int nacell,
                             const int* __restrict__ aBeg, const long long* __restrict__ addPos, const double* __restrict__ addVal,
                             const int* __restrict__ rBeg, const int* __restrict__ raddPos, const double* __restrict__ raddVal,
                             const double* __restrict__ pv0, const int* __restrict__ Jrow, double* __restrict__ J,
                             double* __restrict__ R) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nacell) return;
    const int id = acell[i];
    const int r0 = id < na ? id * nv : na * nv + (id - na);
    const int r1 = id < na ? r0 + nv : r0 + 1;
    if (r1 > nrows) return;
    if (id >= na) {
        for (int k = Jrow[r0]; k < Jrow[r1]; ++k) J[k] = 0.0;
        R[r0] = 0.0;
    }
    for (int k = aBeg[i]; k < aBeg[i + 1]; ++k) J[addPos[k]] += addVal[k];
    for (int k = rBeg[i]; k < rBeg[i + 1]; ++k) R[raddPos[k]] += raddVal[k];
    if (id < na) {
        const double s = dt / pv0[id];
        for (int r = r0; r < r1; ++r) {
            R[r] *= s;
            for (int k = Jrow[r]; k < Jrow[r + 1]; ++k) J[k] *= s;
        }
    }
}

// ---------------------------------------------------------------------------------------------------------------
// host side

int fail(int code, const std::string& msg) {
    rsg::set_last_error(msg);
    return code;
}

template <class T>
int upload(T** d, const std::vector<T>& h, cudaStream_t st) {
    *d = nullptr;
    if (h.empty()) return RSG_OK;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(d), h.size() * sizeof(T), st);
    if (e != cudaSuccess) return fail(RSG_ENOMEM, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
    e = cudaMemcpyAsync(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return fail(RSG_ECUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
    return RSG_OK;
}

}  // namespace

struct rsg_bo_assembler {
    int device = 0;
    int na = 0, nv = 3, nw = 0, nrows = 0;
    long long nnz = 0;
    Model m{};
    cudaStream_t own = nullptr;
    cudaEvent_t last = nullptr;      // recorded after each assembly's work, on the stream it ran on: the next call (and
                                     // the release of the buffers) waits for it, so calls on different streams are ordered
    // device arrays
    double* tab = nullptr;
    Tab* utab = nullptr;
    double* pv0 = nullptr;
    int *adjStart = nullptr, *adjNbr = nullptr, *adjConn = nullptr, *adjPos = nullptr, *connA = nullptr;
    double *trans = nullptr, *dDepth = nullptr;
    int *blkStart = nullptr, *selfPos = nullptr, *Jrow = nullptr;
    double* rec = nullptr;
    int* connB = nullptr;
    int nconn = 0;
    double* flux = nullptr;          // kFluxWords per connection (k_bo_conn)
    unsigned char* flag = nullptr;   // per connection: phases whose potential difference is zero
    // well addend lists: packed on the host, one upload per assembly into a device buffer grown on demand
    std::vector<char> stage;
    char* dstage = nullptr;
    size_t capStage = 0;
    std::vector<int> JrowH;
    std::vector<void*> owned;
    // buffers of the host-vector form (rsg_bo_assemble_host), allocated at its first call
    double *hp = nullptr, *hsw = nullptr, *hx = nullptr, *hacc = nullptr, *hJ = nullptr, *hR = nullptr;
    unsigned char* hst = nullptr;
    long long launches = 0;
};

namespace {

// order key of a double (the device's okey), stored in the table buffer
double host_key(double v) {
    long long b;
    std::memcpy(&b, &v, 8);
    if (b == (long long)0x8000000000000000ULL) b = 0;
    b ^= (b >> 63) & 0x7fffffffffffffffLL;
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}

Tab put_table(std::vector<double>& buf, const rsg_table& t) {
    Tab d{0, 0, 0, 0, 0, 0};
    if (t.n <= 0) return d;
    d.n = t.n;
    d.clamp = t.clamp ? 1 : 0;
    d.x = int(buf.size());
    buf.insert(buf.end(), t.x, t.x + t.n);
    d.y = int(buf.size());
    buf.insert(buf.end(), t.y, t.y + t.n);
    d.s = int(buf.size());
    for (int i = 0; i + 1 < t.n; ++i) {   // Table1D::eval's slope (engine/src/fluid.cpp:22-23)
        const double dx = t.x[i + 1] - t.x[i];
        buf.push_back(dx != 0 ? (t.y[i + 1] - t.y[i]) / dx : 0.0);
    }
    buf.push_back(0.0);
    d.k = int(buf.size());
    for (int i = 0; i < t.n; ++i) buf.push_back(host_key(t.x[i]));
    return d;
}

bool table_ok(const rsg_table& t) { return t.n == 0 || (t.n > 0 && t.x && t.y); }

}  // namespace

extern "C" int rsg_bo_create(rsg_bo_assembler** out, const rsg_bo_grid* g, const rsg_bo_fluid* f, const rsg_bo_satfun* sf,
                             int nrows, int nw, const int* J_rowPtr, const int* J_col, int device) {
    if (!out) return fail(RSG_EINVAL, "rsg_bo_create: null output handle");
    *out = nullptr;
    if (!g || !f || !sf || !J_rowPtr || !J_col) return fail(RSG_EINVAL, "rsg_bo_create: null argument");
    const int na = g->na, nv = g->nv;
    if (na < 1 || nv != 3) return fail(RSG_EINVAL, "rsg_bo_create: na >= 1 and nv = 3 (water, oil, gas) are required");
    if (nw < 0 || (long long)nrows != (long long)na * nv + nw) return fail(RSG_EINVAL, "rsg_bo_create: nrows must be na * nv + nw");
    if (!g->adj_start || !g->adj_nbr || !g->adj_conn || !g->conn_a || !g->conn_trans || !g->conn_ddepth || !g->pore_vol)
        return fail(RSG_EINVAL, "rsg_bo_create: null grid array");
    // the model this path implements: three phases, live oil, dry gas, unscaled tables, ECLIPSE default oil kr
    if (!f->water || !f->oil || !f->gas || !f->live || f->vap)
        return fail(RSG_EINVAL, "rsg_bo_create: only the three-phase live-oil / dry-gas model is supported (water, oil, gas, live, no vaporised oil)");
    if (sf->kro_model != 0 || sf->three_point || !sf->water || !sf->gas)
        return fail(RSG_EINVAL, "rsg_bo_create: only unscaled SWOF / SGOF tables with the default three-phase oil kr are supported");
    if (g->i_sw < 1 || g->i_sw > 2 || g->i_x < 1 || g->i_x > 2 || g->i_sw == g->i_x)
        return fail(RSG_EINVAL, "rsg_bo_create: unknown slots i_sw / i_x must be distinct values in 1..2");
    {
        int seen = 0;
        for (int p = 0; p < 3; ++p) {
            if (g->eq[p] < 0 || g->eq[p] > 2) return fail(RSG_EINVAL, "rsg_bo_create: equation offsets must be 0..2");
            seen |= 1 << g->eq[p];
        }
        if (seen != 7) return fail(RSG_EINVAL, "rsg_bo_create: equation offsets must be a permutation of 0, 1, 2");
    }
    if (f->nsat < 2 || !f->sat_rs || !f->sat_b || !f->sat_bmu || !f->under_b || !f->under_bmu)
        return fail(RSG_EINVAL, "rsg_bo_create: live oil needs at least two saturated nodes with their undersaturated tables");
    const rsg_table* tabs[] = {&f->rs_of_p, &f->pb_of_rs, &f->dead_b, &f->dead_bmu, &f->gas_b, &f->gas_bmu,
                               &sf->krw, &sf->krow, &sf->pcow, &sf->krg, &sf->krog, &sf->pcog};
    for (const rsg_table* t : tabs)
        if (!table_ok(*t)) return fail(RSG_EINVAL, "rsg_bo_create: table with n > 0 and a null array");
    for (int k = 0; k < f->nsat; ++k)
        if (!table_ok(f->under_b[k]) || !table_ok(f->under_bmu[k]) || f->under_b[k].n < 1 || f->under_bmu[k].n < 1)
            return fail(RSG_EINVAL, "rsg_bo_create: empty undersaturated table");

    // pattern: the engine's scalar Jacobian (Simulator::buildPattern, engine/src/simulator.cpp:465-510): cell row
    // a nv + e holds the blocks of the cell and its neighbours in column order, nv columns each, then the cell's well
    // columns; then one row per well
    const long long nconn = g->nconn;
    if (nconn < 0) return fail(RSG_EINVAL, "rsg_bo_create: nconn must be >= 0");
    std::vector<int> adjStart(g->adj_start, g->adj_start + na + 1);
    if (adjStart[0] != 0) return fail(RSG_EINVAL, "rsg_bo_create: adj_start[0] must be 0");
    for (int a = 0; a < na; ++a)
        if (adjStart[a + 1] < adjStart[a]) return fail(RSG_EINVAL, "rsg_bo_create: adj_start must be non-decreasing");
    const int nadj = adjStart[na];
    std::vector<int> adjNbr(g->adj_nbr, g->adj_nbr + nadj), adjConn(g->adj_conn, g->adj_conn + nadj);
    std::vector<int> connA(g->conn_a, g->conn_a + nconn);
    // second cell of each connection, as named from its first cell's adjacency and from its own; how often each side
    // names it
    std::vector<int> connB(size_t(nconn), -1), connB2(size_t(nconn), -1), seenA(size_t(nconn), 0), seenB(size_t(nconn), 0);
    std::vector<int> blkStart(na + 1, 0), selfPos(na), adjPos(nadj);
    std::vector<int> nb;
    std::vector<int> JrowH(J_rowPtr, J_rowPtr + nrows + 1);
    if (JrowH[0] != 0) return fail(RSG_EINVAL, "rsg_bo_create: J_rowPtr[0] must be 0");
    for (int r = 0; r < nrows; ++r)
        if (JrowH[r + 1] < JrowH[r]) return fail(RSG_EINVAL, "rsg_bo_create: J_rowPtr must be non-decreasing");
    for (int a = 0; a < na; ++a) {
        nb.clear();
        nb.push_back(a);
        for (int q = adjStart[a]; q < adjStart[a + 1]; ++q) {
            const int b = adjNbr[q], c = adjConn[q];
            if (b < 0 || b >= na || b == a) return fail(RSG_EINVAL, "rsg_bo_create: neighbour index out of range");
            if (c < 0 || c >= nconn) return fail(RSG_EINVAL, "rsg_bo_create: connection index out of range");
            if (connA[size_t(c)] == a) {
                connB[size_t(c)] = b;
                ++seenA[size_t(c)];
            } else if (connA[size_t(c)] == b) {
                connB2[size_t(c)] = a;
                ++seenB[size_t(c)];
            } else {
                return fail(RSG_EINVAL, "rsg_bo_create: adjacency names a connection that does not join its cells");
            }
            nb.push_back(b);
        }
        std::sort(nb.begin(), nb.end());
        if (std::adjacent_find(nb.begin(), nb.end()) != nb.end())
            return fail(RSG_EINVAL, "rsg_bo_create: two connections join the same pair of cells (not supported)");
        blkStart[a + 1] = blkStart[a] + int(nb.size());
        selfPos[a] = int(std::lower_bound(nb.begin(), nb.end(), a) - nb.begin());
        for (int q = adjStart[a]; q < adjStart[a + 1]; ++q)
            adjPos[q] = int(std::lower_bound(nb.begin(), nb.end(), adjNbr[q]) - nb.begin());
        for (int e = 0; e < nv; ++e) {
            const int r = a * nv + e;
            const int len = JrowH[r + 1] - JrowH[r];
            if (len < int(nb.size()) * nv) return fail(RSG_EINVAL, "rsg_bo_create: J row shorter than the cell's blocks");
            int k = JrowH[r];
            for (int b : nb)
                for (int v = 0; v < nv; ++v, ++k)
                    if (J_col[k] != b * nv + v)
                        return fail(RSG_EINVAL, "rsg_bo_create: J pattern is not the engine's (cell " + std::to_string(a) + ", row " +
                                                    std::to_string(e) + ")");
            for (; k < JrowH[r + 1]; ++k)
                if (J_col[k] < na * nv || J_col[k] >= nrows)
                    return fail(RSG_EINVAL, "rsg_bo_create: a cell row's trailing columns must be well columns");
        }
    }

    for (long long c = 0; c < nconn; ++c)
        if (seenA[size_t(c)] != 1 || seenB[size_t(c)] != 1 || connB[size_t(c)] != connB2[size_t(c)])
            return fail(RSG_EINVAL, "rsg_bo_create: every connection must appear once in the adjacency of each of its two cells");
    rsg_bo_assembler* h = new rsg_bo_assembler();
    h->device = device;
    h->na = na; h->nv = nv; h->nw = nw; h->nrows = nrows; h->nnz = JrowH[nrows];
    h->JrowH = JrowH;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { delete h; return fail(RSG_ECUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e)); }
    e = cudaStreamCreateWithFlags(&h->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete h; return fail(RSG_ECUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e)); }
    e = cudaEventCreateWithFlags(&h->last, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        h->last = nullptr;
        rsg_bo_destroy(h);
        return fail(RSG_ECUDA, std::string("cudaEventCreate: ") + cudaGetErrorString(e));
    }

    Model& m = h->m;
    m.water = f->water; m.oil = f->oil; m.gas = f->gas; m.live = f->live;
    m.iSw = g->i_sw; m.iX = g->i_x;
    for (int p = 0; p < 3; ++p) m.eq[p] = g->eq[p];
    m.gravity = g->gravity;
    m.pw_ref = f->pvtw[0]; m.pw_bw = f->pvtw[1]; m.pw_cw = f->pvtw[2]; m.pw_visc = f->pvtw[3]; m.pw_cv = f->pvtw[4];
    m.rock_ref = f->rock[0]; m.rock_cr = f->rock[1];
    m.rho_oil = f->rho_sc[0]; m.rho_water = f->rho_sc[1]; m.rho_gas = f->rho_sc[2]; m.gas_factor = f->gas_factor;
    m.inv_bw = 1.0 / m.pw_bw;
    m.inv_bwvisc = 1.0 / (m.pw_bw * m.pw_visc);
    m.pw_cwv = m.pw_cw - m.pw_cv;
    m.rho_gfac = m.rho_gas * m.gas_factor;
    std::vector<double> tb;
    m.rsOfP = put_table(tb, f->rs_of_p); m.pbOfRs = put_table(tb, f->pb_of_rs);
    m.deadB = put_table(tb, f->dead_b); m.deadBMu = put_table(tb, f->dead_bmu);
    m.gasB = put_table(tb, f->gas_b); m.gasBMu = put_table(tb, f->gas_bmu);
    m.krw = put_table(tb, sf->krw); m.krow = put_table(tb, sf->krow); m.pcow = put_table(tb, sf->pcow);
    m.krg = put_table(tb, sf->krg); m.krog = put_table(tb, sf->krog); m.pcog = put_table(tb, sf->pcog);
    m.swco = sf->swco; m.sat_water = sf->water; m.sat_gas = sf->gas;
    m.nsat = f->nsat;
    m.rs = int(tb.size()); tb.insert(tb.end(), f->sat_rs, f->sat_rs + f->nsat);
    m.rsk = int(tb.size());
    for (int k = 0; k < f->nsat; ++k) tb.push_back(host_key(f->sat_rs[k]));
    m.bsat = int(tb.size()); tb.insert(tb.end(), f->sat_b, f->sat_b + f->nsat);
    m.bmusat = int(tb.size()); tb.insert(tb.end(), f->sat_bmu, f->sat_bmu + f->nsat);
    std::vector<Tab> ut;
    for (int k = 0; k < f->nsat; ++k) {
        ut.push_back(put_table(tb, f->under_b[k]));
        ut.push_back(put_table(tb, f->under_bmu[k]));
    }
    if (m.pbOfRs.n < 1) { delete h; return fail(RSG_EINVAL, "rsg_bo_create: live oil needs the pb(Rs) table"); }

    std::vector<double> trans(g->conn_trans, g->conn_trans + nconn), dd(g->conn_ddepth, g->conn_ddepth + nconn);
    std::vector<double> pv(g->pore_vol, g->pore_vol + na);
    cudaStream_t st = h->own;
    int rc = RSG_OK;
    auto up = [&](auto** d, const auto& v) {
        if (rc != RSG_OK) return;
        rc = upload(d, v, st);
        if (*d) h->owned.push_back(*d);
    };
    up(&h->tab, tb); up(&h->utab, ut); up(&h->pv0, pv);
    up(&h->adjStart, adjStart); up(&h->adjNbr, adjNbr); up(&h->adjConn, adjConn); up(&h->adjPos, adjPos);
    up(&h->connA, connA); up(&h->connB, connB); up(&h->trans, trans); up(&h->dDepth, dd);
    h->nconn = int(nconn);
    up(&h->blkStart, blkStart); up(&h->selfPos, selfPos); up(&h->Jrow, JrowH);
    if (rc == RSG_OK) {
        e = cudaMallocAsync(reinterpret_cast<void**>(&h->rec), size_t(kRecWords) * size_t(na) * sizeof(double), st);
        if (e != cudaSuccess) rc = fail(RSG_ENOMEM, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
        else h->owned.push_back(h->rec);
    }
    if (rc == RSG_OK && nconn > 0) {
        e = cudaMallocAsync(reinterpret_cast<void**>(&h->flux), size_t(kFluxWords) * size_t(nconn) * sizeof(double), st);
        if (e == cudaSuccess) {
            h->owned.push_back(h->flux);
            e = cudaMallocAsync(reinterpret_cast<void**>(&h->flag), size_t(nconn), st);
            if (e == cudaSuccess) h->owned.push_back(h->flag);
        }
        if (e != cudaSuccess) rc = fail(RSG_ENOMEM, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
    }
    if (rc == RSG_OK) {
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = fail(RSG_ECUDA, std::string("rsg_bo_create: ") + cudaGetErrorString(e));
    }
    if (rc != RSG_OK) { rsg_bo_destroy(h); return rc; }
    *out = h;
    return RSG_OK;
}

extern "C" int rsg_bo_assemble(rsg_bo_assembler* h, const double* d_p, const double* d_sw, const double* d_x,
                               const unsigned char* d_state, const double* d_acc_old, double dt, int nadd,
                               const long long* add_pos, const double* add_val, int nradd, const int* radd_pos,
                               const double* radd_val, double* d_J, double* d_R, void* stream) {
    if (!h) return fail(RSG_EINVAL, "rsg_bo_assemble: null handle");
    if (!d_p || !d_sw || !d_x || !d_state || !d_acc_old || !d_J || !d_R) return fail(RSG_EINVAL, "rsg_bo_assemble: null device pointer");
    if (!(dt > 0)) return fail(RSG_EINVAL, "rsg_bo_assemble: dt must be positive");
    if (nadd < 0 || nradd < 0 || (nadd && (!add_pos || !add_val)) || (nradd && (!radd_pos || !radd_val)))
        return fail(RSG_EINVAL, "rsg_bo_assemble: bad addend list");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return fail(RSG_ECUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    cudaStream_t st = static_cast<cudaStream_t>(stream);   // NULL: the legacy default stream
    const int na = h->na, nv = h->nv, nrows = h->nrows;
    e = cudaStreamWaitEvent(st, h->last, 0);               // the previous call's work, whatever stream it ran on
    if (e != cudaSuccess) return fail(RSG_ECUDA, std::string("cudaStreamWaitEvent: ") + cudaGetErrorString(e));
    const std::vector<int>& Jr = h->JrowH;

    // well addends grouped by the cell (or well row) they belong to, the caller's order kept within each group
    struct Add { int id; int idx; };
    std::vector<Add> ja(static_cast<size_t>(nadd)), ra(static_cast<size_t>(nradd));
    for (int k = 0; k < nadd; ++k) {
        const long long pos = add_pos[k];
        if (pos < 0 || pos >= h->nnz) return fail(RSG_EINVAL, "rsg_bo_assemble: J addend position out of range");
        const int r = int(std::upper_bound(Jr.begin(), Jr.end(), int(pos)) - Jr.begin()) - 1;
        ja[size_t(k)] = Add{r < na * nv ? r / nv : na + (r - na * nv), k};
    }
    for (int k = 0; k < nradd; ++k) {
        const int r = radd_pos[k];
        if (r < 0 || r >= nrows) return fail(RSG_EINVAL, "rsg_bo_assemble: R addend position out of range");
        ra[size_t(k)] = Add{r < na * nv ? r / nv : na + (r - na * nv), k};
    }
    auto byId = [](const Add& x, const Add& y) { return x.id < y.id; };
    std::stable_sort(ja.begin(), ja.end(), byId);
    std::stable_sort(ra.begin(), ra.end(), byId);
    std::vector<int> ids;
    for (const Add& x : ja) ids.push_back(x.id);
    for (const Add& x : ra) ids.push_back(x.id);
    for (int w = 0; w < h->nw; ++w) ids.push_back(na + w);   // every well row is rewritten (zero + its terms)
    std::sort(ids.begin(), ids.end());
    ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
    const int nac = int(ids.size());
    std::vector<int> aBeg(size_t(nac) + 1, 0), rBeg(size_t(nac) + 1, 0);
    std::vector<long long> apos(static_cast<size_t>(nadd));
    std::vector<double> aval(static_cast<size_t>(nadd));
    std::vector<int> rpos(static_cast<size_t>(nradd));
    std::vector<double> rval(static_cast<size_t>(nradd));
    {
        size_t j = 0, k = 0;
        for (int i = 0; i < nac; ++i) {
            aBeg[size_t(i)] = int(j);
            while (j < ja.size() && ja[j].id == ids[size_t(i)]) { apos[j] = add_pos[ja[j].idx]; aval[j] = add_val[ja[j].idx]; ++j; }
            rBeg[size_t(i)] = int(k);
            while (k < ra.size() && ra[k].id == ids[size_t(i)]) { rpos[k] = radd_pos[ra[k].idx]; rval[k] = radd_val[ra[k].idx]; ++k; }
        }
        aBeg[size_t(nac)] = int(j);
        rBeg[size_t(nac)] = int(k);
    }
    // the cells among them (ids < na), sorted, for k_bo_cells' lookup: they are the leading part of ids
    const int ncell = int(std::lower_bound(ids.begin(), ids.end(), na) - ids.begin());

    // one packed upload of the lists: ids, group starts, J addends, R addends
    size_t off = 0;
    auto place = [&](size_t bytes) { const size_t o = off; off = (off + bytes + 255) & ~size_t(255); return o; };
    const size_t oId = place(size_t(nac) * 4), oAB = place(size_t(nac + 1) * 4), oRB = place(size_t(nac + 1) * 4);
    const size_t oAP = place(size_t(nadd) * 8), oAV = place(size_t(nadd) * 8), oRP = place(size_t(nradd) * 4),
                 oRV = place(size_t(nradd) * 8);
    h->stage.assign(off, 0);
    auto put = [&](size_t o, const void* src, size_t bytes) { if (bytes) std::memcpy(h->stage.data() + o, src, bytes); };
    put(oId, ids.data(), size_t(nac) * 4);
    put(oAB, aBeg.data(), size_t(nac + 1) * 4);
    put(oRB, rBeg.data(), size_t(nac + 1) * 4);
    put(oAP, apos.data(), size_t(nadd) * 8);
    put(oAV, aval.data(), size_t(nadd) * 8);
    put(oRP, rpos.data(), size_t(nradd) * 4);
    put(oRV, rval.data(), size_t(nradd) * 8);
    if (off > h->capStage) {
        if (h->dstage) cudaFreeAsync(h->dstage, st);
        h->dstage = nullptr;
        h->capStage = 0;
        e = cudaMallocAsync(reinterpret_cast<void**>(&h->dstage), std::max(off, size_t(4096)), st);
        if (e != cudaSuccess) return fail(RSG_ENOMEM, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
        h->capStage = std::max(off, size_t(4096));
    }
    char* D = h->dstage;
    if (off) {
        e = cudaMemcpyAsync(D, h->stage.data(), off, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return fail(RSG_ECUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
    }
    const int* dIds = reinterpret_cast<const int*>(D + oId);
    const int grid = (na + kThreads - 1) / kThreads;
    k_bo_props<<<grid, kThreads, 0, st>>>(na, h->m, h->tab, h->utab, h->pv0, d_p, d_sw, d_x, d_state, h->rec);
    if (h->nconn > 0)
        k_bo_conn<<<(h->nconn + kThreads - 1) / kThreads, kThreads, 0, st>>>(h->nconn, na, h->m, h->rec, h->connA, h->connB, h->trans,
                                                                         h->dDepth, h->flux, h->flag);
    k_bo_cells<<<grid, kThreads, 0, st>>>(na, nv, h->nconn, h->m, dt, h->rec, h->flux, h->flag, d_acc_old, h->pv0, h->adjStart, h->adjNbr,
                                          h->adjConn, h->adjPos,
                                          h->connA, h->trans, h->dDepth, h->blkStart, h->selfPos, h->Jrow, dIds, ncell, d_J, d_R);
    h->launches += h->nconn > 0 ? 3 : 2;
    if (nac > 0) {
        k_bo_addends<<<(nac + 127) / 128, 128, 0, st>>>(na, nv, nrows, dt, dIds, nac, reinterpret_cast<const int*>(D + oAB),
                                                        reinterpret_cast<const long long*>(D + oAP), reinterpret_cast<const double*>(D + oAV),
                                                        reinterpret_cast<const int*>(D + oRB), reinterpret_cast<const int*>(D + oRP),
                                                        reinterpret_cast<const double*>(D + oRV), h->pv0, h->Jrow, d_J, d_R);
        h->launches += 1;
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(h->last, st);
    if (e != cudaSuccess) return fail(RSG_ECUDA, std::string("rsg_bo_assemble launch: ") + cudaGetErrorString(e));
    return RSG_OK;
}

extern "C" int rsg_bo_assemble_host(rsg_bo_assembler* h, const double* p, const double* sw, const double* x, const unsigned char* state,
                                    const double* acc_old, double dt, int nadd, const long long* add_pos, const double* add_val,
                                    int nradd, const int* radd_pos, const double* radd_val, double* J, double* R) {
    if (!h) return fail(RSG_EINVAL, "rsg_bo_assemble_host: null handle");
    if (!p || !sw || !x || !state || !acc_old || !J || !R) return fail(RSG_EINVAL, "rsg_bo_assemble_host: null host pointer");
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return fail(RSG_ECUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    cudaStream_t st = h->own;
    const size_t na = size_t(h->na);
    if (!h->hp) {
        void** bufs[] = {reinterpret_cast<void**>(&h->hp), reinterpret_cast<void**>(&h->hsw), reinterpret_cast<void**>(&h->hx),
                         reinterpret_cast<void**>(&h->hacc), reinterpret_cast<void**>(&h->hJ), reinterpret_cast<void**>(&h->hR),
                         reinterpret_cast<void**>(&h->hst)};
        const size_t sizes[] = {na * 8, na * 8, na * 8, na * 24, size_t(h->nnz) * 8, size_t(h->nrows) * 8, na};
        for (int k = 0; k < 7; ++k) {
            e = cudaMallocAsync(bufs[k], std::max(sizes[k], size_t(8)), st);
            if (e != cudaSuccess) return fail(RSG_ENOMEM, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
            h->owned.push_back(*bufs[k]);
        }
    }
    const struct { void* d; const void* hsrc; size_t n; } in[] = {
        {h->hp, p, na * 8}, {h->hsw, sw, na * 8}, {h->hx, x, na * 8}, {h->hacc, acc_old, na * 24}, {h->hst, state, na}};
    for (const auto& c : in) {
        e = cudaMemcpyAsync(c.d, c.hsrc, c.n, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return fail(RSG_ECUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
    }
    const int rc = rsg_bo_assemble(h, h->hp, h->hsw, h->hx, h->hst, h->hacc, dt, nadd, add_pos, add_val, nradd, radd_pos, radd_val,
                                   h->hJ, h->hR, st);
    if (rc != RSG_OK) return rc;
    e = cudaMemcpyAsync(J, h->hJ, size_t(h->nnz) * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(R, h->hR, size_t(h->nrows) * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(RSG_ECUDA, std::string("rsg_bo_assemble_host: ") + cudaGetErrorString(e));
    return RSG_OK;
}

extern "C" int rsg_bo_destroy(rsg_bo_assembler* h) {
    if (!h) return RSG_OK;
    cudaSetDevice(h->device);
    cudaStream_t st = h->own;
    if (st && h->last) cudaStreamWaitEvent(st, h->last, 0);   // the last assembly's work, on any stream, first
    for (void* p : h->owned) cudaFreeAsync(p, st);
    if (h->dstage) cudaFreeAsync(h->dstage, st);
    if (st) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    if (h->last) cudaEventDestroy(h->last);
    delete h;
    return RSG_OK;
}
