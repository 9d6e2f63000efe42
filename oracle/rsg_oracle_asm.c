/* C restatement of the reference engine's black-oil Jacobian assembly (TEST INFRASTRUCTURE ONLY: the checker of the
 * device assembly, pinned bit for bit to the reference's own J and R by tests/test_oracle.py).
 *
 * Follows, for the standard black-oil model (water, live oil, dry gas, one PVT and one saturation region, unscaled
 * tables, ECLIPSE default three-phase oil kr):
 *   - the forward-mode dual numbers of engine/include/ressim/ad.h (every rule in its order of operations);
 *   - Table1D::eval (engine/src/fluid.cpp:10-26), FluidModel::bw / bwMu / pvMult (:191-203), rsSat (:248-254),
 *     liveOil / liveOilAD (:257-280), SatFunctions::kro (:445-460);
 *   - Simulator::evalCell (engine/src/simulator.cpp:2133-2276) for that model;
 *   - the cell loop of Simulator::assemble (:2500-2686): accumulation, then per connection in adjacency order the
 *     phase fluxes and the dissolved gas carried by the oil;
 *   - the well terms as the caller's ordered addends (the engine's well loop, :2692-2954), then the row scaling
 *     dt / PV (:3010-3032).
 * Written literally: every derivative slot is computed, zero or not. Compiled with -ffp-contract=off.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../include/rsg.h"

typedef struct { double v, d[3]; } ad3;
typedef struct { double v, d[6]; } ad6;

static ad3 c3(double v) { ad3 r = {v, {0, 0, 0}}; return r; }
static ad3 var3(double v, int s) { ad3 r = c3(v); r.d[s] = 1.0; return r; }
static ad3 add3(ad3 a, ad3 b) { a.v += b.v; for (int i = 0; i < 3; ++i) a.d[i] += b.d[i]; return a; }      /* a += b */
static ad3 sub3(ad3 a, ad3 b) { a.v -= b.v; for (int i = 0; i < 3; ++i) a.d[i] -= b.d[i]; return a; }      /* a -= b */
static ad3 mul3(ad3 a, ad3 b) { for (int i = 0; i < 3; ++i) a.d[i] = a.d[i] * b.v + a.v * b.d[i]; a.v *= b.v; return a; }
static ad3 div3(ad3 a, ad3 b) {
    const double inv = 1.0 / b.v;
    for (int i = 0; i < 3; ++i) a.d[i] = (a.d[i] * b.v - a.v * b.d[i]) * inv * inv;
    a.v *= inv;
    return a;
}
static ad3 addc3(ad3 a, double b) { a.v += b; return a; }                                   /* a + b and b + a */
static ad3 subc3(ad3 a, double b) { a.v -= b; return a; }                                   /* a - b */
static ad3 mulc3(ad3 a, double b) { a.v *= b; for (int i = 0; i < 3; ++i) a.d[i] *= b; return a; }
static ad3 divc3(ad3 a, double b) { return mulc3(a, 1.0 / b); }                             /* a / b = a * (1 / b) */
static ad3 neg3(ad3 a) { a.v = -a.v; for (int i = 0; i < 3; ++i) a.d[i] = -a.d[i]; return a; }
static ad3 csub3(double a, ad3 b) { return addc3(neg3(b), a); }                             /* a - b = (-b) += a */
static ad3 chain(ad3 x, double f, double df) { ad3 r = c3(f); for (int i = 0; i < 3; ++i) r.d[i] = df * x.d[i]; return r; }
static ad3 chain2(ad3 x, ad3 y, double f, double fx, double fy) {
    ad3 r = c3(f);
    for (int i = 0; i < 3; ++i) r.d[i] = fx * x.d[i] + fy * y.d[i];
    return r;
}
static ad6 lift(ad3 a, int off) { ad6 r; memset(&r, 0, sizeof r); r.v = a.v; for (int i = 0; i < 3; ++i) r.d[off + i] = a.d[i]; return r; }
static ad6 add6(ad6 a, ad6 b) { a.v += b.v; for (int i = 0; i < 6; ++i) a.d[i] += b.d[i]; return a; }
static ad6 sub6(ad6 a, ad6 b) { a.v -= b.v; for (int i = 0; i < 6; ++i) a.d[i] -= b.d[i]; return a; }
static ad6 mul6(ad6 a, ad6 b) { for (int i = 0; i < 6; ++i) a.d[i] = a.d[i] * b.v + a.v * b.d[i]; a.v *= b.v; return a; }
static ad6 mulc6(ad6 a, double b) { a.v *= b; for (int i = 0; i < 6; ++i) a.d[i] *= b; return a; }

/* Table1D::eval */
static double teval(const rsg_table* t, double xv, double* dydx) {
    const int n = t->n;
    if (n == 0) { *dydx = 0; return 0; }
    if (n == 1) { *dydx = 0; return t->y[0]; }
    if (t->clamp) {
        if (xv <= t->x[0]) { *dydx = 0; return t->y[0]; }
        if (xv >= t->x[n - 1]) { *dydx = 0; return t->y[n - 1]; }
    }
    int i;
    if (xv <= t->x[1]) i = 0;
    else if (xv >= t->x[n - 2]) i = n - 2;
    else {                                     /* upper_bound - 1 */
        int lo = 0, cnt = n;
        while (cnt > 0) {
            const int step = cnt / 2;
            if (!(xv < t->x[lo + step])) { lo += step + 1; cnt -= step + 1; }
            else cnt = step;
        }
        i = lo - 1;
    }
    const double dx = t->x[i + 1] - t->x[i];
    const double s = dx != 0 ? (t->y[i + 1] - t->y[i]) / dx : 0.0;
    *dydx = s;
    return t->y[i] + s * (xv - t->x[i]);
}
static ad3 tad(const rsg_table* t, ad3 x) { double d; const double f = teval(t, x.v, &d); return chain(x, f, d); }

/* FluidModel::liveOil / liveOilAD */
static double live_oil(const rsg_bo_fluid* F, double p, double rs, int which) {
    const int n = F->nsat;
    const double* R = F->sat_rs;
    int k;
    if (rs <= R[1]) k = 0;
    else if (rs >= R[n - 2]) k = n - 2;
    else {
        int lo = 0, cnt = n;
        while (cnt > 0) {
            const int step = cnt / 2;
            if (!(rs < R[lo + step])) { lo += step + 1; cnt -= step + 1; }
            else cnt = step;
        }
        k = lo - 1;
    }
    double d;
    const double pb = teval(&F->pb_of_rs, rs, &d);
    const double dp = p - pb;
    const double* sat = which == 0 ? F->sat_b : F->sat_bmu;
    const rsg_table* ur = which == 0 ? F->under_b : F->under_bmu;
    const double v0 = sat[k] * teval(&ur[k], dp, &d);
    const double v1 = sat[k + 1] * teval(&ur[k + 1], dp, &d);
    const double w = (rs - R[k]) / (R[k + 1] - R[k]);
    return v0 + w * (v1 - v0);
}
static ad3 live_oil_ad(const rsg_bo_fluid* F, ad3 p, ad3 rs, int which) {
    const double f = live_oil(F, p.v, rs.v, which);
    const double hp = 1e-4 * fmax(1.0, fabs(p.v));
    const double hr = 1e-5 * fmax(1e-2, fabs(rs.v));
    const double fp = (live_oil(F, p.v + hp, rs.v, which) - live_oil(F, p.v - hp, rs.v, which)) / (2 * hp);
    const double fr = (live_oil(F, p.v, rs.v + hr, which) - live_oil(F, p.v, rs.v - hr, which)) / (2 * hr);
    return chain2(p, rs, f, fp, fr);
}
static ad3 rs_sat(const rsg_bo_fluid* F, ad3 p) {
    if (!F->live) return c3(0.0);
    double d;
    double r = teval(&F->rs_of_p, p.v, &d);
    if (r < 0) { r = 0; d = 0; }
    return chain(p, r, d);
}
/* SatFunctions::kro, unscaled, ECLIPSE default model */
static ad3 kro(const rsg_bo_satfun* S, ad3 sw, ad3 sg) {
    if (S->water && !S->gas) return tad(&S->krow, sw);
    if (!S->water && S->gas) return tad(&S->krog, sg);
    if (!S->water && !S->gas) return c3(1.0);
    ad3 dw = subc3(sw, S->swco);
    if (dw.v < 0) dw = c3(0.0);
    const ad3 swEff = add3(sw, sg);
    const ad3 sgEff = subc3(add3(sw, sg), S->swco);
    const ad3 den = add3(sg, dw);
    if (den.v < 1e-9) return tad(&S->krow, swEff);
    return div3(add3(mul3(sg, tad(&S->krog, sgEff)), mul3(dw, tad(&S->krow, swEff))), den);
}

typedef struct { ad3 P[3], mob[3], rho[3], mobRs, acc[3]; } cellflux;

/* Simulator::evalCell for this model */
static void eval_cell(const rsg_bo_grid* g, const rsg_bo_fluid* F, const rsg_bo_satfun* S, int c, const double* p, const double* sw,
                      const double* x, const unsigned char* state, cellflux* f) {
    memset(f, 0, sizeof *f);
    const int W = F->water, O = F->oil, G = F->gas;
    const ad3 P = var3(p[c], 0);
    ad3 Sw = c3(W && !O ? 1.0 : 0.0), Sg = c3(0.0), rs = c3(0.0);
    if (g->i_sw >= 0) Sw = var3(sw[c], g->i_sw);
    const int st = state[c];
    if (G) {
        if (st == 1) { Sg = var3(x[c], g->i_x); if (F->live) rs = mulc3(rs_sat(F, P), 1.0); }
        else if (st == 0) rs = var3(x[c], g->i_x);
        else { Sg = csub3(1.0, Sw); if (F->live) rs = mulc3(rs_sat(F, P), 1.0); }
    }
    const ad3 So = (O && !(G && st == 2)) ? sub3(csub3(1.0, Sw), Sg) : c3(0.0);
    ad3 X = mulc3(subc3(P, F->rock[0]), F->rock[1]);
    const ad3 pv = mulc3(add3(addc3(X, 1.0), mulc3(mul3(X, X), 0.5)), g->pore_vol[c]);
    ad3 bo = c3(0.0);
    if (W) {
        f->P[0] = O ? sub3(P, mulc3(mulc3(tad(&S->pcow, Sw), 1.0), 1.0)) : P;
        X = mulc3(subc3(f->P[0], F->pvtw[0]), F->pvtw[2]);
        const ad3 bw = divc3(add3(addc3(X, 1.0), mulc3(mul3(X, X), 0.5)), F->pvtw[1]);
        const ad3 Y = mulc3(subc3(f->P[0], F->pvtw[0]), F->pvtw[2] - F->pvtw[4]);
        const ad3 bwmu = divc3(add3(addc3(Y, 1.0), mulc3(mul3(Y, Y), 0.5)), F->pvtw[1] * F->pvtw[3]);
        const ad3 kr = !O ? c3(1.0) : tad(&S->krw, Sw);
        f->mob[0] = mul3(bwmu, kr);
        f->rho[0] = mulc3(bw, F->rho_sc[1]);
        f->acc[0] = mul3(mul3(pv, bw), Sw);
    }
    if (O) {
        f->P[1] = P;
        bo = F->live ? live_oil_ad(F, P, rs, 0) : tad(&F->dead_b, P);
        ad3 kr = c3(1.0);
        if (W || G) kr = kro(S, Sw, Sg);
        f->mob[1] = mul3(F->live ? live_oil_ad(F, P, rs, 1) : tad(&F->dead_bmu, P), kr);
        f->rho[1] = mul3(bo, addc3(mulc3(rs, F->rho_sc[2] * F->gas_factor), F->rho_sc[0]));
        f->acc[1] = mul3(mul3(pv, bo), So);
        f->mobRs = mul3(f->mob[1], rs);
    }
    if (G) {
        f->P[2] = add3(P, tad(&S->pcog, Sg));
        const ad3 krg = tad(&S->krg, Sg);
        const ad3 bg = tad(&F->gas_b, f->P[2]);
        f->mob[2] = mul3(tad(&F->gas_bmu, f->P[2]), krg);
        f->rho[2] = mulc3(bg, F->rho_sc[2] * F->gas_factor);
        f->acc[2] = mul3(pv, add3(mul3(bg, Sg), O ? mul3(mul3(rs, bo), So) : c3(0.0)));
    }
}

/* J (the engine's scalar pattern, zeroed here) and R at the state: reservoir terms, the addends in list order, the
 * row scaling. Returns 0, or -1 when a cell row does not hold the blocks of its neighbours (pattern mismatch). */
int orc_bo_assemble(const rsg_bo_grid* g, const rsg_bo_fluid* F, const rsg_bo_satfun* S, int nrows, const int* Jrow, const int* Jcol,
                    const double* p, const double* sw, const double* x, const unsigned char* state, const double* accOld, double dt,
                    int nadd, const long long* addPos, const double* addVal, int nradd, const int* raddPos, const double* raddVal,
                    double* J, double* R) {
    const int na = g->na, nv = g->nv;
    memset(J, 0, sizeof(double) * (size_t)Jrow[nrows]);
    memset(R, 0, sizeof(double) * (size_t)nrows);
    cellflux* cf = (cellflux*)malloc(sizeof(cellflux) * (size_t)na);
    if (!cf) return -2;
    for (int c = 0; c < na; ++c) eval_cell(g, F, S, c, p, sw, x, state, &cf[c]);
    const int ph[3] = {F->water, F->oil, F->gas};
    const double invDt = 1.0 / dt;
    for (int a = 0; a < na; ++a) {
        /* position of a column cell b among the row's blocks: its index in the row's block columns */
        const int r0 = a * nv;
        const int nblk = (Jrow[r0 + 1] - Jrow[r0]);
        int self = -1;
        for (int q = 0; q < nblk; q += nv) if (Jcol[Jrow[r0] + q] == a * nv) self = q / nv;
        if (self < 0) { free(cf); return -1; }
        for (int pp = 0; pp < 3; ++pp) {
            if (!ph[pp]) continue;
            ad3 acc = cf[a].acc[pp];
            acc.v -= accOld[(size_t)a * 3 + pp];
            const int r = r0 + g->eq[pp];
            R[r] += acc.v * invDt;
            double* row = J + Jrow[r] + self * nv;
            for (int k = 0; k < nv; ++k) row[k] += acc.d[k] * invDt;
        }
        for (int e = g->adj_start[a]; e < g->adj_start[a + 1]; ++e) {
            const int cn = g->adj_conn[e], b = g->adj_nbr[e];
            const double dD = g->conn_a[cn] == a ? g->conn_ddepth[cn] : -g->conn_ddepth[cn];
            int nbp = -1;
            for (int q = 0; q < nblk; q += nv) if (Jcol[Jrow[r0] + q] == b * nv) nbp = q / nv;
            if (nbp < 0) { free(cf); return -1; }
            const double tr = g->conn_trans[cn];
            for (int pp = 0; pp < 3; ++pp) {
                if (!ph[pp]) continue;
                const ad6 rho = mulc6(add6(lift(cf[a].rho[pp], 0), lift(cf[b].rho[pp], 3)), 0.5);
                const ad6 dphi = add6(sub6(lift(cf[a].P[pp], 0), lift(cf[b].P[pp], 3)), mulc6(rho, g->gravity * dD));
                const int upA = dphi.v >= 0;
                for (int pass = 0; pass < 2; ++pass) {       /* the phase's flux; then, for oil, its dissolved gas */
                    if (pass == 1 && !(pp == 1 && F->live)) break;
                    const ad3 mA = pass == 0 ? cf[a].mob[pp] : cf[a].mobRs;
                    const ad3 mB = pass == 0 ? cf[b].mob[pp] : cf[b].mobRs;
                    const ad6 mob = upA ? lift(mA, 0) : lift(mB, 3);
                    const ad6 Fl = mulc6(mul6(mob, dphi), tr);
                    const int r = r0 + g->eq[pass == 0 ? pp : 2];
                    R[r] += Fl.v;
                    double* rs = J + Jrow[r] + self * nv;
                    double* rn = J + Jrow[r] + nbp * nv;
                    for (int k = 0; k < nv; ++k) { rs[k] += Fl.d[k]; rn[k] += Fl.d[3 + k]; }
                }
            }
        }
    }
    free(cf);
    for (int k = 0; k < nadd; ++k) J[addPos[k]] += addVal[k];
    for (int k = 0; k < nradd; ++k) R[raddPos[k]] += raddVal[k];
    for (int a = 0; a < na; ++a) {
        const double s = dt / g->pore_vol[a];
        for (int e = 0; e < nv; ++e) {
            const int r = a * nv + e;
            R[r] *= s;
            for (int q = Jrow[r]; q < Jrow[r + 1]; ++q) J[q] *= s;
        }
    }
    return 0;
}
