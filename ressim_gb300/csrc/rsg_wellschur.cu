// Well Schur complement on the device: the Newton Jacobian with its well (BHP) rows in, the block system of the cells
// out, every Newton iteration, without the values ever visiting the host.
//
// The engine eliminates the wells before its block solver (WellSchur::build / buildInPlace / reduceRhs / recover,
// engine/src/bsr.cpp:733-990): with nc = na * nv cell rows and nw well rows,
//   S = A_cc - A_cw D_ww^-1 A_wc,   b_c' = b_c - A_cw D_ww^-1 b_w,   x_w = D_ww^-1 (b_w - A_wc x_c),
// where D_ww is diagonal (a well row couples only to its own BHP) and the fill of S is the clique of cells of every
// well. The block pattern of S depends on the scalar pattern and on which cell-to-well couplings are nonzero; the
// engine keeps it while those are unchanged (its pattern hash, bsr.cpp:759-769), which is the common case for a whole
// run. Here that split is explicit:
//
// * The plan (host, rebuilt only when the pattern or the nonzero set of the couplings changes): the S pattern, and
//   for every S value the Jacobian entry it starts from and the ordered list of well terms subtracted from it -- the
//   order of the engine's own loops (cell row, then its couplings in row order, then the well row's cells in row
//   order), so that every value is rounded as the engine rounds it.
// * Every call: a kernel tests the couplings for zeros and the wells for a usable BHP derivative (the only
//   value-dependent inputs of the plan; a few kilobytes come back to the host), then one kernel writes every value of
//   S straight into the solver's block storage. The right-hand side reduction and the BHP recovery are one kernel
//   each around the solve.
#include "rsg_impl.h"
#include "rsg_block3.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <unordered_map>
#include <vector>

namespace rsg {

namespace {

__device__ __forceinline__ double wdm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double wds(double a, double b) { return __dsub_rn(a, b); }

// nonzero flags of the cell-to-well couplings and, per well, whether its row is usable: a BHP derivative larger
// than 1e-12 of the row's largest cell coupling and finite (bsr.cpp:742-746), no nonzero coupling to another well
__global__ void k_ws_check(int ncpl, const int* __restrict__ cplPos, const double* __restrict__ jv, unsigned char* mask, int nwell,
                           const int* __restrict__ diagPos, const int* __restrict__ wcBeg, const int* __restrict__ wcPos,
                           const int* __restrict__ wwBeg, const int* __restrict__ wwPos, unsigned char* wellOk) {
    const int t = int(blockIdx.x * blockDim.x + threadIdx.x), stride = int(gridDim.x * blockDim.x);
    for (int k = t; k < ncpl; k += stride) mask[k] = __ldg(jv + __ldg(cplPos + k)) != 0.0 ? 1 : 0;
    for (int w = t; w < nwell; w += stride) {
        const int dp = __ldg(diagPos + w);
        const double d = dp >= 0 ? __ldg(jv + dp) : 0.0;
        double rowMax = 0;
        for (int q = __ldg(wcBeg + w); q < __ldg(wcBeg + w + 1); ++q) rowMax = fmax(rowMax, fabs(__ldg(jv + __ldg(wcPos + q))));
        bool ok = fabs(d) > 1e-12 * fmax(rowMax, 1e-300) && isfinite(d);
        for (int q = __ldg(wwBeg + w); q < __ldg(wwBeg + w + 1); ++q) ok = ok && __ldg(jv + __ldg(wwPos + q)) == 0.0;
        wellOk[w] = ok ? 1 : 0;
    }
}

// S values: every value starts from its Jacobian entry (0 + a, as the engine accumulates it into a zeroed block) or
// from zero (fill), then the scalars with well terms subtract them in the engine's order: f = a_cw * (1 / d_w),
// s -= f * a_wc (bsr.cpp:813-830), each product and difference rounded on its own
__global__ void k_ws_base(long long nval, const int* __restrict__ base, const double* __restrict__ jv, double* sv) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nval; q += (long long)gridDim.x * blockDim.x) {
        const int p = __ldg(base + q);
        sv[q] = p >= 0 ? __dadd_rn(0.0, __ldg(jv + p)) : 0.0;
    }
}
__global__ void k_ws_fill(int nfill, const long long* __restrict__ scalar, const int* __restrict__ beg, const int* __restrict__ tCw,
                          const int* __restrict__ tDiag, const int* __restrict__ tWc, const double* __restrict__ jv, double* sv) {
    for (int k = int(blockIdx.x * blockDim.x + threadIdx.x); k < nfill; k += int(gridDim.x * blockDim.x)) {
        const long long q = __ldg(scalar + k);
        double s = sv[q];
        for (int t = __ldg(beg + k); t < __ldg(beg + k + 1); ++t) {
            const double dInv = 1.0 / __ldg(jv + __ldg(tDiag + t));
            const double f = wdm(__ldg(jv + __ldg(tCw + t)), dInv);
            s = wds(s, wdm(f, __ldg(jv + __ldg(tWc + t))));
        }
        sv[q] = s;
    }
}

// b_c' = b_c - sum over the row's nonzero couplings of (a_cw * (1 / d_w)) * b_w (bsr.cpp:973-980), into the reduced
// vector (the solver's original row order)
__global__ void k_ws_rhs(int nred, const int* __restrict__ redFull, const int* __restrict__ rBeg, const int* __restrict__ rCw,
                         const int* __restrict__ rDiag, const int* __restrict__ rWellFull, const double* __restrict__ jv,
                         const double* __restrict__ bFull, double* bc) {
    for (int i = int(blockIdx.x * blockDim.x + threadIdx.x); i < nred; i += int(gridDim.x * blockDim.x)) {
        double s = __ldg(bFull + __ldg(redFull + i));
        for (int t = __ldg(rBeg + i); t < __ldg(rBeg + i + 1); ++t) {
            const double dInv = 1.0 / __ldg(jv + __ldg(rDiag + t));
            s = wds(s, wdm(wdm(__ldg(jv + __ldg(rCw + t)), dInv), __ldg(bFull + __ldg(rWellFull + t))));
        }
        bc[i] = s;
    }
}

// x = [x_c ; (b_w - sum a_wc x_c) * (1 / d_w)] (bsr.cpp:982-990)
__global__ void k_ws_recover(int nred, const int* __restrict__ redFull, const double* __restrict__ xc, int nwell,
                             const int* __restrict__ wellFull, const int* __restrict__ diagPos, const int* __restrict__ wcBeg,
                             const int* __restrict__ wcPos, const int* __restrict__ wcRed, const double* __restrict__ jv,
                             const double* __restrict__ bFull, double* xFull) {
    const int t = int(blockIdx.x * blockDim.x + threadIdx.x), stride = int(gridDim.x * blockDim.x);
    for (int i = t; i < nred; i += stride) xFull[__ldg(redFull + i)] = xc[i];
    for (int w = t; w < nwell; w += stride) {
        const int wf = __ldg(wellFull + w);
        double s = __ldg(bFull + wf);
        for (int q = __ldg(wcBeg + w); q < __ldg(wcBeg + w + 1); ++q) s = wds(s, wdm(__ldg(jv + __ldg(wcPos + q)), xc[__ldg(wcRed + q)]));
        xFull[wf] = wdm(s, 1.0 / __ldg(jv + __ldg(diagPos + w)));
    }
}

int grid_of(long long n) {
    const long long cap = 16LL * device_sm_count();
    const long long b = (n + 255) / 256;
    return int(std::max(1LL, std::min(b, cap)));
}

}  // namespace

// ---- host plan
bool ws_same_pattern(const WsPlan& W, int nsys, int nv, const int* nrows, const int* na, const int* nw, const int* const* rowPtr,
                     const int* const* col) {
    if (W.nsys != nsys || W.nv != nv) return false;
    for (int s = 0; s < nsys; ++s) {
        const size_t su = size_t(s);
        if (W.nrows[su] != nrows[s] || W.na[su] != na[s] || W.nw[su] != nw[s]) return false;
        const int nnz = rowPtr[s][nrows[s]];
        if (W.jrp[su].size() != size_t(nrows[s]) + 1 || W.jci[su].size() != size_t(nnz)) return false;
        if (!std::equal(W.jrp[su].begin(), W.jrp[su].end(), rowPtr[s])) return false;
        if (!std::equal(W.jci[su].begin(), W.jci[su].end(), col[s])) return false;
    }
    return true;
}

// Pattern part: everything that does not depend on which couplings are nonzero (the coupling and well lists).
bool ws_plan_pattern(WsPlan& W, int nsys, int nv, const int* nrows, const int* na, const int* nw, const int* const* rowPtr,
                     const int* const* col, std::string& err) {
    W = WsPlan{};
    W.nsys = nsys;
    W.nv = nv;
    W.nrows.assign(nrows, nrows + nsys);
    W.na.assign(na, na + nsys);
    W.nw.assign(nw, nw + nsys);
    W.jEnt0.assign(size_t(nsys) + 1, 0);
    W.full0.assign(size_t(nsys) + 1, 0);
    W.red0.assign(size_t(nsys) + 1, 0);
    W.well0.assign(size_t(nsys) + 1, 0);
    W.jrp.resize(size_t(nsys));
    W.jci.resize(size_t(nsys));
    W.wcBeg.assign(1, 0);
    W.wwBeg.assign(1, 0);
    for (int s = 0; s < nsys; ++s) {
        const size_t su = size_t(s);
        const int nc = na[s] * nv;
        if (na[s] < 1 || nw[s] < 0 || nrows[s] != nc + nw[s]) { err = "system " + std::to_string(s) + ": nrows must be na * nv + nw"; return false; }
        const int* rp = rowPtr[s];
        const int* ci = col[s];
        if (rp[0] != 0) { err = "rowPtr[0] must be 0 (system " + std::to_string(s) + ")"; return false; }
        W.jrp[su].assign(rp, rp + nrows[s] + 1);
        W.jci[su].assign(ci, ci + rp[nrows[s]]);
        const int e0 = W.jEnt0[su];
        W.jEnt0[su + 1] = e0 + rp[nrows[s]];
        W.full0[su + 1] = W.full0[su] + nrows[s];
        W.red0[su + 1] = W.red0[su] + nc;
        W.well0[su + 1] = W.well0[su] + nw[s];
        for (int r = 0; r < nc; ++r) W.redFull.push_back(W.full0[su] + r);
        for (int r = 0; r < nrows[s]; ++r)
            for (int p = rp[r]; p < rp[r + 1]; ++p)
                if (ci[p] < 0 || ci[p] >= nrows[s]) { err = "column out of range in system " + std::to_string(s); return false; }
        // cell rows: their couplings to wells, in row order (the candidates; which are nonzero is decided per call)
        for (int r = 0; r < nc; ++r)
            for (int p = rp[r]; p < rp[r + 1]; ++p)
                if (ci[p] >= nc) { W.cplPos.push_back(e0 + p); W.cplRow.push_back(W.red0[su] + r); W.cplWell.push_back(W.well0[su] + ci[p] - nc); }
        // well rows: diagonal, cell entries (all of them, in row order) and couplings to other wells
        for (int w = 0; w < nw[s]; ++w) {
            const int r = nc + w;
            int dp = -1;
            for (int p = rp[r]; p < rp[r + 1]; ++p) {
                const int c = ci[p];
                if (c == r) dp = e0 + p;
                else if (c < nc) { W.wcPos.push_back(e0 + p); W.wcRed.push_back(W.red0[su] + c); }
                else W.wwPos.push_back(e0 + p);
            }
            W.diagPos.push_back(dp);
            W.wellFull.push_back(W.full0[su] + r);
            W.wcBeg.push_back(int(W.wcPos.size()));
            W.wwBeg.push_back(int(W.wwPos.size()));
        }
    }
    W.mask.clear();
    return true;
}

// Value-structure part: the S pattern and the maps of its values, for the nonzero set `mask` of the couplings.
bool ws_plan_values(WsPlan& W, const std::vector<unsigned char>& mask, std::string& err) {
    const int nv = W.nv, nv2 = nv * nv;
    W.mask = mask;
    W.srp.assign(size_t(W.nsys), {});
    W.sci.assign(size_t(W.nsys), {});
    W.sBase.clear();
    W.fillScalar.clear();
    W.fillBeg.assign(1, 0);
    W.tCw.clear();
    W.tDiag.clear();
    W.tWc.clear();
    W.rBeg.assign(size_t(W.red0.back()) + 1, 0);
    W.rCw.clear();
    W.rDiag.clear();
    W.rWellFull.clear();
    // active couplings per cell row (global reduced row): (J entry, global well), in row order
    std::vector<int> cBeg(size_t(W.red0.back()) + 1, 0);
    for (size_t k = 0; k < W.cplPos.size(); ++k)
        if (mask[k]) ++cBeg[size_t(W.cplRow[k]) + 1];
    for (size_t i = 0; i + 1 < cBeg.size(); ++i) cBeg[i + 1] += cBeg[i];
    std::vector<int> cPos(size_t(cBeg.back())), cWell(size_t(cBeg.back()));
    {
        std::vector<int> fillAt(cBeg.begin(), cBeg.end() - 1);
        for (size_t k = 0; k < W.cplPos.size(); ++k)
            if (mask[k]) {
                const int at = fillAt[size_t(W.cplRow[k])]++;
                cPos[size_t(at)] = W.cplPos[k];
                cWell[size_t(at)] = W.cplWell[k];
            }
    }
    // the right-hand side terms are exactly these lists
    for (size_t i = 0; i + 1 < cBeg.size(); ++i) {
        for (int t = cBeg[i]; t < cBeg[i + 1]; ++t) {
            const int w = cWell[size_t(t)];
            W.rCw.push_back(cPos[size_t(t)]);
            W.rDiag.push_back(W.diagPos[size_t(w)]);
            W.rWellFull.push_back(W.wellFull[size_t(w)]);
        }
        W.rBeg[i + 1] = int(W.rCw.size());
    }
    long long blocks = 0;
    std::vector<long long> sBlk0(size_t(W.nsys) + 1, 0);
    for (int s = 0; s < W.nsys; ++s) {
        const size_t su = size_t(s);
        const int na = W.na[su], nc = na * nv, e0 = W.jEnt0[su], red0 = W.red0[su];
        const std::vector<int>& rp = W.jrp[su];
        const std::vector<int>& ci = W.jci[su];
        // the cells of every well: block columns of its row's cell entries, sorted and unique
        std::vector<std::vector<int>> cells(size_t(W.nw[su]));
        for (int w = 0; w < W.nw[su]; ++w) {
            const int gw = W.well0[su] + w;
            auto& v = cells[size_t(w)];
            for (int q = W.wcBeg[size_t(gw)]; q < W.wcBeg[size_t(gw) + 1]; ++q) v.push_back((W.wcRed[size_t(q)] - red0) / nv);
            std::sort(v.begin(), v.end());
            v.erase(std::unique(v.begin(), v.end()), v.end());
        }
        // S row i: its own block columns, its diagonal, the cells of the wells its equations couple to
        std::vector<int>& srp = W.srp[su];
        std::vector<int>& sci = W.sci[su];
        srp.assign(size_t(na) + 1, 0);
        std::vector<int> seen(size_t(na), -1), cols;
        for (int i = 0; i < na; ++i) {
            cols.clear();
            auto add = [&](int j) { if (seen[size_t(j)] != i) { seen[size_t(j)] = i; cols.push_back(j); } };
            add(i);
            for (int e = 0; e < nv; ++e) {
                const int r = i * nv + e;
                for (int p = rp[size_t(r)]; p < rp[size_t(r) + 1]; ++p)
                    if (ci[size_t(p)] < nc) add(ci[size_t(p)] / nv);
                for (int t = cBeg[size_t(red0 + r)]; t < cBeg[size_t(red0 + r) + 1]; ++t)
                    for (int j : cells[size_t(cWell[size_t(t)] - W.well0[su])]) add(j);
            }
            std::sort(cols.begin(), cols.end());
            sci.insert(sci.end(), cols.begin(), cols.end());
            srp[size_t(i) + 1] = int(sci.size());
        }
        sBlk0[su + 1] = sBlk0[su] + (long long)sci.size();
        blocks = sBlk0[su + 1];
        // base entries and well terms of every S value, in the engine's order
        const size_t vals0 = size_t(sBlk0[su]) * size_t(nv2);
        W.sBase.resize(vals0 + sci.size() * size_t(nv2), -1);
        std::unordered_map<long long, std::vector<int>> terms;   // S value -> term ids (into the tmp lists below)
        std::vector<int> tc, td, tw;
        std::vector<long long> order;
        for (int i = 0; i < na; ++i) {
            const int b0 = srp[size_t(i)], b1 = srp[size_t(i) + 1];
            auto blockOf = [&](int j) {
                const int* lo = sci.data() + b0;
                const int* hi = sci.data() + b1;
                const int* hit = std::lower_bound(lo, hi, j);
                return int(hit - sci.data());
            };
            for (int e = 0; e < nv; ++e) {
                const int r = i * nv + e;
                for (int p = rp[size_t(r)]; p < rp[size_t(r) + 1]; ++p) {
                    const int c = ci[size_t(p)];
                    if (c >= nc) continue;
                    const size_t q = vals0 + size_t(blockOf(c / nv)) * size_t(nv2) + size_t(e * nv + c % nv);
                    if (W.sBase[q] >= 0) { err = "duplicate Jacobian entry in system " + std::to_string(s); return false; }
                    W.sBase[q] = e0 + p;
                }
                for (int t = cBeg[size_t(red0 + r)]; t < cBeg[size_t(red0 + r) + 1]; ++t) {
                    const int gw = cWell[size_t(t)];
                    for (int q = W.wcBeg[size_t(gw)]; q < W.wcBeg[size_t(gw) + 1]; ++q) {
                        const int c = W.wcRed[size_t(q)] - red0;
                        const long long v = (long long)vals0 + (long long)blockOf(c / nv) * nv2 + (e * nv + c % nv);
                        auto it = terms.find(v);
                        if (it == terms.end()) { it = terms.emplace(v, std::vector<int>()).first; order.push_back(v); }
                        it->second.push_back(int(tc.size()));
                        tc.push_back(cPos[size_t(t)]);
                        td.push_back(W.diagPos[size_t(gw)]);
                        tw.push_back(W.wcPos[size_t(q)]);
                    }
                }
            }
        }
        std::sort(order.begin(), order.end());
        for (long long v : order) {
            W.fillScalar.push_back(v);
            for (int id : terms[v]) {
                W.tCw.push_back(tc[size_t(id)]);
                W.tDiag.push_back(td[size_t(id)]);
                W.tWc.push_back(tw[size_t(id)]);
            }
            W.fillBeg.push_back(int(W.tCw.size()));
        }
    }
    W.nnzbS = blocks;
    return true;
}

// ---- launches
void launch_ws_check(const WsDev& D, const double* jv, cudaStream_t st) {
    const int n = std::max(D.ncpl, D.nwell);
    if (n > 0)
        k_ws_check<<<grid_of(n), 256, 0, st>>>(D.ncpl, D.cplPos, jv, D.mask, D.nwell, D.diagPos, D.wcBeg, D.wcPos, D.wwBeg, D.wwPos,
                                               D.wellOk);
}
void launch_ws_values(const WsDev& D, const double* jv, double* sv, cudaStream_t st) {
    k_ws_base<<<grid_of(D.nval), 256, 0, st>>>(D.nval, D.sBase, jv, sv);
    if (D.nfill > 0) k_ws_fill<<<grid_of(D.nfill), 256, 0, st>>>(D.nfill, D.fillScalar, D.fillBeg, D.tCw, D.tDiag, D.tWc, jv, sv);
}
void launch_ws_rhs(const WsDev& D, const double* jv, const double* bFull, double* bc, cudaStream_t st) {
    k_ws_rhs<<<grid_of(D.nred), 256, 0, st>>>(D.nred, D.redFull, D.rBeg, D.rCw, D.rDiag, D.rWellFull, jv, bFull, bc);
}
void launch_ws_recover(const WsDev& D, const double* jv, const double* bFull, const double* xc, double* xFull, cudaStream_t st) {
    k_ws_recover<<<grid_of(std::max(D.nred, D.nwell)), 256, 0, st>>>(D.nred, D.redFull, xc, D.nwell, D.wellFull, D.diagPos, D.wcBeg,
                                                                    D.wcPos, D.wcRed, jv, bFull, xFull);
}

}  // namespace rsg
