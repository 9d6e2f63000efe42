// Host-side, pattern-only planning of the device solve: level schedules (claim orders of the sync-free sweeps),
// BILU0 elimination lists, tiles of the tile kernels, and the well Schur complement.
#include "rsg_impl.h"

#include <algorithm>
#include <atomic>
#include <thread>
#include <cmath>
#include <cstring>
#include <numeric>

namespace rsg {

namespace {
// counting sort of rows by level, ascending row index inside a level (engine/src/bsr.cpp:286-292)
void order_by_level(const std::vector<int>& lev, int nl, std::vector<int>& ord) {
    const int n = int(lev.size());
    std::vector<int> start(size_t(nl) + 1, 0);
    for (int i = 0; i < n; ++i) start[size_t(lev[size_t(i)]) + 1]++;
    for (int l = 0; l < nl; ++l) start[size_t(l) + 1] += start[size_t(l)];
    ord.assign(size_t(n), 0);
    for (int i = 0; i < n; ++i) ord[size_t(start[size_t(lev[size_t(i)])]++)] = i;
}
}  // namespace

// Multicolour ordering of every system of a batch (MCBILU0's colouring and P A P^T, engine/src/bsr.cpp:599-653): the
// symmetric block graph of the system coloured greedily in largest-degree-first order (ties by index, as a stable
// sort leaves them; a colour is taken if none of the row's neighbours has it), rows renumbered colour by colour
// (ascending original index inside a colour), every row's entries sorted by their new column. Output: the permuted
// block-diagonal pattern, the original row of every permuted row and the original block of every permuted block.
void multicolour_batch(int nsys, const std::vector<int>& sysRow0, const std::vector<int>& rp, const std::vector<int>& ci,
                       std::vector<int>& rp2, std::vector<int>& ci2, std::vector<int>& rowOrig, std::vector<int>& blockOrig) {
    const int n = int(rp.size()) - 1;
    rp2.assign(size_t(n) + 1, 0);
    ci2.assign(ci.size(), 0);
    rowOrig.assign(size_t(n), 0);
    blockOrig.assign(ci.size(), 0);
    std::vector<int> iperm(size_t(n), 0);
    for (int s = 0; s < nsys; ++s) {
        const int r0 = sysRow0[size_t(s)], m = sysRow0[size_t(s) + 1] - r0;
        std::vector<std::vector<int>> adj(static_cast<size_t>(m));
        for (int i = 0; i < m; ++i)
            for (int p = rp[size_t(r0 + i)]; p < rp[size_t(r0 + i) + 1]; ++p) {
                const int j = ci[size_t(p)] - r0;
                if (j != i) { adj[size_t(i)].push_back(j); adj[size_t(j)].push_back(i); }
            }
        for (auto& v : adj) { std::sort(v.begin(), v.end()); v.erase(std::unique(v.begin(), v.end()), v.end()); }
        std::vector<int> order(static_cast<size_t>(m));
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return adj[size_t(a)].size() > adj[size_t(b)].size(); });
        std::vector<int> colour(static_cast<size_t>(m), -1);
        std::vector<char> taken;
        int colours = 0;
        for (int i : order) {
            const size_t deg = adj[size_t(i)].size();
            taken.assign(deg + 2, 0);
            for (int j : adj[size_t(i)]) {
                const int c = colour[size_t(j)];
                if (c >= 0 && size_t(c) < taken.size()) taken[size_t(c)] = 1;
            }
            int c = 0;
            while (taken[size_t(c)]) ++c;
            colour[size_t(i)] = c;
            colours = std::max(colours, c + 1);
        }
        std::vector<int> start(size_t(colours) + 1, 0);
        for (int i = 0; i < m; ++i) start[size_t(colour[size_t(i)]) + 1]++;
        for (int c = 0; c < colours; ++c) start[size_t(c) + 1] += start[size_t(c)];
        for (int i = 0; i < m; ++i) {
            const int k = start[size_t(colour[size_t(i)])]++;
            rowOrig[size_t(r0 + k)] = r0 + i;
            iperm[size_t(r0 + i)] = r0 + k;
        }
    }
    std::vector<std::pair<int, int>> row;
    for (int k = 0; k < n; ++k) {
        const int i = rowOrig[size_t(k)];
        row.clear();
        for (int p = rp[size_t(i)]; p < rp[size_t(i) + 1]; ++p) row.push_back({iperm[size_t(ci[size_t(p)])], p});
        std::sort(row.begin(), row.end());
        rp2[size_t(k) + 1] = rp2[size_t(k)] + int(row.size());
        int q = rp2[size_t(k)];
        for (const auto& e : row) {
            ci2[size_t(q)] = e.first;
            blockOrig[size_t(q)] = e.second;
            ++q;
        }
    }
}

bool build_plan(HostPlan& P, int nsys, const std::vector<int>& sysRow0, const std::vector<int>& rowPtr0,
                const std::vector<int>& col0, std::string& err, int threads) {
    const int n = int(rowPtr0.size()) - 1;
    if (n < 1) { err = "empty matrix (n < 1)"; return false; }
    if (rowPtr0[0] != 0) { err = "rowPtr[0] must be 0"; return false; }
    for (int i = 0; i < n; ++i)
        if (rowPtr0[size_t(i) + 1] < rowPtr0[size_t(i)]) { err = "rowPtr is not monotone"; return false; }
    const int nnzb = rowPtr0[size_t(n)];
    if (int(col0.size()) < nnzb) { err = "col shorter than rowPtr[n]"; return false; }
    P = HostPlan{};
    P.n = n; P.nnzb = nnzb; P.nsys = nsys;
    P.rowPtr0 = rowPtr0;
    P.col0.assign(col0.begin(), col0.begin() + nnzb);
    P.sysRow0 = sysRow0;
    P.rowSys.assign(size_t(n), 0);
    for (int s = 0; s < nsys; ++s)
        for (int i = sysRow0[size_t(s)]; i < sysRow0[size_t(s) + 1]; ++i) P.rowSys[size_t(i)] = s;
    // validation of the original pattern: sorted columns, in range, inside the row's own system, diagonal present
    std::vector<int> diag0(size_t(n), -1);
    for (int i = 0; i < n; ++i) {
        const int s = P.rowSys[size_t(i)];
        const int lo = sysRow0[size_t(s)], hi = sysRow0[size_t(s) + 1];
        for (int p = rowPtr0[size_t(i)]; p < rowPtr0[size_t(i) + 1]; ++p) {
            const int c = P.col0[size_t(p)];
            if (c < lo || c >= hi) { err = "column index out of range in block row " + std::to_string(i - lo); return false; }
            if (p > rowPtr0[size_t(i)] && c <= P.col0[size_t(p) - 1]) {
                err = "columns not strictly increasing in block row " + std::to_string(i - lo);
                return false;
            }
            if (c == i) diag0[size_t(i)] = p;
        }
        if (diag0[size_t(i)] < 0) { err = "missing diagonal block in block row " + std::to_string(i - lo); return false; }
    }
    // forward levels of the L dependencies (engine/src/bsr.cpp:270-293)
    std::vector<int> lev(size_t(n), 0);
    for (int i = 0; i < n; ++i) {
        int l = 0;
        for (int p = rowPtr0[size_t(i)]; p < diag0[size_t(i)]; ++p) l = std::max(l, lev[size_t(P.col0[size_t(p)])] + 1);
        lev[size_t(i)] = l;
    }
    // level space: inside every system, rows renumbered by (forward level, row); a topological order of L, so
    // ILU(0) is unchanged (the reference's level-ordered contiguous storage, engine/src/bsr.cpp:315-345). The
    // entries of a row keep their original order, so every row is eliminated / swept in the reference's order.
    P.perm.assign(size_t(n), 0);
    P.iperm.assign(size_t(n), 0);
    P.lvlStart.clear();
    P.sysLvl0.assign(size_t(nsys) + 1, 0);
    P.maxSysRows = 0;
    std::vector<int> levNew(size_t(n), 0);
    for (int s = 0; s < nsys; ++s) {
        const int r0 = sysRow0[size_t(s)], r1 = sysRow0[size_t(s) + 1];
        P.maxSysRows = std::max(P.maxSysRows, r1 - r0);
        int nls = 0;
        for (int i = r0; i < r1; ++i) nls = std::max(nls, lev[size_t(i)] + 1);
        std::vector<int> cnt(size_t(nls) + 1, 0);
        for (int i = r0; i < r1; ++i) cnt[size_t(lev[size_t(i)]) + 1]++;
        for (int l = 0; l < nls; ++l) cnt[size_t(l) + 1] += cnt[size_t(l)];
        P.sysLvl0[size_t(s)] = int(P.lvlStart.size());
        for (int l = 0; l <= nls; ++l) P.lvlStart.push_back(r0 + cnt[size_t(l)]);
        for (int i = r0; i < r1; ++i) {
            const int k = r0 + cnt[size_t(lev[size_t(i)])]++;
            P.perm[size_t(k)] = i;
            P.iperm[size_t(i)] = k;
            levNew[size_t(k)] = lev[size_t(i)];
        }
        P.nlevF = std::max(P.nlevF, nls);
    }
    P.sysLvl0[size_t(nsys)] = int(P.lvlStart.size());
    // permuted pattern (entry order inside a row preserved) and the block source map of the value gather
    P.rowPtr.assign(size_t(n) + 1, 0);
    P.col.resize(size_t(nnzb));
    P.valSrc.resize(size_t(nnzb));
    P.diag.assign(size_t(n), -1);
    for (int k = 0; k < n; ++k) {
        const int i = P.perm[size_t(k)];
        P.rowPtr[size_t(k) + 1] = P.rowPtr[size_t(k)] + (rowPtr0[size_t(i) + 1] - rowPtr0[size_t(i)]);
    }
    parallel_ranges(n, threads, [&](int lo, int hi) {
        for (int k = lo; k < hi; ++k) {
            const int i = P.perm[size_t(k)];
            int q = P.rowPtr[size_t(k)];
            for (int p = rowPtr0[size_t(i)]; p < rowPtr0[size_t(i) + 1]; ++p, ++q) {
                P.col[size_t(q)] = P.iperm[size_t(P.col0[size_t(p)])];
                P.valSrc[size_t(q)] = p;
                if (p == diag0[size_t(i)]) P.diag[size_t(k)] = q;
            }
        }
    });
    // structural symmetry (then the reversed forward levels are a topological order of the U dependencies)
    {
        std::atomic<bool> sym{true};
        parallel_ranges(n, threads, [&](int lo, int hi) {
            for (int i = lo; i < hi && sym.load(std::memory_order_relaxed); ++i)
                for (int p = rowPtr0[size_t(i)]; p < rowPtr0[size_t(i) + 1]; ++p) {
                    const int j = P.col0[size_t(p)];
                    const int* c0 = P.col0.data() + rowPtr0[size_t(j)];
                    const int* c1 = P.col0.data() + rowPtr0[size_t(j) + 1];
                    if (!std::binary_search(c0, c1, i)) { sym.store(false, std::memory_order_relaxed); break; }
                }
        });
        P.symmetric = sym.load();
    }
    // claim orders of the grid-wide sync-free kernels: all systems' rows by forward level
    order_by_level(levNew, P.nlevF, P.ford);
    if (P.symmetric) {
        P.bord.assign(P.ford.rbegin(), P.ford.rend());
        P.nlevB = P.nlevF;
    } else {
        std::vector<int> blev(size_t(n), 0);
        int nb = 0;
        for (int i = n - 1; i >= 0; --i) {                 // original order: U entries point to larger rows
            int l = 0;
            for (int p = diag0[size_t(i)] + 1; p < rowPtr0[size_t(i) + 1]; ++p) l = std::max(l, blev[size_t(P.col0[size_t(p)])] + 1);
            blev[size_t(i)] = l;
            nb = std::max(nb, l + 1);
        }
        std::vector<int> blevNew(size_t(n), 0);
        for (int k = 0; k < n; ++k) blevNew[size_t(k)] = blev[size_t(P.perm[size_t(k)])];
        P.nlevB = nb;
        order_by_level(blevNew, nb, P.bord);
    }
    // BILU0 elimination lists (engine/src/bsr.cpp:193-201): lower entries in row order, the U entries of the
    // eliminating row in row order, target = the block of row i in the same column
    // (rows in parallel: the pairs of every entry counted, then written at their places)
    P.elimPtr.assign(size_t(nnzb) + 1, 0);
    auto elim_rows = [&](int lo, int hi, bool write) {
        std::vector<int> pos(size_t(n), -1);
        for (int i = lo; i < hi; ++i) {
            const int r0 = P.rowPtr[size_t(i)], r1 = P.rowPtr[size_t(i) + 1];
            for (int p = r0; p < r1; ++p) pos[size_t(P.col[size_t(p)])] = p;
            for (int p = r0; p < P.diag[size_t(i)]; ++p) {
                const int k = P.col[size_t(p)];
                int c = write ? P.elimPtr[size_t(p)] : 0;
                for (int q = P.diag[size_t(k)] + 1; q < P.rowPtr[size_t(k) + 1]; ++q) {
                    const int t = pos[size_t(P.col[size_t(q)])];
                    if (t < 0) continue;
                    if (write) { P.elimT[size_t(c)] = t; P.elimQ[size_t(c)] = q; }
                    ++c;
                }
                if (!write) P.elimPtr[size_t(p) + 1] = c;
            }
            for (int p = r0; p < r1; ++p) pos[size_t(P.col[size_t(p)])] = -1;
        }
    };
    parallel_ranges(n, threads, [&](int lo, int hi) { elim_rows(lo, hi, false); });
    for (int p = 0; p < nnzb; ++p) P.elimPtr[size_t(p) + 1] += P.elimPtr[size_t(p)];
    P.elimT.assign(size_t(P.elimPtr[size_t(nnzb)]), 0);
    P.elimQ.assign(size_t(P.elimPtr[size_t(nnzb)]), 0);
    parallel_ranges(n, threads, [&](int lo, int hi) { elim_rows(lo, hi, true); });
    // tiles of TILE_ROWS block rows, never crossing a system boundary
    P.tileRow0.clear(); P.tileSys.clear(); P.sysTile0.assign(size_t(nsys) + 1, 0);
    for (int s = 0; s < nsys; ++s) {
        P.sysTile0[size_t(s)] = int(P.tileSys.size());
        for (int r = sysRow0[size_t(s)]; r < sysRow0[size_t(s) + 1]; r += TILE_ROWS) {
            P.tileRow0.push_back(r);
            P.tileSys.push_back(s);
        }
    }
    P.sysTile0[size_t(nsys)] = int(P.tileSys.size());
    P.tileRow0.push_back(n);
    // slot storage of the thread-block sweeps (rows of a level contiguous; columns local to the system)
    P.Lslot.assign(size_t(n) * 4, -1);
    P.Uslot.assign(size_t(n) * 4, -1);
    P.LslotSrc.assign(size_t(n) * SLOTS, -1);
    P.UslotSrc.assign(size_t(n) * SLOTS, -1);
    P.Dsrc.assign(size_t(n), 0);
    P.LovCol.clear(); P.LovSrc.clear(); P.UovCol.clear(); P.UovSrc.clear();
    auto fill = [&](int k, int p0, int p1, int base, std::vector<int>& slot, std::vector<int>& slotSrc, std::vector<int>& ovCol,
                    std::vector<int>& ovSrc) {
        for (int p = p0, j = 0; p < p1; ++p, ++j) {
            if (j < SLOTS) {
                slot[size_t(k) * 4 + size_t(j)] = P.col[size_t(p)] - base;
                slotSrc[size_t(k) * SLOTS + size_t(j)] = p;
            } else {
                if (j == SLOTS) slot[size_t(k) * 4 + 3] = int(ovCol.size());
                ovCol.push_back(P.col[size_t(p)] - base);
                ovSrc.push_back(p);
                if (p + 1 == p1) { ovCol.push_back(-1); ovSrc.push_back(-1); }
            }
        }
    };
    for (int k = 0; k < n; ++k) {
        const int base = sysRow0[size_t(P.rowSys[size_t(k)])];
        fill(k, P.rowPtr[size_t(k)], P.diag[size_t(k)], base, P.Lslot, P.LslotSrc, P.LovCol, P.LovSrc);
        fill(k, P.diag[size_t(k)] + 1, P.rowPtr[size_t(k) + 1], base, P.Uslot, P.UslotSrc, P.UovCol, P.UovSrc);
        P.Dsrc[size_t(k)] = P.diag[size_t(k)];
    }
    for (auto* v : {&P.LovCol, &P.LovSrc, &P.UovCol, &P.UovSrc})
        if (!v->empty()) v->insert(v->end(), size_t(OV_CHUNK - 1), -1);
    return true;
}

namespace {
// One system of a batch against the plan: its row starts relative to the system, its columns relative to the
// system's first row. Branch-free chunks (the compiler vectorises them) with an exit between chunks.
bool same_system(const HostPlan& P, int s, int ns, const int* rp, const int* c) {
    constexpr int CH = 4096;
    const int r0 = P.sysRow0[size_t(s)];
    const int base = P.rowPtr0[size_t(r0)];
    const int* prp = P.rowPtr0.data() + r0;
    for (int i0 = 0; i0 <= ns; i0 += CH) {
        const int i1 = std::min(ns + 1, i0 + CH);
        int diff = 0;
        for (int i = i0; i < i1; ++i) diff |= (prp[i] - base) ^ rp[i];
        if (diff) return false;
    }
    const int* pc = P.col0.data() + base;
    const int m = rp[ns];
    for (int p0 = 0; p0 < m; p0 += CH) {
        const int p1 = std::min(m, p0 + CH);
        int diff = 0;
        for (int p = p0; p < p1; ++p) diff |= (pc[p] - r0) ^ c[p];
        if (diff) return false;
    }
    return true;
}
}  // namespace

bool same_batch_pattern(const HostPlan& P, int nsys, const int* n, const int* const* rowPtr, const int* const* col) {
    if (P.nsys != nsys || int(P.sysRow0.size()) != nsys + 1) return false;
    for (int s = 0; s < nsys; ++s)
        if (P.sysRow0[size_t(s) + 1] - P.sysRow0[size_t(s)] != n[s]) return false;
    // large batches: the systems are compared on several threads (independent, read-only)
    const int hw = int(std::max(1u, std::thread::hardware_concurrency()));
    const int T = P.col0.size() > (size_t(1) << 20) ? std::min({8, hw, nsys}) : 1;
    std::atomic<bool> ok{true};
    std::atomic<int> next{0};
    auto work = [&] {
        for (int s = next++; s < nsys && ok.load(std::memory_order_relaxed); s = next++)
            if (!same_system(P, s, n[s], rowPtr[s], col[s])) ok = false;
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < T; ++t) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    return ok;
}

// ====================================================================== well Schur complement
namespace {
struct WellParts {
    std::vector<double> dInv;
    std::vector<int> wcPtr, wcCol;
    std::vector<double> wcVal;
    std::vector<int> cwPtr, cwWell;
    std::vector<double> cwVal;
};
// well rows (diagonal + cell couplings) and the well columns of the cell rows (engine/src/bsr.cpp:737-757)
bool well_parts(WellParts& W, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw, std::string& err) {
    const int nc = na * nv;
    W.dInv.assign(size_t(nw), 0.0);
    W.wcPtr.assign(size_t(nw) + 1, 0);
    for (int w = 0; w < nw; ++w) {
        const int r = nc + w;
        double d = 0, rowMax = 0;
        for (int p = rowPtr[r]; p < rowPtr[r + 1]; ++p) {
            const int c = col[p];
            if (c == r) d = val[p];
            else if (c < nc) { W.wcCol.push_back(c); W.wcVal.push_back(val[p]); rowMax = std::max(rowMax, std::fabs(val[p])); }
            else if (val[p] != 0.0) { err = "well-well coupling in well row " + std::to_string(w) + " (not supported)"; return false; }
        }
        if (!(std::fabs(d) > 1e-12 * std::max(rowMax, 1e-300)) || !std::isfinite(d)) {
            err = "well row " + std::to_string(w) + " has no usable BHP derivative";
            return false;
        }
        W.dInv[size_t(w)] = 1.0 / d;
        W.wcPtr[size_t(w) + 1] = int(W.wcCol.size());
    }
    W.cwPtr.assign(size_t(nc) + 1, 0);
    for (int r = 0; r < nc; ++r) {
        for (int p = rowPtr[r]; p < rowPtr[r + 1]; ++p)
            if (col[p] >= nc && val[p] != 0.0) { W.cwWell.push_back(col[p] - nc); W.cwVal.push_back(val[p]); }
        W.cwPtr[size_t(r) + 1] = int(W.cwWell.size());
    }
    return true;
}
}  // namespace

int wellschur_reduce(int nrows, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw,
                     const double* b, int* nnzb, int* sRowPtr, int* sCol, double* sVal, double* bc, std::string& err) {
    if (na < 1 || nv < 1 || nw < 0 || nrows != na * nv + nw) { err = "wellschur: nrows must equal na*nv + nw"; return -1; }
    WellParts W;
    if (!well_parts(W, rowPtr, col, val, na, nv, nw, err)) return -1;
    const int nc = na * nv, b2 = nv * nv;
    std::vector<std::vector<int>> wellCells(static_cast<size_t>(nw));
    for (int w = 0; w < nw; ++w) {
        auto& v = wellCells[size_t(w)];
        for (int p = W.wcPtr[size_t(w)]; p < W.wcPtr[size_t(w) + 1]; ++p) v.push_back(W.wcCol[size_t(p)] / nv);
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
    }
    // block pattern: cell pattern + couplings through shared wells (engine/src/bsr.cpp:785-807)
    std::vector<int> rp(size_t(na) + 1, 0), cols_all, mark(size_t(na), -1), cols, wl;
    for (int i = 0; i < na; ++i) {
        cols.clear(); wl.clear();
        for (int e = 0; e < nv; ++e) {
            const int r = i * nv + e;
            for (int p = rowPtr[r]; p < rowPtr[r + 1]; ++p) {
                const int c = col[p];
                if (c < nc) { const int j = c / nv; if (mark[size_t(j)] != i) { mark[size_t(j)] = i; cols.push_back(j); } }
            }
            for (int p = W.cwPtr[size_t(r)]; p < W.cwPtr[size_t(r) + 1]; ++p) wl.push_back(W.cwWell[size_t(p)]);
        }
        if (mark[size_t(i)] != i) { mark[size_t(i)] = i; cols.push_back(i); }
        std::sort(wl.begin(), wl.end());
        wl.erase(std::unique(wl.begin(), wl.end()), wl.end());
        for (int w : wl)
            for (int j : wellCells[size_t(w)])
                if (mark[size_t(j)] != i) { mark[size_t(j)] = i; cols.push_back(j); }
        std::sort(cols.begin(), cols.end());
        cols_all.insert(cols_all.end(), cols.begin(), cols.end());
        rp[size_t(i) + 1] = int(cols_all.size());
    }
    *nnzb = int(cols_all.size());
    if (!sRowPtr) return 0;
    std::memcpy(sRowPtr, rp.data(), sizeof(int) * rp.size());
    std::memcpy(sCol, cols_all.data(), sizeof(int) * cols_all.size());
    std::memset(sVal, 0, sizeof(double) * cols_all.size() * size_t(b2));
    // values S = Acc - Acw Dww^-1 Awc, in the reference's order of operations (engine/src/bsr.cpp:813-830)
    std::vector<int> pos(size_t(na), -1);
    for (int i = 0; i < na; ++i) {
        for (int p = rp[size_t(i)]; p < rp[size_t(i) + 1]; ++p) pos[size_t(cols_all[size_t(p)])] = p;
        for (int e = 0; e < nv; ++e) {
            const int r = i * nv + e;
            for (int p = rowPtr[r]; p < rowPtr[r + 1]; ++p) {
                const int c = col[p];
                if (c < nc) sVal[size_t(pos[size_t(c / nv)]) * b2 + size_t(e * nv + c % nv)] += val[p];
            }
            for (int p = W.cwPtr[size_t(r)]; p < W.cwPtr[size_t(r) + 1]; ++p) {
                const int w = W.cwWell[size_t(p)];
                const double f = W.cwVal[size_t(p)] * W.dInv[size_t(w)];
                for (int q = W.wcPtr[size_t(w)]; q < W.wcPtr[size_t(w) + 1]; ++q) {
                    const int c = W.wcCol[size_t(q)];
                    sVal[size_t(pos[size_t(c / nv)]) * b2 + size_t(e * nv + c % nv)] -= f * W.wcVal[size_t(q)];
                }
            }
        }
    }
    // bc = b_c - Acw Dww^-1 b_w (engine/src/bsr.cpp:973-980)
    if (b && bc)
        for (int r = 0; r < nc; ++r) {
            double s = b[r];
            for (int p = W.cwPtr[size_t(r)]; p < W.cwPtr[size_t(r) + 1]; ++p)
                s -= W.cwVal[size_t(p)] * W.dInv[size_t(W.cwWell[size_t(p)])] * b[nc + W.cwWell[size_t(p)]];
            bc[r] = s;
        }
    return 0;
}

int wellschur_recover(int nrows, const int* rowPtr, const int* col, const double* val, int na, int nv, int nw,
                      const double* b, const double* xc, double* x, std::string& err) {
    if (na < 1 || nv < 1 || nw < 0 || nrows != na * nv + nw) { err = "wellschur: nrows must equal na*nv + nw"; return -1; }
    WellParts W;
    if (!well_parts(W, rowPtr, col, val, na, nv, nw, err)) return -1;
    const int nc = na * nv;
    if (x != xc) std::memcpy(x, xc, sizeof(double) * size_t(nc));
    for (int w = 0; w < nw; ++w) {
        double s = b[nc + w];
        for (int p = W.wcPtr[size_t(w)]; p < W.wcPtr[size_t(w) + 1]; ++p) s -= W.wcVal[size_t(p)] * xc[W.wcCol[size_t(p)]];
        x[nc + w] = s * W.dInv[size_t(w)];
    }
    return 0;
}

}  // namespace rsg

// Diagnostics: whether a batch (b) has the pattern of the plan built from another batch (a), as rsg_set_batch decides
// it (1 same, 0 different, -1 batch a rejected). Host code only.
extern "C" int rsg_debug_same_pattern(int nsys, const int* na, const int* const* rpa, const int* const* cia, int nsysB, const int* nb,
                                      const int* const* rpb, const int* const* cib) {
    using namespace rsg;
    std::vector<int> sysRow0(size_t(nsys) + 1, 0), rp, ci;
    for (int s = 0; s < nsys; ++s) sysRow0[size_t(s) + 1] = sysRow0[size_t(s)] + na[s];
    rp.assign(size_t(sysRow0[size_t(nsys)]) + 1, 0);
    for (int s = 0; s < nsys; ++s) {
        const int r0 = sysRow0[size_t(s)];
        for (int i = 0; i < na[s]; ++i) {
            rp[size_t(r0 + i) + 1] = rp[size_t(r0)] + rpa[s][i + 1];
            for (int p = rpa[s][i]; p < rpa[s][i + 1]; ++p) ci.push_back(cia[s][p] + r0);
        }
    }
    HostPlan P;
    std::string err;
    if (!build_plan(P, nsys, sysRow0, rp, ci, err)) return -1;
    return same_batch_pattern(P, nsysB, nb, rpb, cib) ? 1 : 0;
}
