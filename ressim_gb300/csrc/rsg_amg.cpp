// Host planning of the CPR pressure AMG (engine/src/amg.cpp:137-295): aggregation in the reference's natural
// numbering, then every level mapped to its own "level space" for the device (rows renumbered by forward
// Gauss-Seidel level, entries of a row in their natural order), together with the gather lists that let the
// device recompute the Galerkin operators in the reference's summation order (AMG::refresh, amg.cpp:257-271).
#include "rsg_impl.h"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <thread>

namespace rsg {

namespace {

struct Csr {
    int n = 0;
    std::vector<int> rp, ci;
    std::vector<double> v;
};

std::vector<int> diag_of(const Csr& A) {
    std::vector<int> d(size_t(A.n), -1);
    for (int i = 0; i < A.n; ++i)
        for (int p = A.rp[size_t(i)]; p < A.rp[size_t(i) + 1]; ++p)
            if (A.ci[size_t(p)] == i) { d[size_t(i)] = p; break; }
    return d;
}

// reference aggregation of one level (engine/src/amg.cpp:150-201); returns the number of aggregates
int aggregate(const Csr& A, const std::vector<int>& dg, std::vector<int>& agg, int threads) {
    const int n = A.n;
    const double kTheta = 0.08, kRowTheta = 0.25;
    // strong connections: flagged per entry (rows in parallel), then compacted in row order
    std::vector<unsigned char> strong(A.ci.size(), 0);
    std::vector<int> sp(size_t(n) + 1, 0), sc;
    parallel_ranges(n, threads, [&](int lo, int hi) {
        for (int i = lo; i < hi; ++i) {
            double rowMax = 0;
            for (int p = A.rp[size_t(i)]; p < A.rp[size_t(i) + 1]; ++p)
                if (A.ci[size_t(p)] != i) rowMax = std::max(rowMax, std::fabs(A.v[size_t(p)]));
            const double di = A.v[size_t(dg[size_t(i)])];
            int c = 0;
            for (int p = A.rp[size_t(i)]; p < A.rp[size_t(i) + 1]; ++p) {
                const int j = A.ci[size_t(p)];
                if (j == i) continue;
                const double dj = A.v[size_t(dg[size_t(j)])];
                if (std::fabs(A.v[size_t(p)]) >= kTheta * std::sqrt(std::fabs(di * dj)) || std::fabs(A.v[size_t(p)]) >= kRowTheta * rowMax) {
                    strong[size_t(p)] = 1;
                    ++c;
                }
            }
            sp[size_t(i) + 1] = c;
        }
    });
    for (int i = 0; i < n; ++i) sp[size_t(i) + 1] += sp[size_t(i)];
    sc.resize(size_t(sp[size_t(n)]));
    parallel_ranges(n, threads, [&](int lo, int hi) {
        for (int i = lo; i < hi; ++i) {
            int q = sp[size_t(i)];
            for (int p = A.rp[size_t(i)]; p < A.rp[size_t(i) + 1]; ++p)
                if (strong[size_t(p)]) sc[size_t(q++)] = A.ci[size_t(p)];
        }
    });
    agg.assign(size_t(n), -1);
    int na = 0;
    for (int i = 0; i < n; ++i) {                       // pass 1: roots with free strong neighbourhoods
        if (agg[size_t(i)] >= 0) continue;
        bool fr = true;
        for (int p = sp[size_t(i)]; p < sp[size_t(i) + 1]; ++p)
            if (agg[size_t(sc[size_t(p)])] >= 0) { fr = false; break; }
        if (!fr || sp[size_t(i)] == sp[size_t(i) + 1]) continue;
        agg[size_t(i)] = na;
        for (int p = sp[size_t(i)]; p < sp[size_t(i) + 1]; ++p) agg[size_t(sc[size_t(p)])] = na;
        ++na;
    }
    const std::vector<int> agg1 = agg;
    for (int i = 0; i < n; ++i) {                       // pass 2: join the most strongly coupled pass-1 aggregate
        if (agg[size_t(i)] >= 0) continue;
        double best = 0;
        int ba = -1;
        for (int p = A.rp[size_t(i)]; p < A.rp[size_t(i) + 1]; ++p) {
            const int j = A.ci[size_t(p)];
            if (j != i && agg1[size_t(j)] >= 0 && std::fabs(A.v[size_t(p)]) > best) { best = std::fabs(A.v[size_t(p)]); ba = agg1[size_t(j)]; }
        }
        if (ba >= 0 && sp[size_t(i)] != sp[size_t(i) + 1]) agg[size_t(i)] = ba;
    }
    for (int i = 0; i < n; ++i) {                       // pass 3: leftovers start new aggregates
        if (agg[size_t(i)] >= 0) continue;
        agg[size_t(i)] = na;
        for (int p = sp[size_t(i)]; p < sp[size_t(i) + 1]; ++p)
            if (agg[size_t(sc[size_t(p)])] < 0) agg[size_t(sc[size_t(p)])] = na;
        ++na;
    }
    return na;
}

// Galerkin A_c = P^T A P for an aggregation P, in the reference's order (engine/src/amg.cpp:37-70): AP(i, J) sums
// row i's entries of aggregate column J in row order; A_c(I, J) sums AP(i, J) over the members i of I in ascending
// order. Also returns the two gather lists (positions in A for AP, AP entries for A_c).
struct Galerkin {
    Csr AP, Ac;
    std::vector<int> apPtr, apSrc;   // AP entry -> A positions
    std::vector<int> acPtr, acSrc;   // A_c entry -> AP entries
};
// One output row of a sparse product in the reference's order. The row's contributions arrive in order as
// (column J, value, source); take() sums the values of each J in arrival order, then emit() writes the columns in
// ascending J with their sums and, per column, the sources in arrival order. The buffers live across rows (the
// plan of a large system has millions of rows).
struct RowAccumulator {
    std::vector<int> mark;                      // J -> slot in this row, -1 outside
    std::vector<std::pair<int, int>> cols;      // (J, slot) in first-appearance order
    std::vector<double> vals;                   // per slot
    std::vector<int> srcSlot, src;              // arrivals: slot and source
    std::vector<int> rank, off;                 // per slot: position of its column, first output source
    explicit RowAccumulator(int ncols) : mark(size_t(ncols), -1) {}
    void take(int J, double v, int source) {
        int& m = mark[size_t(J)];
        if (m < 0) { m = int(cols.size()); cols.push_back({J, m}); vals.push_back(v); }
        else vals[size_t(m)] += v;
        srcSlot.push_back(m);
        src.push_back(source);
    }
    // cols sorted by J; sources bucketed by slot, arrival order kept within a bucket
    template <class Emit>
    void emit(std::vector<int>& outSrc, Emit&& emitCol) {
        for (auto& c : cols) mark[size_t(c.first)] = -1;
        const size_t ns = cols.size();
        if (ns <= 32) {                          // a row's few columns (distinct J): insertion sort
            for (size_t a = 1; a < ns; ++a) {
                const std::pair<int, int> c = cols[a];
                size_t b = a;
                for (; b > 0 && cols[b - 1].first > c.first; --b) cols[b] = cols[b - 1];
                cols[b] = c;
            }
        } else {
            std::sort(cols.begin(), cols.end());
        }
        if (rank.size() < ns) rank.resize(ns);
        if (off.size() < ns + 1) off.resize(ns + 1);
        std::fill(off.begin(), off.begin() + long(ns) + 1, 0);
        for (size_t r = 0; r < ns; ++r) rank[size_t(cols[r].second)] = int(r);
        for (int sl : srcSlot) off[size_t(rank[size_t(sl)]) + 1]++;
        for (size_t r = 0; r < ns; ++r) off[r + 1] += off[r];
        const size_t base = outSrc.size();
        outSrc.resize(base + src.size());
        std::vector<int>& pos = rank;           // reused: next free place per column
        for (size_t r = 0; r < ns; ++r) pos[size_t(cols[r].second)] = off[r];
        for (size_t q = 0; q < src.size(); ++q) outSrc[base + size_t(pos[size_t(srcSlot[q])]++)] = src[q];
        for (size_t r = 0; r < ns; ++r) emitCol(cols[r].first, vals[size_t(cols[r].second)], int(base) + off[r + 1]);
        cols.clear(); vals.clear(); srcSlot.clear(); src.clear();
    }
};

// Output rows [lo, hi) of one product, formed by one worker with its own accumulator: the rows' columns and sums,
// their row ends, and per entry the end of its source list, all local to the piece (joined in row order after).
struct ProductPiece {
    std::vector<int> rowEnd{0}, ci, ptr{0}, src;   // rowEnd and ptr open with the piece's start (0)
    std::vector<double> v;
};

// Runs row(w, k, piece) for k in [0, nrows) in `threads` contiguous pieces, piece w on worker w (one thread each;
// 1: the caller's thread), and joins them: out.rp, out.ci, out.v, ptr (entry -> end of its source list, ptr[0] = 0)
// and src. Each row is formed exactly as a serial pass would form it, so the result does not depend on the number
// of pieces. sources(lo, hi): the number of sources rows [lo, hi) take (their entries are at most that plus one per
// row), to size the pieces' buffers once.
template <class Row, class Sources>
void product_rows(int nrows, int threads, Csr& out, std::vector<int>& ptr, std::vector<int>& src, Row&& row, Sources&& sources) {
    const int np = std::max(1, std::min(threads, nrows));
    std::vector<ProductPiece> pc(static_cast<size_t>(np));
    auto bounds = [&](int w) { return std::make_pair(int((long long)nrows * w / np), int((long long)nrows * (w + 1) / np)); };
    auto work = [&](int w) {
        const auto [lo, hi] = bounds(w);
        ProductPiece& q = pc[size_t(w)];
        const size_t ns = sources(lo, hi);
        q.rowEnd.reserve(size_t(hi - lo) + 1);
        q.src.reserve(ns);
        q.ci.reserve(ns + size_t(hi - lo));
        q.v.reserve(ns + size_t(hi - lo));
        q.ptr.reserve(ns + size_t(hi - lo) + 1);
        for (int k = lo; k < hi; ++k) {
            row(w, k, q);
            q.rowEnd.push_back(int(q.ci.size()));
        }
    };
    out.n = nrows;
    if (np == 1) {                                   // one piece: it is the result
        work(0);
        ProductPiece& q = pc[0];
        out.rp = std::move(q.rowEnd);
        out.ci = std::move(q.ci);
        out.v = std::move(q.v);
        ptr = std::move(q.ptr);
        src = std::move(q.src);
        return;
    }
    std::vector<std::thread> pool;
    for (int w = 0; w < np; ++w) {
        try {
            pool.emplace_back(work, w);
        } catch (const std::system_error&) {     // no thread to be had: this piece on the caller's thread
            work(w);
        }
    }
    for (auto& t : pool) t.join();
    std::vector<size_t> e0(size_t(np) + 1, 0), s0(size_t(np) + 1, 0);
    for (int w = 0; w < np; ++w) {
        e0[size_t(w) + 1] = e0[size_t(w)] + pc[size_t(w)].ci.size();
        s0[size_t(w) + 1] = s0[size_t(w)] + pc[size_t(w)].src.size();
    }
    out.rp.resize(size_t(nrows) + 1);
    out.ci.resize(e0[size_t(np)]);
    out.v.resize(e0[size_t(np)]);
    ptr.resize(e0[size_t(np)] + 1);
    src.resize(s0[size_t(np)]);
    out.rp[0] = 0;
    ptr[0] = 0;
    parallel_ranges(np, np, [&](int w0, int w1) {    // each piece copied to its place, offsets added
        for (int w = w0; w < w1; ++w) {
            const ProductPiece& q = pc[size_t(w)];
            const int lo = bounds(w).first;
            const int eb = int(e0[size_t(w)]), sb = int(s0[size_t(w)]);
            for (size_t r = 1; r < q.rowEnd.size(); ++r) out.rp[size_t(lo) + r] = eb + q.rowEnd[r];
            std::copy(q.ci.begin(), q.ci.end(), out.ci.begin() + eb);
            std::copy(q.v.begin(), q.v.end(), out.v.begin() + eb);
            for (size_t e = 1; e < q.ptr.size(); ++e) ptr[size_t(eb) + e] = sb + q.ptr[e];
            std::copy(q.src.begin(), q.src.end(), src.begin() + sb);
        }
    }, 1);
}

// threads: workers for the two products (rows split into contiguous pieces; the result is the same for any count)
void galerkin(const Csr& A, const std::vector<int>& agg, int na, Galerkin& G, int threads) {
    const int n = A.n;
    const int nth = std::max(1, std::min(n >= 65536 ? threads : 1, n));   // small levels: a thread costs more than it saves
    std::vector<RowAccumulator> accs;
    accs.reserve(size_t(nth));
    for (int w = 0; w < nth; ++w) accs.emplace_back(na);
    // AP = A P: row i sums its entries of each aggregate column in row order
    product_rows(n, nth, G.AP, G.apPtr, G.apSrc, [&](int w, int i, ProductPiece& q) {
        RowAccumulator& acc = accs[size_t(w)];
        for (int p = A.rp[size_t(i)]; p < A.rp[size_t(i) + 1]; ++p) acc.take(agg[size_t(A.ci[size_t(p)])], A.v[size_t(p)], p);
        acc.emit(q.src, [&](int J, double v, int end) { q.ci.push_back(J); q.v.push_back(v); q.ptr.push_back(end); });
    }, [&](int lo, int hi) { return size_t(A.rp[size_t(hi)] - A.rp[size_t(lo)]); });
    const Csr& AP = G.AP;
    // members of every aggregate in ascending row order (the rows of R = P^T)
    std::vector<int> mPtr(size_t(na) + 1, 0), mem(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i) mPtr[size_t(agg[size_t(i)]) + 1]++;
    for (int I = 0; I < na; ++I) mPtr[size_t(I) + 1] += mPtr[size_t(I)];
    {
        std::vector<int> fill(mPtr.begin(), mPtr.end() - 1);
        for (int i = 0; i < n; ++i) mem[size_t(fill[size_t(agg[size_t(i)])]++)] = i;
    }
    // A_c = R AP: row I sums the AP rows of its members in ascending order; a row whose columns skip I gets an
    // explicit zero diagonal (engine/src/amg.cpp:83-91)
    product_rows(na, nth, G.Ac, G.acPtr, G.acSrc, [&](int w, int I, ProductPiece& q) {
        RowAccumulator& acc = accs[size_t(w)];
        for (int m = mPtr[size_t(I)]; m < mPtr[size_t(I) + 1]; ++m) {
            const int i = mem[size_t(m)];
            for (int e = AP.rp[size_t(i)]; e < AP.rp[size_t(i) + 1]; ++e) acc.take(AP.ci[size_t(e)], AP.v[size_t(e)], e);
        }
        bool haveDiag = false;
        acc.emit(q.src, [&](int J, double v, int end) {
            if (!haveDiag && J > I) {                      // an empty source list: ends where the previous entry's does
                q.ci.push_back(I); q.v.push_back(0.0); q.ptr.push_back(q.ptr.back()); haveDiag = true;
            }
            if (J == I) haveDiag = true;
            q.ci.push_back(J);
            q.v.push_back(v);
            q.ptr.push_back(end);
        });
        if (!haveDiag) { q.ci.push_back(I); q.v.push_back(0.0); q.ptr.push_back(int(q.src.size())); }
    }, [&](int lo, int hi) {
        size_t c = 0;
        for (int m = mPtr[size_t(lo)]; m < mPtr[size_t(hi)]; ++m) c += size_t(AP.rp[size_t(mem[size_t(m)]) + 1] - AP.rp[size_t(mem[size_t(m)])]);
        return c;
    });
}

void fix_diag(Csr& A, const std::vector<int>& dg) {
    for (int i = 0; i < A.n; ++i)
        if (std::fabs(A.v[size_t(dg[size_t(i)])]) < 1e-300) A.v[size_t(dg[size_t(i)])] = 1.0;
}

// forward Gauss-Seidel levels of a natural-order CSR and the level-space renumbering of its rows
void gs_levels(const Csr& A, const std::vector<int>& dg, std::vector<int>& perm, std::vector<int>& iperm, std::vector<int>& lvlStart) {
    const int n = A.n;
    std::vector<int> lev(size_t(n), 0);
    int nl = 0;
    for (int i = 0; i < n; ++i) {
        int l = 0;
        for (int p = A.rp[size_t(i)]; p < dg[size_t(i)]; ++p) l = std::max(l, lev[size_t(A.ci[size_t(p)])] + 1);
        lev[size_t(i)] = l;
        nl = std::max(nl, l + 1);
    }
    std::vector<int> cnt(size_t(nl) + 1, 0);
    for (int i = 0; i < n; ++i) cnt[size_t(lev[size_t(i)]) + 1]++;
    for (int l = 0; l < nl; ++l) cnt[size_t(l) + 1] += cnt[size_t(l)];
    lvlStart = cnt;
    perm.assign(size_t(n), 0);
    iperm.assign(size_t(n), 0);
    for (int i = 0; i < n; ++i) {
        const int k = cnt[size_t(lev[size_t(i)])]++;
        perm[size_t(k)] = i;
        iperm[size_t(i)] = k;
    }
}

}  // namespace

// Builds the hierarchy of one system. ap0: values of the fine pressure matrix in the system's LEVEL-SPACE block
// order (positions [bp0, bp1) of the block pattern); the level-space pattern and its original numbering come from
// the solver plan. Levels l >= 1 are expressed in their own level space.
bool amg_plan_system(const HostPlan& P, int s, const std::vector<double>& ap0, SysAmg& out, std::string& err, int threads) {
    const int r0 = P.sysRow0[size_t(s)], r1 = P.sysRow0[size_t(s) + 1], n0 = r1 - r0;
    const int b0 = P.rowPtr[size_t(r0)];
    // natural-order fine matrix (original numbering of this system)
    Csr A;
    A.n = n0;
    A.rp.assign(size_t(n0) + 1, 0);
    const size_t nnz0 = size_t(P.rowPtr[size_t(r1)] - b0);
    for (int io = 0; io < n0; ++io) {
        const int k = P.iperm[size_t(r0 + io)];
        A.rp[size_t(io) + 1] = A.rp[size_t(io)] + (P.rowPtr[size_t(k) + 1] - P.rowPtr[size_t(k)]);
    }
    A.ci.resize(nnz0);
    A.v.resize(nnz0);
    std::vector<int> natPos(nnz0);               // natural position -> level-space position (relative to b0)
    parallel_ranges(n0, threads, [&](int lo, int hi) {
        for (int io = lo; io < hi; ++io) {
            const int k = P.iperm[size_t(r0 + io)];
            int q = A.rp[size_t(io)];
            for (int p = P.rowPtr[size_t(k)]; p < P.rowPtr[size_t(k) + 1]; ++p, ++q) {
                A.ci[size_t(q)] = P.perm[size_t(P.col[size_t(p)])] - r0;
                A.v[size_t(q)] = ap0[size_t(p - b0)];
                natPos[size_t(q)] = p - b0;
            }
        }
    });
    std::vector<int> dg = diag_of(A);
    for (int i = 0; i < n0; ++i)
        if (dg[size_t(i)] < 0) { err = "pressure matrix without a diagonal entry"; return false; }
    fix_diag(A, dg);
    out = SysAmg{};
    // level 0 lives in the solver's level space (its GS levels are the BILU0 forward levels)
    {
        AmgLevel L0;
        L0.n = n0;
        L0.rp.resize(size_t(n0) + 1);
        L0.ci.resize(nnz0);
        L0.diag.resize(size_t(n0));
        for (int k = r0; k <= r1; ++k) L0.rp[size_t(k - r0)] = P.rowPtr[size_t(k)] - b0;
        for (int k = r0; k < r1; ++k) L0.diag[size_t(k - r0)] = P.diag[size_t(k)] - b0;
        parallel_ranges(int(nnz0), threads, [&](int lo, int hi) {
            for (int q = lo; q < hi; ++q) L0.ci[size_t(q)] = P.col[size_t(b0 + q)] - r0;
        });
        for (int q = P.sysLvl0[size_t(s)]; q < P.sysLvl0[size_t(s) + 1]; ++q) L0.lvlStart.push_back(P.lvlStart[size_t(q)] - r0);
        L0.perm.resize(size_t(n0));
        L0.iperm.resize(size_t(n0));
        for (int k = 0; k < n0; ++k) { L0.perm[size_t(k)] = P.perm[size_t(r0 + k)] - r0; L0.iperm[size_t(L0.perm[size_t(k)])] = k; }
        L0.val.assign(ap0.begin(), ap0.end());
        for (int k = 0; k < n0; ++k)                                     // tiny diagonals -> 1 (engine/src/amg.cpp:145)
            if (std::fabs(L0.val[size_t(L0.diag[size_t(k)])]) < 1e-300) L0.val[size_t(L0.diag[size_t(k)])] = 1.0;
        out.lv.push_back(std::move(L0));
    }
    std::vector<int> natToLev0 = std::move(natPos);   // natural position -> level-space position of the current level
    Csr cur = std::move(A);
    std::vector<int> curDiag = std::move(dg);
    while (true) {
        if (cur.n <= 400 || int(out.lv.size()) >= 14) break;          // engine/src/amg.cpp:153
        std::vector<int> agg;
        const int na = aggregate(cur, curDiag, agg, threads);
        if (na >= int(0.85 * cur.n) || na < 1) break;                   // coarsening stalled
        Galerkin G;
        galerkin(cur, agg, na, G, threads);
        std::vector<int> cd = diag_of(G.Ac);
        fix_diag(G.Ac, cd);
        AmgLevel& F = out.lv.back();                                    // finer level (level space)
        AmgLevel C;
        C.n = na;
        gs_levels(G.Ac, cd, C.perm, C.iperm, C.lvlStart);
        // coarse level-space CSR (entries in natural order), values, diagonal positions
        std::vector<int> cNat2Lev(G.Ac.ci.size());
        C.rp.assign(size_t(na) + 1, 0);
        C.ci.reserve(G.Ac.ci.size());
        C.val.reserve(G.Ac.ci.size());
        C.diag.reserve(size_t(na));
        for (int k = 0; k < na; ++k) {
            const int I = C.perm[size_t(k)];
            for (int p = G.Ac.rp[size_t(I)]; p < G.Ac.rp[size_t(I) + 1]; ++p) {
                cNat2Lev[size_t(p)] = int(C.ci.size());
                if (p == cd[size_t(I)]) C.diag.push_back(int(C.ci.size()));
                C.ci.push_back(C.iperm[size_t(G.Ac.ci[size_t(p)])]);
                C.val.push_back(G.Ac.v[size_t(p)]);
            }
            C.rp[size_t(k) + 1] = int(C.ci.size());
        }
        // transfer: fine level-space row -> coarse level-space row; members of each coarse row in ascending
        // natural fine order (restriction order)
        F.agg.assign(size_t(cur.n), 0);
        for (int kf = 0; kf < cur.n; ++kf) F.agg[size_t(kf)] = C.iperm[size_t(agg[size_t(F.perm[size_t(kf)])])];
        C.memPtr.assign(size_t(na) + 1, 0);
        for (int i = 0; i < cur.n; ++i) C.memPtr[size_t(C.iperm[size_t(agg[size_t(i)])]) + 1]++;
        for (int k = 0; k < na; ++k) C.memPtr[size_t(k) + 1] += C.memPtr[size_t(k)];
        C.mem.assign(size_t(cur.n), 0);
        {
            std::vector<int> fill(C.memPtr.begin(), C.memPtr.end() - 1);
            for (int i = 0; i < cur.n; ++i) C.mem[size_t(fill[size_t(C.iperm[size_t(agg[size_t(i)])])]++)] = F.iperm[size_t(i)];
        }
        // Galerkin gathers in level-space positions: AP entries (natural) <- finer level-space positions;
        // coarse level-space entries <- AP entries
        C.apPtr = std::move(G.apPtr);
        C.apSrc.resize(G.apSrc.size());
        parallel_ranges(int(G.apSrc.size()), threads, [&](int lo, int hi) {
            for (int q = lo; q < hi; ++q) C.apSrc[size_t(q)] = natToLev0[size_t(G.apSrc[size_t(q)])];
        });
        C.acPtr.assign(G.Ac.ci.size() + 1, 0);
        C.acSrc.clear();
        C.acSrc.reserve(G.acSrc.size());
        {
            std::vector<int> order(G.Ac.ci.size());
            for (size_t p = 0; p < order.size(); ++p) order[size_t(cNat2Lev[p])] = int(p);
            for (size_t e = 0; e < order.size(); ++e) {
                const int p = order[e];
                for (int q = G.acPtr[size_t(p)]; q < G.acPtr[size_t(p) + 1]; ++q) C.acSrc.push_back(G.acSrc[size_t(q)]);
                C.acPtr[e + 1] = int(C.acSrc.size());
            }
        }
        natToLev0 = std::move(cNat2Lev);
        cur = std::move(G.Ac);
        curDiag = std::move(cd);
        out.lv.push_back(std::move(C));
    }
    out.coarseDense = cur.n <= 800;
    return true;
}

}  // namespace rsg

namespace rsg {
void set_last_error(const std::string& msg);
}

// Diagnostics: the AMG hierarchy the plan builds for a single BSR system and pressure-matrix values (original block
// order), reported in each level's natural numbering. Level l: rows[l], nnz[l]; if l == which: its CSR (rp, ci, v)
// and, for which == 0 and a coarser level present, the aggregate of every fine row.
extern "C" int rsg_debug_amg_plan(int n, const int* rowPtr, const int* col, const double* ap, int which, int* levels, int* rows,
                                  int* nnz, int maxLevels, int* rp, int* ci, double* v, int* agg) {
    using namespace rsg;
    std::vector<int> rp0(rowPtr, rowPtr + n + 1), ci0(col, col + rowPtr[n]), s0 = {0, n};
    HostPlan P;
    std::string err;
    if (!build_plan(P, 1, s0, rp0, ci0, err)) { set_last_error(err); return -1; }
    std::vector<double> ap0(size_t(P.nnzb));
    for (int p = 0; p < P.nnzb; ++p) ap0[size_t(p)] = ap[P.valSrc[size_t(p)]];
    SysAmg H;
    if (!amg_plan_system(P, 0, ap0, H, err)) { set_last_error(err); return -1; }
    *levels = int(H.lv.size());
    for (int l = 0; l < int(H.lv.size()) && l < maxLevels; ++l) { rows[l] = H.lv[size_t(l)].n; nnz[l] = int(H.lv[size_t(l)].ci.size()); }
    if (which >= 0 && which < int(H.lv.size())) {
        const AmgLevel& L = H.lv[size_t(which)];
        int c = 0;
        rp[0] = 0;
        for (int I = 0; I < L.n; ++I) {
            const int k = L.iperm[size_t(I)];
            for (int p = L.rp[size_t(k)]; p < L.rp[size_t(k) + 1]; ++p, ++c) { ci[c] = L.perm[size_t(L.ci[size_t(p)])]; v[c] = L.val[size_t(p)]; }
            rp[I + 1] = c;
        }
        if (agg && which + 1 < int(H.lv.size())) {
            const AmgLevel& C = H.lv[size_t(which) + 1];
            for (int i = 0; i < L.n; ++i) agg[i] = C.perm[size_t(L.agg[size_t(L.iperm[size_t(i)])])];
        }
    }
    return 0;
}

namespace {
// FNV-1a over the bytes of a plan's arrays and sizes
struct Digest {
    unsigned long long h = 1469598103934665603ULL;
    void bytes(const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        for (size_t i = 0; i < n; ++i) { h ^= b[i]; h *= 1099511628211ULL; }
    }
    void num(long long x) { bytes(&x, sizeof x); }
    template <class T> void vec(const std::vector<T>& v) { num((long long)v.size()); bytes(v.data(), v.size() * sizeof(T)); }
};
}  // namespace

// Diagnostics: digests of the whole solver plan (every array of the pattern plan) and of the whole AMG plan of one
// system, built with `threads` host threads -- the plans must not depend on the thread count.
extern "C" int rsg_debug_plan_digest(int n, const int* rowPtr, const int* col, const double* ap, int threads,
                                     unsigned long long* planDigest, unsigned long long* amgDigest) {
    using namespace rsg;
    std::vector<int> rp0(rowPtr, rowPtr + n + 1), ci0(col, col + rowPtr[n]), s0 = {0, n};
    HostPlan P;
    std::string err;
    if (!build_plan(P, 1, s0, rp0, ci0, err, threads)) { set_last_error(err); return -1; }
    Digest d;
    for (long long x : {(long long)P.n, (long long)P.nnzb, (long long)P.nsys, (long long)P.nlevF, (long long)P.nlevB,
                        (long long)P.symmetric, (long long)P.maxSysRows})
        d.num(x);
    for (const std::vector<int>* v : {&P.rowPtr0, &P.col0, &P.perm, &P.iperm, &P.valSrc, &P.rowPtr, &P.col, &P.diag, &P.ford,
                                      &P.bord, &P.elimPtr, &P.elimT, &P.elimQ, &P.rowSys, &P.sysRow0, &P.tileRow0, &P.tileSys,
                                      &P.sysTile0, &P.lvlStart, &P.sysLvl0, &P.Lslot, &P.LslotSrc, &P.LovCol, &P.LovSrc, &P.Uslot,
                                      &P.UslotSrc, &P.UovCol, &P.UovSrc, &P.Dsrc})
        d.vec(*v);
    *planDigest = d.h;
    std::vector<double> ap0(size_t(P.nnzb));
    for (int p = 0; p < P.nnzb; ++p) ap0[size_t(p)] = ap[P.valSrc[size_t(p)]];
    SysAmg H;
    if (!amg_plan_system(P, 0, ap0, H, err, threads)) { set_last_error(err); return -1; }
    Digest a;
    a.num(H.coarseDense ? 1 : 0);
    a.num((long long)H.lv.size());
    for (const AmgLevel& L : H.lv) {
        a.num(L.n);
        for (const std::vector<int>* v : {&L.rp, &L.ci, &L.diag, &L.lvlStart, &L.perm, &L.iperm, &L.agg, &L.memPtr, &L.mem, &L.apPtr,
                                          &L.apSrc, &L.acPtr, &L.acSrc})
            a.vec(*v);
        a.vec(L.val);
    }
    *amgDigest = a.h;
    return 0;
}
