// Restarted flexible GMRES(m) of a batch of systems on the device (engine/src/linsolve.cpp:218-273).
//
// All systems of the batch step in lockstep: a restart cycle runs inner steps j = 0, 1, ... with the per-system
// Hessenberg matrix, Givens rotations and right-hand side g resident on the device; a system whose cycle ends
// (convergence, m steps or the iteration limit) is frozen by its status until the cycle-end update x += Z y.
// Every inner product is reduced per tile and then per system in a fixed order (deterministic). Vector arithmetic
// follows the reference's loop order with explicitly rounded operations:
//   r = b - A x, V_0 = r / beta; Z_j = M V_j; w = A Z_j; for i <= j: h_ij = <w, V_i>, w -= h_ij V_i (MGS);
//   h_{j+1,j} = ||w||, V_{j+1} = w / h_{j+1,j}; Givens on column j; rel = |g_{j+1}| / ||b||;
//   cycle end: y = H^-1 g (back substitution), x += sum_i y_i Z_i.
#include "rsg_impl.h"
#include "rsg_block3.cuh"
#include "rsg_reduce.cuh"

#include <cuda_runtime.h>

namespace rsg {

namespace {

// component e of (A x) for block row `row` (engine/src/bsr.cpp:109-117 order)
__device__ __forceinline__ double spmv_comp(const int* __restrict__ rowPtr, const int* __restrict__ col, const double* __restrict__ val,
                                            const double* x, int row, int e) {
    double yv = 0;
    const int p1 = __ldg(rowPtr + row + 1);
    for (int p = __ldg(rowPtr + row); p < p1; ++p) {
        const double* a = val + size_t(p) * 9 + e * 3;
        const double* xc = x + size_t(__ldg(col + p)) * 3;
        yv = da(yv, da(da(dm(__ldg(a), xc[0]), dm(__ldg(a + 1), xc[1])), dm(__ldg(a + 2), xc[2])));
    }
    return yv;
}

struct Tiles {
    int ntiles, nsys;
    const int *tileRow0, *tileSys, *sysTile0;
};
__device__ __forceinline__ double* gm_H(double* H, int s, int m) { return H + size_t(s) * gm_stride(m); }

// x = 0 and ||b|| for the (re)started systems; their scalars reset
__global__ void __launch_bounds__(kTileThreads) k_gm_init(Tiles T, const double* __restrict__ b, double* x, KScal* ks, double tol, int maxit,
                                                         int onlyFailed, double* part, unsigned* done, double* sysdot, int* active) {
    __shared__ double sh[MAX_DOTS * kTileThreads];
    const int tile = blockIdx.x, s = __ldg(T.tileSys + tile);
    const bool restart = !onlyFailed || ks[s].status != ST_CONV;
    double acc[MAX_DOTS] = {0, 0, 0, 0};
    if (restart) {
        const size_t q0 = size_t(__ldg(T.tileRow0 + tile)) * 3, q1 = size_t(__ldg(T.tileRow0 + tile + 1)) * 3;
        for (size_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
            const double bq = __ldg(b + q);
            x[q] = 0;
            acc[0] += bq * bq;
        }
    }
    block_reduce<1>(acc, sh);
    if (threadIdx.x == 0) part[size_t(tile) * MAX_DOTS] = acc[0];
    if (!last_tile_reduce<1>(T.ntiles, T.nsys, T.sysTile0, part, done, sysdot, sh)) return;
    if (threadIdx.x == 0) *active = 0;
    __syncthreads();
    int nact = 0;
    for (int q = threadIdx.x; q < T.nsys; q += blockDim.x) {
        KScal& K = ks[q];
        if (onlyFailed && K.status == ST_CONV) continue;
        const double bb = sysdot[size_t(q) * MAX_DOTS];
        K.bn = sqrt(bb);
        K.tol = tol; K.maxit = maxit; K.its = 0; K.relres = 0; K.gj = 0; K.gend = 0; K.hn = 0;
        if (K.bn == 0) { K.status = ST_CONV; }                       // engine/src/linsolve.cpp:223
        else if (!isfinite(bb)) { K.status = ST_BREAKDOWN; }
        else if (maxit < 1) { K.status = ST_MAXIT; }
        else { K.status = ST_RUNNING; ++nact; }
    }
    if (nact) atomicAdd(active, nact);
}

// cycle start: r = b - A x into V_0 and ||r||; tests; g = beta e_1
__global__ void __launch_bounds__(kTileThreads) k_gm_resid(Tiles T, const int* __restrict__ rowPtr, const int* __restrict__ col,
                                                          const double* __restrict__ val, const double* __restrict__ b, const double* x,
                                                          double* V0, KScal* ks, double* H, int m, double* part, unsigned* done,
                                                          double* sysdot, int* active, int* inner) {
    __shared__ double sh[MAX_DOTS * kTileThreads];
    const int tile = blockIdx.x, s = __ldg(T.tileSys + tile);
    double acc[MAX_DOTS] = {0, 0, 0, 0};
    if (ks[s].status == ST_RUNNING) {
        const int r0 = __ldg(T.tileRow0 + tile), r1 = __ldg(T.tileRow0 + tile + 1);
        const int e = threadIdx.x % 3;
        for (int row = r0 + int(threadIdx.x) / 3; row < r1; row += kTileThreads / 3) {
            const size_t q = size_t(row) * 3 + e;
            const double rq = ds(__ldg(b + q), spmv_comp(rowPtr, col, val, x, row, e));
            V0[q] = rq;
            acc[0] += rq * rq;
        }
    }
    block_reduce<1>(acc, sh);
    if (threadIdx.x == 0) part[size_t(tile) * MAX_DOTS] = acc[0];
    if (!last_tile_reduce<1>(T.ntiles, T.nsys, T.sysTile0, part, done, sysdot, sh)) return;
    if (threadIdx.x == 0) *inner = 0;
    __syncthreads();
    int nin = 0;
    for (int q = threadIdx.x; q < T.nsys; q += blockDim.x) {
        KScal& K = ks[q];
        if (K.status != ST_RUNNING) continue;
        const double beta = sqrt(sysdot[size_t(q) * MAX_DOTS]);
        const double rel = beta / K.bn;
        K.relres = rel;
        if (rel < K.tol) { K.status = ST_CONV; atomicSub(active, 1); continue; }   // linsolve.cpp:232-236
        if (!isfinite(beta)) { K.status = ST_BREAKDOWN; atomicSub(active, 1); continue; }
        K.beta = beta;
        K.gj = 0; K.gend = 0;
        double* g = gm_H(H, q, m) + size_t(m + 1) * m + 2 * size_t(m);
        g[0] = beta;
        for (int i = 1; i <= m; ++i) g[i] = 0;
        ++nin;
    }
    if (nin) atomicAdd(inner, nin);
}

// dst = src / (beta or h_{j+1,j}) for the systems in the inner loop (V_0, V_{j+1})
__global__ void __launch_bounds__(kTileThreads) k_gm_scale(Tiles T, const double* src, double* dst, const KScal* ks, int useHn) {
    const int tile = blockIdx.x, s = __ldg(T.tileSys + tile);
    const KScal& K = ks[s];
    if (K.status != ST_RUNNING) return;
    const double d = useHn ? K.hn : K.beta;
    if (!(d > 0)) return;                                            // linsolve.cpp:249: V_{j+1} kept when h = 0
    const size_t q0 = size_t(__ldg(T.tileRow0 + tile)) * 3, q1 = size_t(__ldg(T.tileRow0 + tile + 1)) * 3;
    for (size_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) dst[q] = __ddiv_rn(src[q], d);
}

// w = A Z_j and <w, V_0> -> h_0j
__global__ void __launch_bounds__(kTileThreads) k_gm_av(Tiles T, const int* __restrict__ rowPtr, const int* __restrict__ col,
                                                       const double* __restrict__ val, const double* z, const double* v0, double* w,
                                                       const KScal* ks, double* H, int m, int j, double* part, unsigned* done,
                                                       double* sysdot) {
    __shared__ double sh[MAX_DOTS * kTileThreads];
    const int tile = blockIdx.x, s = __ldg(T.tileSys + tile);
    double acc[MAX_DOTS] = {0, 0, 0, 0};
    if (ks[s].status == ST_RUNNING) {
        const int r0 = __ldg(T.tileRow0 + tile), r1 = __ldg(T.tileRow0 + tile + 1);
        const int e = threadIdx.x % 3;
        for (int row = r0 + int(threadIdx.x) / 3; row < r1; row += kTileThreads / 3) {
            const size_t q = size_t(row) * 3 + e;
            const double wq = spmv_comp(rowPtr, col, val, z, row, e);
            w[q] = wq;
            acc[0] += wq * v0[q];
        }
    }
    block_reduce<1>(acc, sh);
    if (threadIdx.x == 0) part[size_t(tile) * MAX_DOTS] = acc[0];
    if (!last_tile_reduce<1>(T.ntiles, T.nsys, T.sysTile0, part, done, sysdot, sh)) return;
    for (int q = threadIdx.x; q < T.nsys; q += blockDim.x)
        if (ks[q].status == ST_RUNNING) gm_H(H, q, m)[size_t(0) * m + j] = sysdot[size_t(q) * MAX_DOTS];
}

// MGS step i of column j: w -= h_{i-1,j} V_{i-1}, then <w, V_i> -> h_ij (linsolve.cpp:241-245)
__global__ void __launch_bounds__(kTileThreads) k_gm_mgs(Tiles T, const double* vprev, const double* vi, double* w, const KScal* ks,
                                                        double* H, int m, int i, int j, double* part, unsigned* done, double* sysdot) {
    __shared__ double sh[MAX_DOTS * kTileThreads];
    const int tile = blockIdx.x, s = __ldg(T.tileSys + tile);
    double acc[MAX_DOTS] = {0, 0, 0, 0};
    if (ks[s].status == ST_RUNNING) {
        const double hh = gm_H(H, s, m)[size_t(i - 1) * m + j];
        const size_t q0 = size_t(__ldg(T.tileRow0 + tile)) * 3, q1 = size_t(__ldg(T.tileRow0 + tile + 1)) * 3;
        for (size_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
            const double wq = ds(w[q], dm(hh, vprev[q]));
            w[q] = wq;
            acc[0] += wq * vi[q];
        }
    }
    block_reduce<1>(acc, sh);
    if (threadIdx.x == 0) part[size_t(tile) * MAX_DOTS] = acc[0];
    if (!last_tile_reduce<1>(T.ntiles, T.nsys, T.sysTile0, part, done, sysdot, sh)) return;
    for (int q = threadIdx.x; q < T.nsys; q += blockDim.x)
        if (ks[q].status == ST_RUNNING) gm_H(H, q, m)[size_t(i) * m + j] = sysdot[size_t(q) * MAX_DOTS];
}

// last MGS update w -= h_jj V_j, ||w|| -> h_{j+1,j}; Givens rotations, g, residual estimate, cycle-end tests
// (linsolve.cpp:246-264)
__global__ void __launch_bounds__(kTileThreads) k_gm_norm(Tiles T, const double* vj, double* w, KScal* ks, double* H, int m, int j,
                                                         double* part, unsigned* done, double* sysdot, int* active, int* inner) {
    __shared__ double sh[MAX_DOTS * kTileThreads];
    const int tile = blockIdx.x, s = __ldg(T.tileSys + tile);
    double acc[MAX_DOTS] = {0, 0, 0, 0};
    if (ks[s].status == ST_RUNNING) {
        const double hh = gm_H(H, s, m)[size_t(j) * m + j];
        const size_t q0 = size_t(__ldg(T.tileRow0 + tile)) * 3, q1 = size_t(__ldg(T.tileRow0 + tile + 1)) * 3;
        for (size_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
            const double wq = ds(w[q], dm(hh, vj[q]));
            w[q] = wq;
            acc[0] += wq * wq;
        }
    }
    block_reduce<1>(acc, sh);
    if (threadIdx.x == 0) part[size_t(tile) * MAX_DOTS] = acc[0];
    if (!last_tile_reduce<1>(T.ntiles, T.nsys, T.sysTile0, part, done, sysdot, sh)) return;
    for (int q = threadIdx.x; q < T.nsys; q += blockDim.x) {
        KScal& K = ks[q];
        if (K.status != ST_RUNNING) continue;
        double* Hs = gm_H(H, q, m);
        double* cs = Hs + size_t(m + 1) * m;
        double* sn = cs + m;
        double* g = sn + m;
        const double hn = sqrt(sysdot[size_t(q) * MAX_DOTS]);
        K.hn = hn;
        Hs[size_t(j + 1) * m + j] = hn;
        for (int i = 0; i < j; ++i) {
            const double a = Hs[size_t(i) * m + j], c = Hs[size_t(i + 1) * m + j];
            const double t = da(dm(cs[i], a), dm(sn[i], c));
            Hs[size_t(i + 1) * m + j] = da(dm(-sn[i], a), dm(cs[i], c));
            Hs[size_t(i) * m + j] = t;
        }
        const double hjj = Hs[size_t(j) * m + j], hj1 = Hs[size_t(j + 1) * m + j];
        const double den = hypot(hjj, hj1);
        cs[j] = den > 0 ? __ddiv_rn(hjj, den) : 1.0;
        sn[j] = den > 0 ? __ddiv_rn(hj1, den) : 0.0;
        Hs[size_t(j) * m + j] = den;
        Hs[size_t(j + 1) * m + j] = 0;
        g[j + 1] = dm(-sn[j], g[j]);
        g[j] = dm(cs[j], g[j]);
        const double rel = fabs(g[j + 1]) / K.bn;
        K.relres = rel;
        K.its += 1;
        K.gj = j + 1;
        if (!isfinite(hn) || !isfinite(rel)) {
            K.status = ST_BREAKDOWN;
            atomicSub(active, 1);
            atomicSub(inner, 1);
        } else if (rel < K.tol) {
            K.status = ST_CYCLE; K.gend = 1;
            atomicSub(inner, 1);
        } else if (j + 1 == m || K.its >= K.maxit) {
            K.status = ST_CYCLE; K.gend = 0;
            atomicSub(inner, 1);
        }
    }
}

// y = H^-1 g by back substitution over the cycle's steps (linsolve.cpp:265-269), one thread per system
__global__ void k_gm_solve(int nsys, const KScal* ks, double* H, int m) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nsys || ks[q].status != ST_CYCLE) return;
    double* Hs = gm_H(H, q, m);
    const double* g = Hs + size_t(m + 1) * m + 2 * size_t(m);
    double* y = Hs + size_t(m + 1) * m + 3 * size_t(m) + 1;
    const int jn = ks[q].gj;
    for (int i = jn - 1; i >= 0; --i) {
        double s = g[i];
        for (int k = i + 1; k < jn; ++k) s = ds(s, dm(Hs[size_t(i) * m + k], y[k]));
        y[i] = __ddiv_rn(s, Hs[size_t(i) * m + i]);
    }
}

// x += sum_i y_i Z_i, each entry in ascending i (linsolve.cpp:270-271)
__global__ void __launch_bounds__(kTileThreads) k_gm_xupd(Tiles T, double* x, const double* Z, size_t N, const KScal* ks, const double* H,
                                                         int m) {
    const int tile = blockIdx.x, s = __ldg(T.tileSys + tile);
    if (ks[s].status != ST_CYCLE) return;
    const double* y = H + size_t(s) * gm_stride(m) + size_t(m + 1) * m + 3 * size_t(m) + 1;
    const int jn = ks[s].gj;
    const size_t q0 = size_t(__ldg(T.tileRow0 + tile)) * 3, q1 = size_t(__ldg(T.tileRow0 + tile + 1)) * 3;
    for (size_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
        double xq = x[q];
        for (int i = 0; i < jn; ++i) xq = da(xq, dm(y[i], Z[size_t(i) * N + q]));
        x[q] = xq;
    }
}

// converged (linsolve.cpp:272), iteration limit, or restart
__global__ void k_gm_status(int nsys, KScal* ks, int* active) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nsys) return;
    KScal& K = ks[q];
    if (K.status != ST_CYCLE) return;
    if (K.gend) { K.status = ST_CONV; atomicSub(active, 1); }
    else if (K.its >= K.maxit) { K.status = ST_MAXIT; atomicSub(active, 1); }
    else K.status = ST_RUNNING;
}

// the fallback keeps the GMRES result only where its recursive residual is smaller (engine/src/simulator.cpp:3397)
__global__ void __launch_bounds__(kTileThreads) k_gm_pick_x(Tiles T, double* x, const double* xPrev, const KScal* ksPrev, const KScal* ks) {
    const int tile = blockIdx.x, s = __ldg(T.tileSys + tile);
    if (ksPrev[s].status == ST_CONV) return;                         // not retried
    if (ks[s].relres < ksPrev[s].relres) return;                     // GMRES better: keep
    const size_t q0 = size_t(__ldg(T.tileRow0 + tile)) * 3, q1 = size_t(__ldg(T.tileRow0 + tile + 1)) * 3;
    for (size_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) x[q] = xPrev[q];
}
__global__ void k_gm_pick_scal(int nsys, const KScal* ksPrev, KScal* ks) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nsys || ksPrev[q].status == ST_CONV) return;
    const int its = ksPrev[q].its + ks[q].its;                       // both solves count (simulator.cpp:3396)
    if (!(ks[q].relres < ksPrev[q].relres)) ks[q] = ksPrev[q];
    ks[q].its = its;
}

Tiles tiles_of(const DevPlan& P) { return Tiles{P.ntiles, P.nsys, P.tileRow0, P.tileSys, P.sysTile0}; }

}  // namespace

void launch_gm_init(const DevPlan& P, const double* b, double* x, KScal* ks, ReduceState& R, double tol, int maxit, bool onlyFailed,
                    int* active, cudaStream_t st) {
    k_gm_init<<<P.ntiles, kTileThreads, 0, st>>>(tiles_of(P), b, x, ks, tol, maxit, onlyFailed ? 1 : 0, R.part, R.done, R.sysdot, active);
}

void launch_gm_cycle_start(const DevPlan& P, const double* val, const double* b, const double* x, GmState& G, KScal* ks, ReduceState& R,
                           int* active, cudaStream_t st) {
    const Tiles T = tiles_of(P);
    k_gm_resid<<<P.ntiles, kTileThreads, 0, st>>>(T, P.rowPtr, P.col, val, b, x, G.V, ks, G.H, G.m, R.part, R.done, R.sysdot, active,
                                                   G.inner);
    k_gm_scale<<<P.ntiles, kTileThreads, 0, st>>>(T, G.V, G.V, ks, 0);
}

void launch_gm_step(const DevPlan& P, const double* val, int j, GmState& G, KScal* ks, ReduceState& R, int* active, cudaStream_t st) {
    const Tiles T = tiles_of(P);
    const size_t N = size_t(P.n) * 3;
    k_gm_av<<<P.ntiles, kTileThreads, 0, st>>>(T, P.rowPtr, P.col, val, G.Z + size_t(j) * N, G.V, G.w, ks, G.H, G.m, j, R.part, R.done,
                                                R.sysdot);
    for (int i = 1; i <= j; ++i)
        k_gm_mgs<<<P.ntiles, kTileThreads, 0, st>>>(T, G.V + size_t(i - 1) * N, G.V + size_t(i) * N, G.w, ks, G.H, G.m, i, j, R.part,
                                                     R.done, R.sysdot);
    k_gm_norm<<<P.ntiles, kTileThreads, 0, st>>>(T, G.V + size_t(j) * N, G.w, ks, G.H, G.m, j, R.part, R.done, R.sysdot, active,
                                                  G.inner);
    k_gm_scale<<<P.ntiles, kTileThreads, 0, st>>>(T, G.w, G.V + size_t(j + 1) * N, ks, 1);
}

void launch_gm_cycle_end(const DevPlan& P, double* x, GmState& G, KScal* ks, int* active, cudaStream_t st) {
    const int g = (P.nsys + 127) / 128;
    k_gm_solve<<<g, 128, 0, st>>>(P.nsys, ks, G.H, G.m);
    k_gm_xupd<<<P.ntiles, kTileThreads, 0, st>>>(tiles_of(P), x, G.Z, size_t(P.n) * 3, ks, G.H, G.m);
    k_gm_status<<<g, 128, 0, st>>>(P.nsys, ks, active);
}

void launch_gm_pick(const DevPlan& P, double* x, const double* xPrev, const KScal* ksPrev, KScal* ks, cudaStream_t st) {
    k_gm_pick_x<<<P.ntiles, kTileThreads, 0, st>>>(tiles_of(P), x, xPrev, ksPrev, ks);
    k_gm_pick_scal<<<(P.nsys + 127) / 128, 128, 0, st>>>(P.nsys, ksPrev, ks);
}

void launch_precond_gm(const DevPlan& P, const PrecDev& M, const double* r, double* z, const KScal* ks, SweepState& S, int* err,
                       cudaStream_t st) {
    if (M.devcpr) launch_devcpr(P, *M.amg, M.val, 0, r, nullptr, nullptr, z, ks, st);
    else if (M.cpr && M.cta && !M.split) launch_cpr_cta(P, M, *M.amg, 0, M.kind != 0, r, nullptr, nullptr, z, ks, st);
    else if (M.cpr) launch_cpr_grid(P, M, *M.amg, 0, r, nullptr, nullptr, z, ks, S, err, st);
    else if (M.cta) launch_ilu_cta_apply_ks(P, M, r, z, ks, st);
    else if (M.kind == 0) launch_ilu_apply_f64(P, M.lu, r, z, S, err, st);
    else if (M.kind == 1) launch_ilu_apply_mixed(P, M.luf, r, z, S, err, st);
    else if (M.kind == 3) launch_ilu_apply_f32(P, M.luf, r, z, M.yt, S, err, st);
    else launch_block_jacobi_apply(P, M.dinv, r, z, st);
}

}  // namespace rsg
