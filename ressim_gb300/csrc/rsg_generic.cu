// Block-size-generic solve path (nb x nb blocks, 1 <= nb <= 16): SpMV, BILU0 factorisation and sweeps, BlockCPR
// (weights, pressure matrix, aggregation-AMG V-cycle, second stage) and BiCGSTAB / GMRES(m), one system per handle,
// FP64.
//
// Layout: the matrix stays in the caller's block order (rowPtr, col, nb*nb row-major blocks); the factors overwrite a
// copy of it. Dependent row sets run level by level: the forward levels of the L pattern (the factorisation and the
// forward sweep) and the backward levels of U (the backward sweep), computed on the host once per pattern as the
// reference does (engine/src/bsr.cpp:270-300). A system whose level sweeps fit one thread block runs each sweep in
// one launch (a barrier per level); larger ones launch once per level.
//
// Rows of nb values are handled by nb consecutive threads (SpMV, sweeps, CPR stages: one thread per row element, each
// computing the reference's sum for that element in its order); the factorisation and the block inversions take a
// warp per row, its lanes over block elements and, in the Gauss-Jordan inversion, over the 2 nb columns of [A | I].
// The CPR pressure AMG reuses the library's host aggregation plan (bit for bit the reference's hierarchy) and
// recomputes every level's values on the device at each set-up from its Galerkin gather lists.
#include "rsg_generic.h"
#include "rsg_impl.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

namespace rsg {
void set_last_error(const std::string& msg);

namespace {

#define GEN_CUDA(x)                                                                                    \
    do {                                                                                               \
        cudaError_t e_ = (x);                                                                          \
        if (e_ != cudaSuccess) return gfail(RSG_ECUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
    } while (0)

int gfail(int code, const std::string& msg) {
    set_last_error(msg);
    return code;
}

// separately rounded FP64 operations: the reference's arithmetic without contraction into fused multiply-adds
__device__ __forceinline__ double gm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ga(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double gs(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double gd(double a, double b) { return __ddiv_rn(a, b); }

constexpr int kCtaThreads = 1024;   // one-block level sweeps
constexpr int kWarpsPerBlock = 4;   // factorisation / weights: a warp per row (8 KB of shared memory each)

// ------------------------------------------------------------------ SpMV: y = S x (engine/src/bsr.cpp:109-126)
__global__ void k_gen_spmv(int n, int nb, const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ val,
                           const double* __restrict__ x, double* __restrict__ y) {
    const int b2 = nb * nb;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (long long)n * nb; q += (long long)gridDim.x * blockDim.x) {
        const int i = int(q / nb), e = int(q % nb);
        double yi = 0;
        for (int p = rp[i]; p < rp[i + 1]; ++p) {
            const double* a = val + size_t(p) * b2 + size_t(e) * nb;
            const double* xc = x + size_t(ci[p]) * nb;
            double s = 0;
            for (int f = 0; f < nb; ++f) s = ga(s, gm(a[f], xc[f]));
            yi = ga(yi, s);
        }
        y[q] = yi;
    }
}

// ------------------------------------------------------------------ warp Gauss-Jordan (invertBlock, bsr.cpp:67-87)
// m: this warp's nb x 2 nb work matrix in shared memory (row stride 2 * GEN_MAX_NB). Lane j < 2 nb owns column j.
// Returns (to every lane) whether the block was invertible; on success a[] holds the inverse.
__device__ bool warp_invert(double* m, double* a, int nb) {
    const int lane = int(threadIdx.x & 31);
    constexpr int RS = 2 * GEN_MAX_NB;
    double sc = 0;
    for (int t = lane; t < nb * nb; t += 32) sc = fmax(sc, fabs(a[t]));
    for (int o = 16; o > 0; o >>= 1) sc = fmax(sc, __shfl_xor_sync(0xffffffffu, sc, o));
    if (lane < 2 * nb)
        for (int i = 0; i < nb; ++i) m[i * RS + lane] = lane < nb ? a[i * nb + lane] : (lane - nb == i ? 1.0 : 0.0);
    __syncwarp();
    if (!(sc > 0) || !isfinite(sc)) return false;
    const double thr = gm(1e-14, sc);
    for (int k = 0; k < nb; ++k) {
        int pr = k;
        for (int i = k + 1; i < nb; ++i)
            if (fabs(m[i * RS + k]) > fabs(m[pr * RS + k])) pr = i;
        if (fabs(m[pr * RS + k]) <= thr) return false;   // every lane decides the same
        if (pr != k && lane < 2 * nb) {
            const double t = m[k * RS + lane];
            m[k * RS + lane] = m[pr * RS + lane];
            m[pr * RS + lane] = t;
        }
        __syncwarp();
        const double inv = gd(1.0, m[k * RS + k]);
        __syncwarp();
        if (lane < 2 * nb) m[k * RS + lane] = gm(m[k * RS + lane], inv);
        __syncwarp();
        double f[GEN_MAX_NB];
#pragma unroll
        for (int i = 0; i < GEN_MAX_NB; ++i) f[i] = i < nb ? m[i * RS + k] : 0.0;
        __syncwarp();
        if (lane < 2 * nb) {
            const double mk = m[k * RS + lane];
#pragma unroll
            for (int i = 0; i < GEN_MAX_NB; ++i)
                if (i < nb && i != k && f[i] != 0.0) m[i * RS + lane] = gs(m[i * RS + lane], gm(f[i], mk));
        }
        __syncwarp();
    }
    if (lane < nb)
        for (int i = 0; i < nb; ++i) a[i * nb + lane] = m[i * RS + nb + lane];
    __syncwarp();
    return true;
}

// the pivot block of a factored row: inverse, or the reference's regularised inverse (bsr.cpp:204-212)
__device__ void warp_pivot(double* m, double* d, double* keep, int nb, int* nreg) {
    const int lane = int(threadIdx.x & 31), b2 = nb * nb;
    for (int t = lane; t < b2; t += 32) keep[t] = d[t];
    __syncwarp();
    if (warp_invert(m, d, nb)) return;
    if (lane == 0) atomicAdd(nreg, 1);
    double sc = 0;
    for (int t = lane; t < b2; t += 32) sc = fmax(sc, fabs(keep[t]));
    for (int o = 16; o > 0; o >>= 1) sc = fmax(sc, __shfl_xor_sync(0xffffffffu, sc, o));
    if (!(sc > 0) || !isfinite(sc)) sc = 1.0;
    for (int t = lane; t < b2; t += 32) d[t] = keep[t];
    __syncwarp();
    if (lane < nb) {
        const double v = d[lane * nb + lane];
        d[lane * nb + lane] = ga(v, ga(gm(v >= 0 ? 1e-8 : -1e-8, sc), v == 0 ? gm(sc, 1e-8) : 0.0));
    }
    __syncwarp();
    if (warp_invert(m, d, nb)) return;
    for (int t = lane; t < b2; t += 32) d[t] = 0.0;
    __syncwarp();
    if (lane < nb) d[lane * nb + lane] = gd(1.0, sc);
    __syncwarp();
}

// ------------------------------------------------------------------ BILU0 factorisation (bilu0Row, bsr.cpp:183-215)
// One warp per row of rows[r0, r1) (a forward level); LU holds the matrix values and is factored in place.
struct GenWarpSmem {
    double m[GEN_MAX_NB * 2 * GEN_MAX_NB];
    double tmp[GEN_MAX_NB * GEN_MAX_NB];
    double keep[GEN_MAX_NB * GEN_MAX_NB];
};

__device__ int find_col(const int* __restrict__ ci, int lo, int hi, int j) {
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const int c = ci[mid];
        if (c == j) return mid;
        if (c < j) lo = mid + 1;
        else hi = mid;
    }
    return -1;
}

__device__ void factor_row(int i, int nb, const int* __restrict__ rp, const int* __restrict__ ci, const int* __restrict__ dg, double* LU,
                           GenWarpSmem& W, int* nreg) {
    const int lane = int(threadIdx.x & 31), b2 = nb * nb;
    const int r0 = rp[i], r1 = rp[i + 1];
    for (int p = r0; p < r1; ++p) {
        const int k = ci[p];
        if (k >= i) break;
        // L_ik = A_ik U_kk^-1 (gemm: every element summed over m in order from zero)
        const double* d = LU + size_t(dg[k]) * b2;
        double* aik = LU + size_t(p) * b2;
        for (int t = lane; t < b2; t += 32) {
            const int r = t / nb, c = t % nb;
            double s = 0;
            for (int q = 0; q < nb; ++q) s = ga(s, gm(aik[r * nb + q], d[q * nb + c]));
            W.tmp[t] = s;
        }
        __syncwarp();
        for (int t = lane; t < b2; t += 32) aik[t] = W.tmp[t];
        __syncwarp();
        for (int q = dg[k] + 1; q < rp[k + 1]; ++q) {
            const int pj = find_col(ci, r0, r1, ci[q]);
            if (pj < 0) continue;
            const double* u = LU + size_t(q) * b2;
            double* tgt = LU + size_t(pj) * b2;
            for (int t = lane; t < b2; t += 32) {   // gemmSub: c -= sum_m tmp[r][m] u[m][c]
                const int r = t / nb, c = t % nb;
                double s = 0;
                for (int m = 0; m < nb; ++m) s = ga(s, gm(W.tmp[r * nb + m], u[m * nb + c]));
                tgt[t] = gs(tgt[t], s);
            }
            __syncwarp();
        }
    }
    warp_pivot(W.m, LU + size_t(dg[i]) * b2, W.keep, nb, nreg);
}

__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_gen_factor_level(int r0, int r1, const int* __restrict__ ord, int nb,
                                                                         const int* __restrict__ rp, const int* __restrict__ ci,
                                                                         const int* __restrict__ dg, double* LU, int* nreg) {
    __shared__ GenWarpSmem W[kWarpsPerBlock];
    const int w = int(threadIdx.x >> 5);
    for (int q = r0 + int(blockIdx.x) * kWarpsPerBlock + w; q < r1; q += int(gridDim.x) * kWarpsPerBlock)
        factor_row(ord[q], nb, rp, ci, dg, LU, W[w], nreg);
}
// every level in one block (small systems): the warps take the rows of a level, a barrier between levels
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_gen_factor_cta(int nl, const int* __restrict__ lvl, const int* __restrict__ ord,
                                                                       int nb, const int* __restrict__ rp, const int* __restrict__ ci,
                                                                       const int* __restrict__ dg, double* LU, int* nreg) {
    __shared__ GenWarpSmem W[kWarpsPerBlock];
    const int w = int(threadIdx.x >> 5);
    for (int l = 0; l < nl; ++l) {
        for (int q = lvl[l] + w; q < lvl[l + 1]; q += kWarpsPerBlock) factor_row(ord[q], nb, rp, ci, dg, LU, W[w], nreg);
        __syncthreads();
    }
}

// ------------------------------------------------------------------ BILU0 sweeps (BILU0::apply, bsr.cpp:437-596)
// forward row i, element e: z_i[e] = r_i[e] - sum over L entries (row order) of sum_f L[e][f] z_k[f]
__device__ __forceinline__ void fwd_elem(int i, int e, int nb, const int* __restrict__ rp, const int* __restrict__ ci,
                                         const int* __restrict__ dg, const double* __restrict__ LU, const double* r, double* z) {
    const int b2 = nb * nb;
    double zi = r[size_t(i) * nb + e];
    for (int p = rp[i]; p < dg[i]; ++p) {
        const double* a = LU + size_t(p) * b2 + size_t(e) * nb;
        const double* zk = z + size_t(ci[p]) * nb;
        double s = 0;
        for (int f = 0; f < nb; ++f) s = ga(s, gm(a[f], zk[f]));
        zi = gs(zi, s);
    }
    z[size_t(i) * nb + e] = zi;
}
// backward row i (nb consecutive lanes of one warp, lane e): t = y_i - sum over U entries; z_i = U_ii^-1 t
__device__ __forceinline__ void bwd_row(int i, int e, bool act, int nb, const int* __restrict__ rp, const int* __restrict__ ci,
                                        const int* __restrict__ dg, const double* __restrict__ LU, double* z, unsigned mask, int base) {
    const int b2 = nb * nb;
    double zi = 0;
    if (act) {
        zi = z[size_t(i) * nb + e];
        for (int p = dg[i] + 1; p < rp[i + 1]; ++p) {
            const double* a = LU + size_t(p) * b2 + size_t(e) * nb;
            const double* zj = z + size_t(ci[p]) * nb;
            double s = 0;
            for (int f = 0; f < nb; ++f) s = ga(s, gm(a[f], zj[f]));
            zi = gs(zi, s);
        }
    }
    // the row's elements from the lanes that hold them, then t[e] = 0 + sum_f D[e][f] zi[f] (gemvAddN from zero)
    double t = 0;
    const double* d = act ? LU + size_t(dg[i]) * b2 + size_t(e) * nb : nullptr;
    for (int f = 0; f < nb; ++f) {
        const double zf = __shfl_sync(mask, zi, base + f);
        if (act) t = ga(t, gm(d[f], zf));
    }
    double t0 = 0;
    if (act) t0 = ga(0.0, t);
    if (act) z[size_t(i) * nb + e] = t0;
}

// threads of a level: nb per row (rows of the level in groups of 32 / nb per warp for the backward sweep)
__device__ __forceinline__ void fwd_level(int r0, int r1, const int* __restrict__ ord, int nb, const int* __restrict__ rp,
                                          const int* __restrict__ ci, const int* __restrict__ dg, const double* __restrict__ LU,
                                          const double* r, double* z, int tid, int nthr) {
    const long long tot = (long long)(r1 - r0) * nb;
    for (long long q = tid; q < tot; q += nthr) fwd_elem(ord[r0 + int(q / nb)], int(q % nb), nb, rp, ci, dg, LU, r, z);
}
__device__ __forceinline__ void bwd_level(int r0, int r1, const int* __restrict__ ord, int nb, const int* __restrict__ rp,
                                          const int* __restrict__ ci, const int* __restrict__ dg, const double* __restrict__ LU, double* z,
                                          int tid, int nthr) {
    const int per = 32 / nb;                       // rows per warp
    const int lane = tid & 31, slot = lane / nb, e = lane % nb;
    const int wid = tid >> 5, nw = nthr >> 5;
    const int base = slot * nb;
    const unsigned grp = (nb == 32 ? 0xffffffffu : (((1u << nb) - 1u) << base));
    for (int g = wid; g * per < r1 - r0; g += nw) {
        const int q = r0 + g * per + slot;
        const bool inSlot = slot < per;
        const bool act = inSlot && q < r1;
        if (inSlot) bwd_row(act ? ord[q] : 0, e, act, nb, rp, ci, dg, LU, z, grp, base);
    }
}

__global__ void k_gen_fwd_level(int r0, int r1, const int* __restrict__ ord, int nb, const int* __restrict__ rp, const int* __restrict__ ci,
                                const int* __restrict__ dg, const double* __restrict__ LU, const double* r, double* z) {
    fwd_level(r0, r1, ord, nb, rp, ci, dg, LU, r, z, int(blockIdx.x * blockDim.x + threadIdx.x), int(gridDim.x * blockDim.x));
}
__global__ void k_gen_bwd_level(int r0, int r1, const int* __restrict__ ord, int nb, const int* __restrict__ rp, const int* __restrict__ ci,
                                const int* __restrict__ dg, const double* __restrict__ LU, double* z) {
    bwd_level(r0, r1, ord, nb, rp, ci, dg, LU, z, int(blockIdx.x * blockDim.x + threadIdx.x), int(gridDim.x * blockDim.x));
}
__global__ void __launch_bounds__(kCtaThreads) k_gen_sweep_cta(int nlf, const int* __restrict__ fl, const int* __restrict__ fo, int nlb,
                                                               const int* __restrict__ bl, const int* __restrict__ bo, int nb,
                                                               const int* __restrict__ rp, const int* __restrict__ ci,
                                                               const int* __restrict__ dg, const double* __restrict__ LU, const double* r,
                                                               double* z) {
    const int tid = int(threadIdx.x), nt = int(blockDim.x);
    for (int l = 0; l < nlf; ++l) {
        fwd_level(fl[l], fl[l + 1], fo, nb, rp, ci, dg, LU, r, z, tid, nt);
        __syncthreads();
    }
    for (int l = 0; l < nlb; ++l) {
        bwd_level(bl[l], bl[l + 1], bo, nb, rp, ci, dg, LU, z, tid, nt);
        __syncthreads();
    }
}

// ------------------------------------------------------------------ CPR set-up (BlockCPR::setup, bsr.cpp:993-1059)
// one warp per cell: weights w_i = first row of D^-1, D the accumulation block when its inverse is well conditioned
// (true-IMPES), else the diagonal block of S (quasi-IMPES)
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_gen_weights(int n, int nb, const int* __restrict__ dg, const double* __restrict__ S,
                                                                    const double* __restrict__ acc, double* w, int* nfb) {
    __shared__ GenWarpSmem W[kWarpsPerBlock];
    const int wi = int(threadIdx.x >> 5), lane = int(threadIdx.x & 31), b2 = nb * nb;
    GenWarpSmem& M = W[wi];
    for (int i = int(blockIdx.x) * kWarpsPerBlock + wi; i < n; i += int(gridDim.x) * kWarpsPerBlock) {
        const double* sd = S + size_t(dg[i]) * b2;
        double* D = M.tmp;
        for (int t = lane; t < b2; t += 32) D[t] = sd[t];
        __syncwarp();
        bool inverted = false;
        if (acc) {
            const double* B = acc + size_t(i) * b2;
            double* inv = M.keep;
            for (int t = lane; t < b2; t += 32) inv[t] = B[t];
            __syncwarp();
            if (warp_invert(M.m, inv, nb)) {
                double c = 0, d = 0;                   // column sums of |B| and |B^-1| (lane = column)
                if (lane < nb)
                    for (int r = 0; r < nb; ++r) { c = ga(c, fabs(B[r * nb + lane])); d = ga(d, fabs(inv[r * nb + lane])); }
                double n1 = c, ni = d;
                for (int o = 16; o > 0; o >>= 1) {
                    n1 = fmax(n1, __shfl_xor_sync(0xffffffffu, n1, o));
                    ni = fmax(ni, __shfl_xor_sync(0xffffffffu, ni, o));
                }
                if (nb == 1 || gm(n1, ni) <= 1e10) {
                    for (int t = lane; t < b2; t += 32) D[t] = inv[t];
                    inverted = true;
                } else if (lane == 0) {
                    atomicAdd(nfb, 1);
                }
            } else if (nb == 1) {
                for (int t = lane; t < b2; t += 32) D[t] = B[t];
            } else if (lane == 0) {
                atomicAdd(nfb, 1);
            }
            __syncwarp();
        }
        double wv = 1.0;
        if (inverted || warp_invert(M.m, D, nb)) {
            if (lane < nb) wv = D[lane];
        } else {
            double s = 0;
            for (int e = 0; e < nb; ++e) s = ga(s, sd[e * nb]);
            wv = fabs(s) > 1e-300 ? gd(1.0, s) : 1.0;
        }
        double wm = lane < nb ? fabs(wv) : 0.0;
        for (int o = 16; o > 0; o >>= 1) wm = fmax(wm, __shfl_xor_sync(0xffffffffu, wm, o));
        if (!(wm > 0) || !isfinite(wm)) wv = 1.0;
        if (lane < nb) w[size_t(i) * nb + lane] = wv;
        __syncwarp();
    }
}
// Ap_p = sum_e w_ie S_p[e][0] for every block p of row i
__global__ void k_gen_pressure(int n, int nb, const int* __restrict__ rp, const double* __restrict__ S, const double* __restrict__ w,
                               double* ap) {
    const int b2 = nb * nb;
    for (int i = int(blockIdx.x * blockDim.x + threadIdx.x); i < n; i += int(gridDim.x * blockDim.x)) {
        const double* wi = w + size_t(i) * nb;
        for (int p = rp[i]; p < rp[i + 1]; ++p) {
            const double* a = S + size_t(p) * b2;
            double s = 0;
            for (int e = 0; e < nb; ++e) s = ga(s, gm(wi[e], a[e * nb]));
            ap[p] = s;
        }
    }
}
// level 0 of the hierarchy in its level space: values gathered from the pressure matrix, tiny diagonals -> 1
__global__ void k_gen_amg_level0(int nnz, const int* __restrict__ src, const double* __restrict__ ap, double* v) {
    for (int p = int(blockIdx.x * blockDim.x + threadIdx.x); p < nnz; p += int(gridDim.x * blockDim.x)) v[p] = ap[src[p]];
}
__global__ void k_gen_gather_sum(int cnt, const int* __restrict__ ptr, const int* __restrict__ src, const double* __restrict__ in,
                                 double* out) {
    for (int e = int(blockIdx.x * blockDim.x + threadIdx.x); e < cnt; e += int(gridDim.x * blockDim.x)) {
        const int q0 = ptr[e], q1 = ptr[e + 1];
        double s = 0;
        if (q0 < q1) {
            s = in[src[q0]];
            for (int q = q0 + 1; q < q1; ++q) s = ga(s, in[src[q]]);
        }
        out[e] = s;
    }
}
__global__ void k_gen_diag_fix(int n, const int* __restrict__ dg, double* v) {
    for (int i = int(blockIdx.x * blockDim.x + threadIdx.x); i < n; i += int(gridDim.x * blockDim.x))
        if (fabs(v[dg[i]]) < 1e-300) v[dg[i]] = 1.0;
}
// dense LU with partial pivoting of the coarsest level in its natural numbering (AMG::factorCoarsest,
// engine/src/amg.cpp:273-295), one thread block; lu is m x m, perm: level-space row -> natural row
__global__ void __launch_bounds__(1024) k_gen_coarse_lu(int m, const int* __restrict__ rp, const int* __restrict__ ci,
                                                        const double* __restrict__ v, const int* __restrict__ perm, double* lu, int* piv) {
    __shared__ double smx[32];
    __shared__ int sid[32];
    __shared__ int spr;
    const int tid = int(threadIdx.x), nt = int(blockDim.x);
    for (long long q = tid; q < (long long)m * m; q += nt) lu[q] = 0.0;
    __syncthreads();
    for (int k = tid; k < m; k += nt) {
        const int I = perm[k];
        for (int p = rp[k]; p < rp[k + 1]; ++p) lu[size_t(I) * m + perm[ci[p]]] = v[p];
    }
    __syncthreads();
    for (int k = 0; k < m; ++k) {
        // pivot: the first row i >= k of the largest |lu[i][k]| (strictly greater replaces)
        double best = -1.0;
        int bi = m;
        for (int i = k + tid; i < m; i += nt) {
            const double a = fabs(lu[size_t(i) * m + k]);
            if (a > best || (a == best && i < bi)) { best = a; bi = i; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if ((tid & 31) == 0) { smx[tid >> 5] = best; sid[tid >> 5] = bi; }
        __syncthreads();
        if (tid == 0) {
            double b = smx[0];
            int id = sid[0];
            for (int w = 1; w < (nt + 31) / 32; ++w)
                if (smx[w] > b || (smx[w] == b && sid[w] < id)) { b = smx[w]; id = sid[w]; }
            // the reference keeps k unless a later row is strictly larger: the smallest index among equal maxima
            // is k itself whenever |lu[k][k]| is the maximum
            spr = (id < m) ? id : k;
            if (!(fabs(lu[size_t(spr) * m + k]) > fabs(lu[size_t(k) * m + k]))) spr = k;
            piv[k] = spr;
        }
        __syncthreads();
        const int pr = spr;
        if (pr != k)
            for (int j = tid; j < m; j += nt) {
                const double t = lu[size_t(k) * m + j];
                lu[size_t(k) * m + j] = lu[size_t(pr) * m + j];
                lu[size_t(pr) * m + j] = t;
            }
        __syncthreads();
        if (tid == 0 && fabs(lu[size_t(k) * m + k]) < 1e-300) lu[size_t(k) * m + k] = 1e-300;
        __syncthreads();
        const double dk = lu[size_t(k) * m + k];
        for (int i = k + 1 + tid; i < m; i += nt) lu[size_t(i) * m + k] = gd(lu[size_t(i) * m + k], dk);
        __syncthreads();
        const int w = m - k - 1;
        for (long long q = tid; q < (long long)w * w; q += nt) {
            const int i = k + 1 + int(q / w), j = k + 1 + int(q % w);
            const double f = lu[size_t(i) * m + k];
            if (f != 0) lu[size_t(i) * m + j] = gs(lu[size_t(i) * m + j], gm(f, lu[size_t(k) * m + j]));
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ AMG V-cycle (AMG::cycle, engine/src/amg.cpp:303-337)
// Gauss-Seidel row k of a level (level space, entries in natural order): x_k = (b_k - sum_{j != k} a_kj x_j) / a_kk
__device__ __forceinline__ void gs_row(int k, const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ v,
                                       const int* __restrict__ dg, const double* b, double* x) {
    double s = b[k];
    for (int p = rp[k]; p < rp[k + 1]; ++p)
        if (ci[p] != k) s = gs(s, gm(v[p], x[ci[p]]));
    x[k] = gd(s, v[dg[k]]);
}
__global__ void k_gen_gs_level(int r0, int r1, const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ v,
                               const int* __restrict__ dg, const double* b, double* x) {
    for (int k = r0 + int(blockIdx.x * blockDim.x + threadIdx.x); k < r1; k += int(gridDim.x * blockDim.x)) gs_row(k, rp, ci, v, dg, b, x);
}
// a whole sweep in one block; forward: levels 0..nl-1, backward: nl-1..0 (rows of a level independent either way)
__global__ void __launch_bounds__(kCtaThreads) k_gen_gs_cta(int nl, const int* __restrict__ lvl, int fwd, int reps,
                                                            const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ v,
                                                            const int* __restrict__ dg, const double* b, double* x) {
    for (int it = 0; it < reps; ++it)
        for (int pass = 0; pass < 2; ++pass) {
            if (reps == 1 && pass == 1) break;
            const bool f = reps == 1 ? fwd != 0 : pass == 0;
            for (int q = 0; q < nl; ++q) {
                const int l = f ? q : nl - 1 - q;
                for (int k = lvl[l] + int(threadIdx.x); k < lvl[l + 1]; k += int(blockDim.x)) gs_row(k, rp, ci, v, dg, b, x);
                __syncthreads();
            }
        }
}
__global__ void k_gen_resid(int n, const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ v, const double* b,
                            const double* x, double* r) {
    for (int k = int(blockIdx.x * blockDim.x + threadIdx.x); k < n; k += int(gridDim.x * blockDim.x)) {
        double s = 0;
        for (int p = rp[k]; p < rp[k + 1]; ++p) s = ga(s, gm(v[p], x[ci[p]]));
        r[k] = gs(b[k], s);
    }
}
// restriction R r (members of each coarse row in ascending natural order, unit weights)
__global__ void k_gen_restrict(int nc, const int* __restrict__ mp, const int* __restrict__ mem, const double* r, double* bc) {
    for (int K = int(blockIdx.x * blockDim.x + threadIdx.x); K < nc; K += int(gridDim.x * blockDim.x)) {
        double s = 0;
        for (int q = mp[K]; q < mp[K + 1]; ++q) s = ga(s, gm(1.0, r[mem[q]]));
        bc[K] = s;
    }
}
// prolongation x += P x_c (unit weights)
__global__ void k_gen_prolong(int n, const int* __restrict__ agg, const double* xc, double* x) {
    for (int k = int(blockIdx.x * blockDim.x + threadIdx.x); k < n; k += int(gridDim.x * blockDim.x))
        x[k] = ga(x[k], ga(0.0, gm(1.0, xc[agg[k]])));
}
// coarsest dense solve: row interchanges, L y = b column by column (the reference's order), U x = y column by column
__global__ void __launch_bounds__(1024) k_gen_coarse_solve(int m, const double* __restrict__ lu, const int* __restrict__ piv,
                                                           const int* __restrict__ perm, const double* b, double* x, double* work) {
    const int tid = int(threadIdx.x), nt = int(blockDim.x);
    for (int k = tid; k < m; k += nt) work[perm[k]] = b[k];
    __syncthreads();
    if (tid == 0)
        for (int k = 0; k < m; ++k)
            if (piv[k] != k) { const double t = work[k]; work[k] = work[piv[k]]; work[piv[k]] = t; }
    __syncthreads();
    for (int k = 0; k < m; ++k) {
        const double xk = work[k];
        for (int i = k + 1 + tid; i < m; i += nt) work[i] = gs(work[i], gm(lu[size_t(i) * m + k], xk));
        __syncthreads();
    }
    for (int k = m - 1; k >= 0; --k) {
        if (tid == 0) work[k] = gd(work[k], lu[size_t(k) * m + k]);
        __syncthreads();
        const double xk = work[k];
        for (int i = tid; i < k; i += nt) work[i] = gs(work[i], gm(lu[size_t(i) * m + k], xk));
        __syncthreads();
    }
    for (int k = tid; k < m; k += nt) x[k] = work[perm[k]];
}

// ------------------------------------------------------------------ CPR application (BlockCPR::apply, bsr.cpp:1061-1084)
// rp_i = sum_e w_ie r_ie, placed at the level-space row of cell i
__global__ void k_gen_cpr_in(int n, int nb, const int* __restrict__ perm, const double* __restrict__ w, const double* r, double* b0) {
    for (int k = int(blockIdx.x * blockDim.x + threadIdx.x); k < n; k += int(gridDim.x * blockDim.x)) {
        const int i = perm[k];
        double s = 0;
        for (int e = 0; e < nb; ++e) s = ga(s, gm(w[size_t(i) * nb + e], r[size_t(i) * nb + e]));
        b0[k] = s;
    }
}
// t_ie = r_ie - sum over the row's blocks of S_p[e][0] xp_col (the pressure column of the blocks)
__global__ void k_gen_cpr_t(int n, int nb, const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ S,
                            const int* __restrict__ iperm, const double* x0, const double* r, double* t) {
    const int b2 = nb * nb;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (long long)n * nb; q += (long long)gridDim.x * blockDim.x) {
        const int i = int(q / nb), e = int(q % nb);
        double a = r[q];
        for (int p = rp[i]; p < rp[i + 1]; ++p) a = gs(a, gm(S[size_t(p) * b2 + size_t(e) * nb], x0[iperm[ci[p]]]));
        t[q] = a;
    }
}
__global__ void k_gen_cpr_zp(int n, int nb, const int* __restrict__ iperm, const double* x0, double* z) {
    for (int i = int(blockIdx.x * blockDim.x + threadIdx.x); i < n; i += int(gridDim.x * blockDim.x))
        z[size_t(i) * nb] = ga(z[size_t(i) * nb], x0[iperm[i]]);
}

// ------------------------------------------------------------------ Krylov vector kernels
constexpr int kDotBlocks = 256, kDotThreads = 256;
// deterministic inner product: a fixed grid, each thread's elements in order, then fixed trees
__global__ void __launch_bounds__(kDotThreads) k_gen_dot(long long N, const double* __restrict__ x, const double* __restrict__ y,
                                                         double* part) {
    __shared__ double sh[kDotThreads / 32];
    double s = 0;
    for (long long q = blockIdx.x * (long long)kDotThreads + threadIdx.x; q < N; q += (long long)kDotBlocks * kDotThreads)
        s = ga(s, gm(x[q], y[q]));
    for (int o = 16; o > 0; o >>= 1) s = ga(s, __shfl_down_sync(0xffffffffu, s, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < kDotThreads / 32; ++w) t = ga(t, sh[w]);
        part[blockIdx.x] = t;
    }
}
__global__ void k_gen_dot_final(const double* __restrict__ part, double* out) {
    __shared__ double sh[kDotBlocks];
    sh[threadIdx.x] = part[threadIdx.x];
    __syncthreads();
    for (int o = kDotBlocks / 2; o > 0; o >>= 1) {
        if (int(threadIdx.x) < o) sh[threadIdx.x] = ga(sh[threadIdx.x], sh[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}
// y = a x + b y (+ c z), element by element in the reference's expression order
__global__ void k_gen_bicg_p(long long N, double beta, double omega, const double* r, const double* v, double* p) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < N; q += (long long)gridDim.x * blockDim.x)
        p[q] = ga(r[q], gm(beta, gs(p[q], gm(omega, v[q]))));
}
__global__ void k_gen_axpy_to(long long N, double a, const double* x, const double* y, double* out) {   // out = y - a x
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < N; q += (long long)gridDim.x * blockDim.x)
        out[q] = gs(y[q], gm(a, x[q]));
}
__global__ void k_gen_axpy(long long N, double a, const double* x, double* y) {   // y += a x
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < N; q += (long long)gridDim.x * blockDim.x)
        y[q] = ga(y[q], gm(a, x[q]));
}
__global__ void k_gen_bicg_xr(long long N, double alpha, double omega, const double* ph, const double* sh, const double* s, const double* t,
                              double* x, double* r) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < N; q += (long long)gridDim.x * blockDim.x) {
        x[q] = ga(x[q], ga(gm(alpha, ph[q]), gm(omega, sh[q])));
        r[q] = gs(s[q], gm(omega, t[q]));
    }
}
__global__ void k_gen_scale(long long N, double inv, const double* x, double* y, int divide) {   // y = x / d or x * a
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < N; q += (long long)gridDim.x * blockDim.x)
        y[q] = divide ? gd(x[q], inv) : gm(x[q], inv);
}
__global__ void k_gen_sub_from(long long N, const double* b, double* r) {   // r = b - r
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < N; q += (long long)gridDim.x * blockDim.x) r[q] = gs(b[q], r[q]);
}

int grid_of(long long work, int threads = 256) {
    long long g = (work + threads - 1) / threads;
    const long long cap = 4LL * device_sm_count() * 8;
    if (g > cap) g = cap;
    return int(std::max(1LL, g));
}

}  // namespace

// ------------------------------------------------------------------ host engine
struct GenLevel {
    int n = 0, nnz = 0;
    int *rp = nullptr, *ci = nullptr, *dg = nullptr, *lvl = nullptr, *agg = nullptr, *memPtr = nullptr, *mem = nullptr;
    int *apPtr = nullptr, *apSrc = nullptr, *acPtr = nullptr, *acSrc = nullptr, *perm = nullptr;
    int nAP = 0;
    std::vector<int> lvlHost;          // GS level starts
    double *v = nullptr, *x = nullptr, *b = nullptr, *r = nullptr;
    bool coarse = false, dense = false;
    double* lu = nullptr;
    int* piv = nullptr;
};

struct GenEngine {
    cudaStream_t st = nullptr;
    std::vector<void*> pat, vals;      // device allocations: per pattern / per value set
    // pattern
    int n = 0, nb = 0, nnzb = 0;
    std::vector<int> rp0, ci0;
    HostPlan plan;                     // level-space plan of the pattern (validation, AMG level 0)
    std::vector<int> fStart, bStart;   // host level starts
    int *rp = nullptr, *ci = nullptr, *dg = nullptr, *fOrd = nullptr, *bOrd = nullptr, *fLvl = nullptr, *bLvl = nullptr;
    int *valSrc = nullptr, *perm0 = nullptr, *iperm0 = nullptr;
    bool oneCta = false;
    // values and factors
    double *S = nullptr, *LU = nullptr;
    bool haveMatrix = false, haveSetup = false;
    int precond = RSG_PREC_BILU0;
    // CPR
    bool haveAmg = false;
    std::vector<GenLevel> lv;
    double *w = nullptr, *ap = nullptr, *apTmp = nullptr, *xpWork = nullptr, *T = nullptr;
    // Krylov vectors, reductions
    double *vx = nullptr, *vr = nullptr, *vrh = nullptr, *vp = nullptr, *vv = nullptr, *vs = nullptr, *vt = nullptr, *vph = nullptr,
           *vsh = nullptr, *vb = nullptr;
    std::vector<double*> V, Z;
    int gmM = 0;
    double *stIn = nullptr, *stOut = nullptr;   // staging of host vectors
    double *part = nullptr, *dotOut = nullptr, *hpin = nullptr;
    int *dCnt = nullptr;
    size_t bytesPat = 0, bytesVal = 0;
    rsg_stats stt{};
    long long launches = 0;
};

namespace {

template <class T>
int galloc(GenEngine& g, std::vector<void*>& list, size_t& bytes, T** p, size_t count) {
    const size_t by = std::max<size_t>(count, 1) * sizeof(T);
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(p), by, g.st);
    if (e != cudaSuccess) return gfail(RSG_ENOMEM, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
    list.push_back(*p);
    bytes += by;
    return RSG_OK;
}
template <class T>
int gupload(GenEngine& g, T** p, const std::vector<T>& v) {
    int rc = galloc(g, g.pat, g.bytesPat, p, v.size());
    if (rc) return rc;
    if (!v.empty()) GEN_CUDA(cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, g.st));
    return RSG_OK;
}
void release(GenEngine& g, std::vector<void*>& list, size_t& bytes) {
    for (void* p : list) cudaFreeAsync(p, g.st);
    list.clear();
    bytes = 0;
}
void drop_pattern(GenEngine& g) {
    release(g, g.vals, g.bytesVal);
    release(g, g.pat, g.bytesPat);
    g.lv.clear();
    g.V.clear();
    g.Z.clear();
    g.gmM = 0;
    g.haveMatrix = g.haveSetup = g.haveAmg = false;
    g.S = g.LU = g.w = g.ap = g.apTmp = g.xpWork = g.T = nullptr;
    g.vx = g.vr = g.vrh = g.vp = g.vv = g.vs = g.vt = g.vph = g.vsh = g.vb = nullptr;
    g.stIn = g.stOut = nullptr;
}

// level sets of the L (forward) or U (backward) dependency graph (engine/src/bsr.cpp:270-300): rows grouped by level
void level_sets(int n, const std::vector<int>& rp, const std::vector<int>& ci, const std::vector<int>& dg, bool forward,
                std::vector<int>& ord, std::vector<int>& start) {
    std::vector<int> lev(size_t(n), 0);
    int nl = 0;
    if (forward) {
        for (int i = 0; i < n; ++i) {
            int l = 0;
            for (int p = rp[size_t(i)]; p < dg[size_t(i)]; ++p) l = std::max(l, lev[size_t(ci[size_t(p)])] + 1);
            lev[size_t(i)] = l;
            nl = std::max(nl, l + 1);
        }
    } else {
        for (int i = n - 1; i >= 0; --i) {
            int l = 0;
            for (int p = dg[size_t(i)] + 1; p < rp[size_t(i) + 1]; ++p) l = std::max(l, lev[size_t(ci[size_t(p)])] + 1);
            lev[size_t(i)] = l;
            nl = std::max(nl, l + 1);
        }
    }
    start.assign(size_t(nl) + 1, 0);
    for (int i = 0; i < n; ++i) start[size_t(lev[size_t(i)]) + 1]++;
    for (int l = 0; l < nl; ++l) start[size_t(l) + 1] += start[size_t(l)];
    std::vector<int> fill(start.begin(), start.end() - 1);
    ord.assign(size_t(n), 0);
    for (int i = 0; i < n; ++i) ord[size_t(fill[size_t(lev[size_t(i)])]++)] = i;
}

// deterministic inner products, read back to the host (one synchronisation per call)
int gdot(GenEngine& g, const double* x, const double* y, double* out) {
    const long long N = (long long)g.n * g.nb;
    k_gen_dot<<<kDotBlocks, kDotThreads, 0, g.st>>>(N, x, y, g.part);
    k_gen_dot_final<<<1, kDotBlocks, 0, g.st>>>(g.part, g.dotOut);
    g.launches += 2;
    GEN_CUDA(cudaMemcpyAsync(g.hpin, g.dotOut, sizeof(double), cudaMemcpyDeviceToHost, g.st));
    GEN_CUDA(cudaStreamSynchronize(g.st));
    *out = g.hpin[0];
    return RSG_OK;
}

void spmv(GenEngine& g, const double* x, double* y) {
    k_gen_spmv<<<grid_of((long long)g.n * g.nb), 256, 0, g.st>>>(g.n, g.nb, g.rp, g.ci, g.S, x, y);
    ++g.launches;
}

void ilu_apply(GenEngine& g, const double* r, double* z) {
    const int nlf = int(g.fStart.size()) - 1, nlb = int(g.bStart.size()) - 1;
    if (g.oneCta) {
        k_gen_sweep_cta<<<1, kCtaThreads, 0, g.st>>>(nlf, g.fLvl, g.fOrd, nlb, g.bLvl, g.bOrd, g.nb, g.rp, g.ci, g.dg, g.LU, r, z);
        ++g.launches;
        return;
    }
    for (int l = 0; l < nlf; ++l) {
        const int r0 = g.fStart[size_t(l)], r1 = g.fStart[size_t(l) + 1];
        k_gen_fwd_level<<<grid_of((long long)(r1 - r0) * g.nb), 256, 0, g.st>>>(r0, r1, g.fOrd, g.nb, g.rp, g.ci, g.dg, g.LU, r, z);
    }
    for (int l = 0; l < nlb; ++l) {
        const int r0 = g.bStart[size_t(l)], r1 = g.bStart[size_t(l) + 1];
        k_gen_bwd_level<<<grid_of((long long)(r1 - r0) * 32 / std::max(1, 32 / g.nb)), 256, 0, g.st>>>(r0, r1, g.bOrd, g.nb, g.rp, g.ci,
                                                                                                     g.dg, g.LU, z);
    }
    g.launches += nlf + nlb;
}

void gs_sweep(GenEngine& g, GenLevel& L, bool fwd, int reps) {
    const int nl = int(L.lvlHost.size()) - 1;
    if (L.n <= 16 * kCtaThreads || reps > 1) {
        k_gen_gs_cta<<<1, kCtaThreads, 0, g.st>>>(nl, L.lvl, fwd ? 1 : 0, reps, L.rp, L.ci, L.v, L.dg, L.b, L.x);
        ++g.launches;
        return;
    }
    for (int q = 0; q < nl; ++q) {
        const int l = fwd ? q : nl - 1 - q;
        const int r0 = L.lvlHost[size_t(l)], r1 = L.lvlHost[size_t(l) + 1];
        k_gen_gs_level<<<grid_of(r1 - r0), 256, 0, g.st>>>(r0, r1, L.rp, L.ci, L.v, L.dg, L.b, L.x);
    }
    g.launches += nl;
}

void vcycle(GenEngine& g, int l) {
    GenLevel& L = g.lv[size_t(l)];
    if (L.coarse) {
        if (L.dense) {
            k_gen_coarse_solve<<<1, 1024, 0, g.st>>>(L.n, L.lu, L.piv, L.perm, L.b, L.x, L.r);
            ++g.launches;
        } else {
            cudaMemsetAsync(L.x, 0, sizeof(double) * size_t(L.n), g.st);
            gs_sweep(g, L, true, 20);
        }
        return;
    }
    GenLevel& C = g.lv[size_t(l) + 1];
    cudaMemsetAsync(L.x, 0, sizeof(double) * size_t(L.n), g.st);
    gs_sweep(g, L, true, 1);
    k_gen_resid<<<grid_of(L.n), 256, 0, g.st>>>(L.n, L.rp, L.ci, L.v, L.b, L.x, L.r);
    k_gen_restrict<<<grid_of(C.n), 256, 0, g.st>>>(C.n, C.memPtr, C.mem, L.r, C.b);
    g.launches += 2;
    vcycle(g, l + 1);
    k_gen_prolong<<<grid_of(L.n), 256, 0, g.st>>>(L.n, L.agg, C.x, L.x);
    ++g.launches;
    gs_sweep(g, L, false, 1);
}

void precond(GenEngine& g, const double* r, double* z) {
    if (g.precond == RSG_PREC_CPR) {
        GenLevel& L0 = g.lv[0];
        k_gen_cpr_in<<<grid_of(g.n), 256, 0, g.st>>>(g.n, g.nb, g.perm0, g.w, r, L0.b);
        ++g.launches;
        vcycle(g, 0);
        k_gen_cpr_t<<<grid_of((long long)g.n * g.nb), 256, 0, g.st>>>(g.n, g.nb, g.rp, g.ci, g.S, g.iperm0, L0.x, r, g.T);
        ++g.launches;
        ilu_apply(g, g.T, z);
        k_gen_cpr_zp<<<grid_of(g.n), 256, 0, g.st>>>(g.n, g.nb, g.iperm0, L0.x, z);
        ++g.launches;
        return;
    }
    ilu_apply(g, r, z);
}

// the CPR hierarchy's device arrays from the host aggregation plan (first set-up of a pattern)
int build_amg(GenEngine& g, const std::vector<double>& ap0) {
    SysAmg H;
    std::string err;
    if (!amg_plan_system(g.plan, 0, ap0, H, err, host_threads())) return gfail(RSG_EINVAL, err);
    g.lv.assign(H.lv.size(), GenLevel{});
    for (size_t l = 0; l < H.lv.size(); ++l) {
        const AmgLevel& A = H.lv[l];
        GenLevel& L = g.lv[l];
        L.n = A.n;
        L.nnz = int(A.ci.size());
        L.lvlHost = A.lvlStart;
        L.coarse = l + 1 == H.lv.size();
        L.dense = L.coarse && H.coarseDense;
        int rc;
        if ((rc = gupload(g, &L.rp, A.rp)) || (rc = gupload(g, &L.ci, A.ci)) || (rc = gupload(g, &L.dg, A.diag)) ||
            (rc = gupload(g, &L.lvl, A.lvlStart)) || (rc = gupload(g, &L.perm, A.perm)) ||
            (rc = galloc(g, g.pat, g.bytesPat, &L.v, size_t(L.nnz))) || (rc = galloc(g, g.pat, g.bytesPat, &L.x, size_t(L.n))) ||
            (rc = galloc(g, g.pat, g.bytesPat, &L.b, size_t(L.n))) || (rc = galloc(g, g.pat, g.bytesPat, &L.r, size_t(L.n))))
            return rc;
        if (!A.agg.empty() && (rc = gupload(g, &L.agg, A.agg))) return rc;
        if (l > 0) {
            L.nAP = int(A.apPtr.size()) - 1;
            if ((rc = gupload(g, &L.memPtr, A.memPtr)) || (rc = gupload(g, &L.mem, A.mem)) || (rc = gupload(g, &L.apPtr, A.apPtr)) ||
                (rc = gupload(g, &L.apSrc, A.apSrc)) || (rc = gupload(g, &L.acPtr, A.acPtr)) || (rc = gupload(g, &L.acSrc, A.acSrc)))
                return rc;
        }
        if (L.dense && ((rc = galloc(g, g.pat, g.bytesPat, &L.lu, size_t(L.n) * size_t(L.n))) ||
                        (rc = galloc(g, g.pat, g.bytesPat, &L.piv, size_t(L.n)))))
            return rc;
    }
    size_t maxAP = 1;
    for (const GenLevel& L : g.lv) maxAP = std::max(maxAP, size_t(L.nAP));
    int rc = galloc(g, g.pat, g.bytesPat, &g.apTmp, maxAP);
    if (rc) return rc;
    g.haveAmg = true;
    return RSG_OK;
}

// every level's values from the fine pressure matrix (Galerkin gathers in the reference's summation order), tiny
// diagonals -> 1, and the coarsest LU
void refresh_amg(GenEngine& g) {
    GenLevel& L0 = g.lv[0];
    k_gen_amg_level0<<<grid_of(L0.nnz), 256, 0, g.st>>>(L0.nnz, g.valSrc, g.ap, L0.v);
    k_gen_diag_fix<<<grid_of(L0.n), 256, 0, g.st>>>(L0.n, L0.dg, L0.v);
    g.launches += 2;
    for (size_t l = 1; l < g.lv.size(); ++l) {
        GenLevel& F = g.lv[l - 1];
        GenLevel& C = g.lv[l];
        if (C.nAP > 0) k_gen_gather_sum<<<grid_of(C.nAP), 256, 0, g.st>>>(C.nAP, C.apPtr, C.apSrc, F.v, g.apTmp);
        k_gen_gather_sum<<<grid_of(C.nnz), 256, 0, g.st>>>(C.nnz, C.acPtr, C.acSrc, g.apTmp, C.v);
        k_gen_diag_fix<<<grid_of(C.n), 256, 0, g.st>>>(C.n, C.dg, C.v);
        g.launches += 3;
    }
    GenLevel& Lc = g.lv.back();
    if (Lc.dense) {
        k_gen_coarse_lu<<<1, 1024, 0, g.st>>>(Lc.n, Lc.rp, Lc.ci, Lc.v, Lc.perm, Lc.lu, Lc.piv);
        ++g.launches;
    }
}

int ensure_krylov(GenEngine& g, bool gmres, int m) {
    const size_t N = size_t(g.n) * g.nb;
    int rc;
    if (!g.vx) {
        double** vs[] = {&g.vx, &g.vr, &g.vrh, &g.vp, &g.vv, &g.vs, &g.vt, &g.vph, &g.vsh, &g.vb};
        for (double** v : vs)
            if ((rc = galloc(g, g.pat, g.bytesPat, v, N))) return rc;
    }
    if (gmres && g.gmM < m) {                    // the basis of the largest restart used with this pattern
        g.V.assign(size_t(m) + 1, nullptr);
        g.Z.assign(size_t(m), nullptr);
        for (auto& p : g.V)
            if ((rc = galloc(g, g.pat, g.bytesPat, &p, N))) return rc;
        for (auto& p : g.Z)
            if ((rc = galloc(g, g.pat, g.bytesPat, &p, N))) return rc;
        g.gmM = m;
    }
    return RSG_OK;
}

// BiCGSTAB (engine/src/linsolve.cpp:159-216) on device vectors; b in vb, x into vx
int bicgstab(GenEngine& g, double tol, int maxIt, int* itsOut, double* rrOut, bool* conv) {
    const long long N = (long long)g.n * g.nb;
    const int gr = grid_of(N);
    *conv = false;
    *itsOut = 0;
    *rrOut = 1.0;
    GEN_CUDA(cudaMemsetAsync(g.vx, 0, size_t(N) * sizeof(double), g.st));
    GEN_CUDA(cudaMemcpyAsync(g.vr, g.vb, size_t(N) * sizeof(double), cudaMemcpyDeviceToDevice, g.st));
    GEN_CUDA(cudaMemcpyAsync(g.vrh, g.vb, size_t(N) * sizeof(double), cudaMemcpyDeviceToDevice, g.st));
    GEN_CUDA(cudaMemsetAsync(g.vp, 0, size_t(N) * sizeof(double), g.st));
    GEN_CUDA(cudaMemsetAsync(g.vv, 0, size_t(N) * sizeof(double), g.st));
    double bn2, rc;
    int e;
    if ((e = gdot(g, g.vb, g.vb, &bn2))) return e;
    const double bn = std::sqrt(bn2);
    if (bn == 0) { *conv = true; *rrOut = 0; return RSG_OK; }
    double rho = 1, alpha = 1, omega = 1;
    for (int it = 1; it <= maxIt; ++it) {
        double rhoN;
        if ((e = gdot(g, g.vrh, g.vr, &rhoN))) return e;
        if (std::fabs(rhoN) < 1e-300) break;
        const double beta = (rhoN / rho) * (alpha / omega);
        rho = rhoN;
        k_gen_bicg_p<<<gr, 256, 0, g.st>>>(N, beta, omega, g.vr, g.vv, g.vp);
        ++g.launches;
        precond(g, g.vp, g.vph);
        spmv(g, g.vph, g.vv);
        double rv;
        if ((e = gdot(g, g.vrh, g.vv, &rv))) return e;
        if (std::fabs(rv) < 1e-300) break;
        alpha = rho / rv;
        k_gen_axpy_to<<<gr, 256, 0, g.st>>>(N, alpha, g.vv, g.vr, g.vs);
        ++g.launches;
        double sn2;
        if ((e = gdot(g, g.vs, g.vs, &sn2))) return e;
        const double sn = std::sqrt(sn2);
        if (sn / bn < tol) {
            k_gen_axpy<<<gr, 256, 0, g.st>>>(N, alpha, g.vph, g.vx);
            ++g.launches;
            *conv = true;
            *itsOut = it;
            *rrOut = sn / bn;
            return RSG_OK;
        }
        precond(g, g.vs, g.vsh);
        spmv(g, g.vsh, g.vt);
        double tt, ts;
        if ((e = gdot(g, g.vt, g.vt, &tt)) || (e = gdot(g, g.vt, g.vs, &ts))) return e;
        omega = tt > 0 ? ts / tt : 0;
        k_gen_bicg_xr<<<gr, 256, 0, g.st>>>(N, alpha, omega, g.vph, g.vsh, g.vs, g.vt, g.vx, g.vr);
        ++g.launches;
        if ((e = gdot(g, g.vr, g.vr, &rc))) return e;
        const double rn = std::sqrt(rc);
        *itsOut = it;
        *rrOut = rn / bn;
        if (rn / bn < tol) { *conv = true; return RSG_OK; }
        if (omega == 0) break;
    }
    return RSG_OK;
}

// flexible GMRES(m) with modified Gram-Schmidt and Givens rotations (engine/src/linsolve.cpp:218-273)
int gmres(GenEngine& g, double tol, int maxIt, int m, int* itsOut, double* rrOut, bool* conv) {
    const long long N = (long long)g.n * g.nb;
    const int gr = grid_of(N);
    *conv = false;
    *itsOut = 0;
    *rrOut = 1.0;
    GEN_CUDA(cudaMemsetAsync(g.vx, 0, size_t(N) * sizeof(double), g.st));
    double bn2;
    int e;
    if ((e = gdot(g, g.vb, g.vb, &bn2))) return e;
    const double bn = std::sqrt(bn2);
    if (bn == 0) { *conv = true; *rrOut = 0; return RSG_OK; }
    std::vector<double> H(static_cast<size_t>(m + 1) * static_cast<size_t>(m), 0.0), cs(static_cast<size_t>(m)), sn(static_cast<size_t>(m)),
        gv(static_cast<size_t>(m) + 1);
    auto Hat = [&](int i, int j) -> double& { return H[size_t(i) * m + j]; };
    int total = 0;
    double rel = 1.0;
    double* w = g.vt;
    while (total < maxIt) {
        spmv(g, g.vx, g.vr);
        k_gen_sub_from<<<gr, 256, 0, g.st>>>(N, g.vb, g.vr);
        ++g.launches;
        double b2;
        if ((e = gdot(g, g.vr, g.vr, &b2))) return e;
        const double beta = std::sqrt(b2);
        rel = beta / bn;
        if (rel < tol) { *conv = true; *itsOut = total; *rrOut = rel; return RSG_OK; }
        k_gen_scale<<<gr, 256, 0, g.st>>>(N, beta, g.vr, g.V[0], 1);
        ++g.launches;
        std::fill(gv.begin(), gv.end(), 0.0);
        gv[0] = beta;
        int j = 0;
        for (; j < m && total < maxIt; ++j, ++total) {
            precond(g, g.V[size_t(j)], g.Z[size_t(j)]);
            spmv(g, g.Z[size_t(j)], w);
            for (int i = 0; i <= j; ++i) {
                double h;
                if ((e = gdot(g, w, g.V[size_t(i)], &h))) return e;
                Hat(i, j) = h;
                k_gen_axpy<<<gr, 256, 0, g.st>>>(N, -h, g.V[size_t(i)], w);
                ++g.launches;
            }
            double hn2;
            if ((e = gdot(g, w, w, &hn2))) return e;
            const double hn = std::sqrt(hn2);
            Hat(j + 1, j) = hn;
            if (hn > 0) {
                k_gen_scale<<<gr, 256, 0, g.st>>>(N, hn, w, g.V[size_t(j) + 1], 1);
                ++g.launches;
            }
            for (int i = 0; i < j; ++i) {
                const double t = cs[size_t(i)] * Hat(i, j) + sn[size_t(i)] * Hat(i + 1, j);
                Hat(i + 1, j) = -sn[size_t(i)] * Hat(i, j) + cs[size_t(i)] * Hat(i + 1, j);
                Hat(i, j) = t;
            }
            const double den = std::hypot(Hat(j, j), Hat(j + 1, j));
            cs[size_t(j)] = den > 0 ? Hat(j, j) / den : 1;
            sn[size_t(j)] = den > 0 ? Hat(j + 1, j) / den : 0;
            Hat(j, j) = den;
            Hat(j + 1, j) = 0;
            gv[size_t(j) + 1] = -sn[size_t(j)] * gv[size_t(j)];
            gv[size_t(j)] = cs[size_t(j)] * gv[size_t(j)];
            rel = std::fabs(gv[size_t(j) + 1]) / bn;
            if (rel < tol) { ++j; ++total; break; }
        }
        std::vector<double> y(static_cast<size_t>(j));
        for (int i = j - 1; i >= 0; --i) {
            double s = gv[size_t(i)];
            for (int k = i + 1; k < j; ++k) s -= Hat(i, k) * y[size_t(k)];
            y[size_t(i)] = s / Hat(i, i);
        }
        for (int i = 0; i < j; ++i) {
            k_gen_axpy<<<gr, 256, 0, g.st>>>(N, y[size_t(i)], g.Z[size_t(i)], g.vx);
            ++g.launches;
        }
        *itsOut = total;
        *rrOut = rel;
        if (rel < tol) { *conv = true; return RSG_OK; }
    }
    return RSG_OK;
}

}  // namespace

GenEngine* gen_create(cudaStream_t st) {
    GenEngine* g = new GenEngine();
    g->st = st;
    return g;
}

void gen_destroy(GenEngine* g) {
    if (!g) return;
    drop_pattern(*g);
    if (g->part) cudaFreeAsync(g->part, g->st);
    if (g->dotOut) cudaFreeAsync(g->dotOut, g->st);
    if (g->dCnt) cudaFreeAsync(g->dCnt, g->st);
    if (g->hpin) cudaFreeHost(g->hpin);
    cudaStreamSynchronize(g->st);
    delete g;
}

int gen_set_matrix(GenEngine* gp, const rsg_options& o, int n, int nb, const int* rowPtr, const int* col, const double* val) {
    GenEngine& g = *gp;
    if (nb < 1 || nb > GEN_MAX_NB) return gfail(RSG_EINVAL, "block size nb = " + std::to_string(nb) + " outside [1, 16]");
    if (n < 1 || !rowPtr || !col || !val) return gfail(RSG_EINVAL, "set_matrix: empty system or null argument");
    if (o.precision != RSG_FP64) return gfail(RSG_EINVAL, "block sizes other than 3 are solved in FP64 (precision RSG_FP64)");
    if (o.precond != RSG_PREC_BILU0 && o.precond != RSG_PREC_CPR)
        return gfail(RSG_EINVAL, "block sizes other than 3 take the BILU0 or CPR preconditioner");
    if (rowPtr[0] != 0) return gfail(RSG_EINVAL, "rowPtr[0] must be 0");
    const int nnzb = rowPtr[n];
    const bool same = g.haveMatrix && g.n == n && g.nb == nb && g.nnzb == nnzb && std::equal(rowPtr, rowPtr + n + 1, g.rp0.begin()) &&
                      std::equal(col, col + nnzb, g.ci0.begin());
    if (!g.part) {
        int rc;
        if ((rc = galloc(g, g.pat, g.bytesPat, &g.part, kDotBlocks))) return rc;
        g.pat.pop_back();                                   // kept across patterns (freed by gen_destroy)
        if ((rc = galloc(g, g.pat, g.bytesPat, &g.dotOut, 1))) return rc;
        g.pat.pop_back();
        if ((rc = galloc(g, g.pat, g.bytesPat, &g.dCnt, 2))) return rc;
        g.pat.pop_back();
        GEN_CUDA(cudaMallocHost(reinterpret_cast<void**>(&g.hpin), 4 * sizeof(double)));
    }
    if (!same) {
        drop_pattern(g);
        g.n = n;
        g.nb = nb;
        g.nnzb = nnzb;
        g.rp0.assign(rowPtr, rowPtr + n + 1);
        g.ci0.assign(col, col + nnzb);
        std::string err;
        if (!build_plan(g.plan, 1, std::vector<int>{0, n}, g.rp0, g.ci0, err, host_threads())) return gfail(RSG_EINVAL, err);
        std::vector<int> dg(static_cast<size_t>(n));
        for (int i = 0; i < n; ++i)
            for (int p = rowPtr[i]; p < rowPtr[i + 1]; ++p)
                if (col[p] == i) { dg[size_t(i)] = p; break; }
        std::vector<int> fOrd, bOrd;
        level_sets(n, g.rp0, g.ci0, dg, true, fOrd, g.fStart);
        level_sets(n, g.rp0, g.ci0, dg, false, bOrd, g.bStart);
        // a system whose sweep fits one block at a few rows per thread runs each sweep in one launch
        int widest = 1;
        for (size_t l = 0; l + 1 < g.fStart.size(); ++l) widest = std::max(widest, g.fStart[l + 1] - g.fStart[l]);
        for (size_t l = 0; l + 1 < g.bStart.size(); ++l) widest = std::max(widest, g.bStart[l + 1] - g.bStart[l]);
        g.oneCta = (long long)widest * nb <= 4LL * kCtaThreads;
        int rc;
        if ((rc = gupload(g, &g.rp, g.rp0)) || (rc = gupload(g, &g.ci, g.ci0)) || (rc = gupload(g, &g.dg, dg)) ||
            (rc = gupload(g, &g.fOrd, fOrd)) || (rc = gupload(g, &g.bOrd, bOrd)) || (rc = gupload(g, &g.fLvl, g.fStart)) ||
            (rc = gupload(g, &g.bLvl, g.bStart)) || (rc = gupload(g, &g.valSrc, g.plan.valSrc)) || (rc = gupload(g, &g.perm0, g.plan.perm)) ||
            (rc = gupload(g, &g.iperm0, g.plan.iperm)))
            return rc;
        const size_t E = size_t(nnzb) * nb * nb, N = size_t(n) * nb;
        if ((rc = galloc(g, g.pat, g.bytesPat, &g.S, E)) || (rc = galloc(g, g.pat, g.bytesPat, &g.LU, E)) ||
            (rc = galloc(g, g.pat, g.bytesPat, &g.w, N)) || (rc = galloc(g, g.pat, g.bytesPat, &g.ap, size_t(nnzb))) ||
            (rc = galloc(g, g.pat, g.bytesPat, &g.T, N)))
            return rc;
    }
    GEN_CUDA(cudaMemcpyAsync(g.S, val, size_t(nnzb) * nb * nb * sizeof(double), cudaMemcpyHostToDevice, g.st));
    g.haveMatrix = true;
    g.haveSetup = false;
    return RSG_OK;
}

int gen_set_values_device(GenEngine* gp, const double* d_val) {
    GenEngine& g = *gp;
    if (!g.S) return gfail(RSG_ESTATE, "values before a pattern");
    GEN_CUDA(cudaMemcpyAsync(g.S, d_val, size_t(g.nnzb) * g.nb * g.nb * sizeof(double), cudaMemcpyDeviceToDevice, g.st));
    g.haveMatrix = true;
    g.haveSetup = false;
    return RSG_OK;
}

int gen_setup(GenEngine* gp, const rsg_options& o, const double* acc) {
    GenEngine& g = *gp;
    if (!g.haveMatrix) return gfail(RSG_ESTATE, "setup before set_matrix");
    const auto t0 = std::chrono::steady_clock::now();
    g.precond = o.precond;
    const int b2 = g.nb * g.nb;
    GEN_CUDA(cudaMemsetAsync(g.dCnt, 0, 2 * sizeof(int), g.st));
    if (g.precond == RSG_PREC_CPR) {
        if (!g.plan.symmetric) return gfail(RSG_EINVAL, "the CPR preconditioner needs a structurally symmetric pattern");
        double* dacc = nullptr;
        if (acc) {
            GEN_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&dacc), size_t(g.n) * b2 * sizeof(double), g.st));
            GEN_CUDA(cudaMemcpyAsync(dacc, acc, size_t(g.n) * b2 * sizeof(double), cudaMemcpyHostToDevice, g.st));
        }
        k_gen_weights<<<grid_of((long long)g.n * 32, kWarpsPerBlock * 32), kWarpsPerBlock * 32, 0, g.st>>>(g.n, g.nb, g.dg, g.S, dacc, g.w,
                                                                                                         g.dCnt + 1);
        k_gen_pressure<<<grid_of(g.n), 256, 0, g.st>>>(g.n, g.nb, g.rp, g.S, g.w, g.ap);
        g.launches += 2;
        if (dacc) cudaFreeAsync(dacc, g.st);
        if (!g.haveAmg) {
            // first set-up of this pattern: the aggregation on the host from the level-space pressure values
            std::vector<double> apo(static_cast<size_t>(g.nnzb)), ap0(static_cast<size_t>(g.nnzb));
            GEN_CUDA(cudaMemcpyAsync(apo.data(), g.ap, apo.size() * sizeof(double), cudaMemcpyDeviceToHost, g.st));
            GEN_CUDA(cudaStreamSynchronize(g.st));
            for (int p = 0; p < g.nnzb; ++p) ap0[size_t(p)] = apo[size_t(g.plan.valSrc[size_t(p)])];
            int rc = build_amg(g, ap0);
            if (rc) return rc;
        }
        refresh_amg(g);
    }
    GEN_CUDA(cudaMemcpyAsync(g.LU, g.S, size_t(g.nnzb) * b2 * sizeof(double), cudaMemcpyDeviceToDevice, g.st));
    const int nlf = int(g.fStart.size()) - 1;
    if (g.n <= 2048) {                                     // small: every level in one block
        k_gen_factor_cta<<<1, kWarpsPerBlock * 32, 0, g.st>>>(nlf, g.fLvl, g.fOrd, g.nb, g.rp, g.ci, g.dg, g.LU, g.dCnt);
        ++g.launches;
    } else {
        for (int l = 0; l < nlf; ++l) {
            const int r0 = g.fStart[size_t(l)], r1 = g.fStart[size_t(l) + 1];
            k_gen_factor_level<<<grid_of((long long)(r1 - r0) * 32, kWarpsPerBlock * 32), kWarpsPerBlock * 32, 0, g.st>>>(
                r0, r1, g.fOrd, g.nb, g.rp, g.ci, g.dg, g.LU, g.dCnt);
        }
        g.launches += nlf;
    }
    GEN_CUDA(cudaGetLastError());
    int cnt[2] = {0, 0};
    GEN_CUDA(cudaMemcpyAsync(cnt, g.dCnt, 2 * sizeof(int), cudaMemcpyDeviceToHost, g.st));
    GEN_CUDA(cudaStreamSynchronize(g.st));
    g.stt.regularised_blocks = cnt[0];
    g.stt.amg_levels = g.precond == RSG_PREC_CPR ? int(g.lv.size()) : 0;
    g.stt.setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    g.haveSetup = true;
    return RSG_OK;
}

int gen_solve_device(GenEngine* gp, const rsg_options& o, const double* d_b, double* d_x, double tol, int maxIt, int* its, double* relres) {
    GenEngine& g = *gp;
    if (!g.haveSetup) return gfail(RSG_ESTATE, "solve before setup");
    const auto t0 = std::chrono::steady_clock::now();
    const bool useGm = o.krylov == RSG_KRYLOV_GMRES;
    const int m = o.restart > 0 ? o.restart : 40;
    int rc = ensure_krylov(g, useGm || o.gmres_fallback, m);
    if (rc) return rc;
    const size_t N = size_t(g.n) * g.nb;
    GEN_CUDA(cudaMemcpyAsync(g.vb, d_b, N * sizeof(double), cudaMemcpyDeviceToDevice, g.st));
    int it = 0;
    double rr = 1;
    bool conv = false;
    rc = useGm ? gmres(g, tol, maxIt, m, &it, &rr, &conv) : bicgstab(g, tol, maxIt, &it, &rr, &conv);
    if (rc) return rc;
    if (!conv && !useGm && o.gmres_fallback) {            // engine/src/simulator.cpp:3388-3398: GMRES after BiCGSTAB
        GEN_CUDA(cudaMemcpyAsync(g.vrh, g.vx, N * sizeof(double), cudaMemcpyDeviceToDevice, g.st));
        int it2 = 0;
        double rr2 = 1;
        bool conv2 = false;
        if ((rc = gmres(g, tol, maxIt, m, &it2, &rr2, &conv2))) return rc;
        if (conv2 || rr2 < rr) { it += it2; rr = rr2; conv = conv2; }
        else GEN_CUDA(cudaMemcpyAsync(g.vx, g.vrh, N * sizeof(double), cudaMemcpyDeviceToDevice, g.st));
    }
    GEN_CUDA(cudaMemcpyAsync(d_x, g.vx, N * sizeof(double), cudaMemcpyDeviceToDevice, g.st));
    // true residual in FP64
    spmv(g, g.vx, g.vr);
    k_gen_sub_from<<<grid_of((long long)N), 256, 0, g.st>>>((long long)N, g.vb, g.vr);
    ++g.launches;
    double r2, b2;
    if ((rc = gdot(g, g.vr, g.vr, &r2)) || (rc = gdot(g, g.vb, g.vb, &b2))) return rc;
    GEN_CUDA(cudaGetLastError());
    const double tr = b2 > 0 ? std::sqrt(r2 / b2) : 0.0;
    g.stt.iterations = it;
    g.stt.converged = conv ? 1 : 0;
    g.stt.rel_residual = rr;
    g.stt.true_rel_residual = tr;
    g.stt.solve_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (its) *its = it;
    if (relres) *relres = rr;
    if (!std::isfinite(tr)) return gfail(RSG_ENOTCONV, "non-finite solution");
    return conv ? RSG_OK : RSG_ENOTCONV;
}

namespace {
int ensure_staging(GenEngine& g) {
    if (g.stIn) return RSG_OK;
    const size_t N = size_t(g.n) * g.nb;
    int rc;
    if ((rc = galloc(g, g.pat, g.bytesPat, &g.stIn, N)) || (rc = galloc(g, g.pat, g.bytesPat, &g.stOut, N))) return rc;
    return RSG_OK;
}
}  // namespace

int gen_solve_host(GenEngine* gp, const rsg_options& o, const double* b, double* x, double tol, int maxIt, int* its, double* relres) {
    GenEngine& g = *gp;
    if (!g.haveSetup) return gfail(RSG_ESTATE, "solve before setup");
    int rc = ensure_staging(g);
    if (rc) return rc;
    const size_t N = size_t(g.n) * g.nb;
    GEN_CUDA(cudaMemcpyAsync(g.stIn, b, N * sizeof(double), cudaMemcpyHostToDevice, g.st));
    rc = gen_solve_device(gp, o, g.stIn, g.stOut, tol, maxIt, its, relres);
    if (rc < 0) return rc;
    GEN_CUDA(cudaMemcpyAsync(x, g.stOut, N * sizeof(double), cudaMemcpyDeviceToHost, g.st));
    GEN_CUDA(cudaStreamSynchronize(g.st));
    return rc;
}

int gen_spmv_host(GenEngine* gp, const double* x, double* y) {
    GenEngine& g = *gp;
    if (!g.haveMatrix) return gfail(RSG_ESTATE, "spmv before set_matrix");
    int rc = ensure_staging(g);
    if (rc) return rc;
    const size_t N = size_t(g.n) * g.nb;
    GEN_CUDA(cudaMemcpyAsync(g.stIn, x, N * sizeof(double), cudaMemcpyHostToDevice, g.st));
    spmv(g, g.stIn, g.stOut);
    GEN_CUDA(cudaGetLastError());
    GEN_CUDA(cudaMemcpyAsync(y, g.stOut, N * sizeof(double), cudaMemcpyDeviceToHost, g.st));
    GEN_CUDA(cudaStreamSynchronize(g.st));
    return RSG_OK;
}

int gen_precond_host(GenEngine* gp, const double* r, double* z) {
    GenEngine& g = *gp;
    if (!g.haveSetup) return gfail(RSG_ESTATE, "precond_apply before setup");
    int rc = ensure_staging(g);
    if (rc) return rc;
    const size_t N = size_t(g.n) * g.nb;
    GEN_CUDA(cudaMemcpyAsync(g.stIn, r, N * sizeof(double), cudaMemcpyHostToDevice, g.st));
    precond(g, g.stIn, g.stOut);
    GEN_CUDA(cudaGetLastError());
    GEN_CUDA(cudaMemcpyAsync(z, g.stOut, N * sizeof(double), cudaMemcpyDeviceToHost, g.st));
    GEN_CUDA(cudaStreamSynchronize(g.st));
    return RSG_OK;
}

int gen_spmv_device(GenEngine* gp, const double* d_x, double* d_y) {
    GenEngine& g = *gp;
    if (!g.haveMatrix) return gfail(RSG_ESTATE, "spmv before set_matrix");
    spmv(g, d_x, d_y);
    GEN_CUDA(cudaGetLastError());
    return RSG_OK;
}

int gen_precond_device(GenEngine* gp, const double* d_r, double* d_z) {
    GenEngine& g = *gp;
    if (!g.haveSetup) return gfail(RSG_ESTATE, "precond_apply before setup");
    precond(g, d_r, d_z);
    GEN_CUDA(cudaGetLastError());
    return RSG_OK;
}

int gen_get_factors(GenEngine* gp, double* lu) {
    GenEngine& g = *gp;
    if (!g.haveSetup) return gfail(RSG_ESTATE, "no BILU0 factors (setup not run)");
    GEN_CUDA(cudaMemcpyAsync(lu, g.LU, size_t(g.nnzb) * g.nb * g.nb * sizeof(double), cudaMemcpyDeviceToHost, g.st));
    GEN_CUDA(cudaStreamSynchronize(g.st));
    return RSG_OK;
}

void gen_stats(const GenEngine* g, rsg_stats* st) {
    *st = g->stt;
    st->device_bytes = g->bytesPat + g->bytesVal;
    st->kernel_launches = g->launches;
}

int gen_rows(const GenEngine* g) { return g->n * g->nb; }
bool gen_ready(const GenEngine* g) { return g && g->haveMatrix; }
bool gen_have_setup(const GenEngine* g) { return g && g->haveSetup; }

int gen_amg_level_sizes(const GenEngine* g, int maxlev, long long* rows, long long* nnz, long long* dense) {
    if (!g->haveAmg) return gfail(RSG_ESTATE, "no CPR hierarchy (setup not run, or not a CPR preconditioner)");
    const int nl = std::min(maxlev, int(g->lv.size()));
    for (int l = 0; l < nl; ++l) {
        rows[l] = g->lv[size_t(l)].n;
        nnz[l] = g->lv[size_t(l)].nnz;
    }
    if (dense) *dense = g->lv.back().dense ? (long long)g->lv.back().n * g->lv.back().n : 0;
    return int(g->lv.size());
}

}  // namespace rsg
