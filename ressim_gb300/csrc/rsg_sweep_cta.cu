// Thread-block-per-system BILU0 application: exact natural-order ILU(0) sweeps for systems that fit one SM.
//
// One thread block owns one system of the (block-diagonal) batch and walks its forward levels with a block
// barrier between levels, then the same levels in reverse for the backward sweep (valid for the structurally
// symmetric patterns of reservoir Jacobians; otherwise the plan uses the grid-wide sync-free sweeps). Rows are
// in level space, so a level is a contiguous range of rows, of input vector entries and of split factor blocks.
//
// * The sweep vector y stays on chip between the two sweeps when it fits the block's shared memory (chosen per
//   system at run time), else it lives in the output vector itself (L1 / L2).
// * Each thread prefetches, one row ahead, the next row's input entries, row pointers, column indices and up to
//   kPre factor blocks into registers: the global-memory latency of a level overlaps the previous level's work
//   and barrier, and only the dependency reads of y stay on the critical path.
// * TF = factor storage type, TV = sweep vector type. FP64 (double, double) and mixed (float factors, double
//   vector: the reference's float-factor sweeps, engine/src/bsr.cpp:500-522) use unfused multiply / add in the
//   reference loop order, so their results are bitwise those of the reference's serial sweeps on the same
//   factors. (float, float) is the all-FP32 BILU0f sweep (engine/src/bsr.cpp:1100-1121).
#include "rsg_impl.h"

#include <cuda_runtime.h>
#include <type_traits>

namespace rsg {

namespace {

constexpr int kCtaThreads = 256;
constexpr int kPre = 3;                    // factor blocks per row prefetched into registers (7-point: all of L or U)

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

// one row of a 3x3 block (factor type TF) times a 3-vector of type TV, accumulated from zero left to right
__device__ __forceinline__ double rdot(const double* a, const double* x) { return da(da(dm(a[0], x[0]), dm(a[1], x[1])), dm(a[2], x[2])); }
__device__ __forceinline__ double rdot(const float* a, const double* x) {
    return da(da(dm(double(a[0]), x[0]), dm(double(a[1]), x[1])), dm(double(a[2]), x[2]));
}
__device__ __forceinline__ float rdot(const float* a, const float* x) {
    float s = 0.f;
    s += a[0] * x[0];
    s += a[1] * x[1];
    s += a[2] * x[2];
    return s;
}
__device__ __forceinline__ double vsub(double a, double b) { return ds(a, b); }
__device__ __forceinline__ float vsub(float a, float b) { return a - b; }

enum { IN_PLAIN = 0, IN_PUPDATE = 1, IN_SUPDATE = 2 };

// registers holding one row's prefetched data
template <class TF, int MODE>
struct RowPre {
    int k = -1, p0 = 0, p1 = 0;
    int c[kPre];
    TF a[kPre][9];
    double in[MODE == IN_PUPDATE ? 9 : (MODE == IN_SUPDATE ? 6 : 3)];
};
template <class TF>
struct RowPreB {
    int k = -1, p0 = 0, p1 = 0;
    int c[kPre];
    TF a[kPre][9];
    TF d[9];
};

template <class TF, int MODE>
__device__ __forceinline__ void prefetch_fwd(RowPre<TF, MODE>& R, int k, const int* __restrict__ Lptr, const int* __restrict__ Lcol,
                                             const TF* __restrict__ Lv, const double* r, const double* pv, const double* v) {
    R.k = k;
    if (k < 0) return;
    R.p0 = __ldg(Lptr + k);
    R.p1 = __ldg(Lptr + k + 1);
#pragma unroll
    for (int j = 0; j < kPre; ++j)
        if (R.p0 + j < R.p1) {
            R.c[j] = __ldg(Lcol + R.p0 + j);
#pragma unroll
            for (int e = 0; e < 9; ++e) R.a[j][e] = __ldg(Lv + size_t(R.p0 + j) * 9 + e);
        }
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const size_t q = size_t(k) * 3 + e;
        R.in[e] = r[q];
        if (MODE == IN_PUPDATE) { R.in[3 + e] = pv[q]; R.in[6 + e] = v[q]; }
        if (MODE == IN_SUPDATE) R.in[3 + e] = v[q];
    }
}

template <class TF>
__device__ __forceinline__ void prefetch_bwd(RowPreB<TF>& R, int k, const int* __restrict__ Uptr, const int* __restrict__ Ucol,
                                             const TF* __restrict__ Uv, const TF* __restrict__ Dv) {
    R.k = k;
    if (k < 0) return;
    R.p0 = __ldg(Uptr + k);
    R.p1 = __ldg(Uptr + k + 1);
#pragma unroll
    for (int j = 0; j < kPre; ++j)
        if (R.p0 + j < R.p1) {
            R.c[j] = __ldg(Ucol + R.p0 + j);
#pragma unroll
            for (int e = 0; e < 9; ++e) R.a[j][e] = __ldg(Uv + size_t(R.p0 + j) * 9 + e);
        }
#pragma unroll
    for (int e = 0; e < 9; ++e) R.d[e] = __ldg(Dv + size_t(k) * 9 + e);
}

template <class TF, class TV>
__device__ __forceinline__ void sub_block(TV (&yi)[3], const TF* a, const TV* y, int c) {
    const TV yc[3] = {y[c * 3 + 0], y[c * 3 + 1], y[c * 3 + 2]};
    yi[0] = vsub(yi[0], rdot(a, yc));
    yi[1] = vsub(yi[1], rdot(a + 3, yc));
    yi[2] = vsub(yi[2], rdot(a + 6, yc));
}

// the thread's next row after row k of level L (the next one of the same level, else its first of level L+1)
__device__ __forceinline__ int next_row(int k, int k1, int L, int nl, int l0, const int* __restrict__ lvlStart, int forward) {
    if (k + int(blockDim.x) < k1) return k + int(blockDim.x);
    const int Ln = forward ? L + 1 : L - 1;
    if (Ln < 0 || Ln >= nl) return -1;
    const int a = __ldg(lvlStart + l0 + Ln) + int(threadIdx.x);
    return a < __ldg(lvlStart + l0 + Ln + 1) ? a : -1;
}

// Both sweeps of one system by the calling thread block (y: the sweep vector of this system, on chip or in z).
template <class TF, class TV, int MODE>
__device__ void ilu_body(int row0, int l0, int nl, const int* __restrict__ lvlStart, const int* __restrict__ Lptr,
                         const int* __restrict__ Lcol, const TF* __restrict__ Lv, const int* __restrict__ Uptr,
                         const int* __restrict__ Ucol, const TF* __restrict__ Uv, const TF* __restrict__ Dv, const double* r, double* pv,
                         const double* v, double* z, TV* y, bool writeZ, double beta, double omega, double alpha) {
    const int tid = int(threadIdx.x);
    // ---- forward: y_i = in_i - sum_{k<i} L_ik y_k (engine/src/bsr.cpp:568-575), level by level
    RowPre<TF, MODE> cur, nxt;
    {
        const int a = nl > 0 ? __ldg(lvlStart + l0) + tid : -1;
        prefetch_fwd(cur, (nl > 0 && a < __ldg(lvlStart + l0 + 1)) ? a : -1, Lptr, Lcol, Lv, r, pv, v);
    }
    for (int L = 0; L < nl; ++L) {
        const int k1 = __ldg(lvlStart + l0 + L + 1);
        for (int k = __ldg(lvlStart + l0 + L) + tid; k < k1; k += blockDim.x) {
            if (cur.k != k) prefetch_fwd(cur, k, Lptr, Lcol, Lv, r, pv, v);
            prefetch_fwd(nxt, next_row(k, k1, L, nl, l0, lvlStart, 1), Lptr, Lcol, Lv, r, pv, v);
            TV yi[3];
#pragma unroll
            for (int e = 0; e < 3; ++e) {
                const size_t q = size_t(k) * 3 + e;
                if (MODE == IN_PUPDATE) {
                    const double pe = da(cur.in[e], dm(beta, ds(cur.in[3 + e], dm(omega, cur.in[6 + e]))));   // linsolve.cpp:173
                    pv[q] = pe;
                    yi[e] = TV(pe);
                } else if (MODE == IN_SUPDATE) {
                    const double se = ds(cur.in[e], dm(alpha, cur.in[3 + e]));                               // linsolve.cpp:183
                    pv[q] = se;
                    yi[e] = TV(se);
                } else {
                    yi[e] = TV(cur.in[e]);
                }
            }
#pragma unroll
            for (int j = 0; j < kPre; ++j)
                if (cur.p0 + j < cur.p1) sub_block(yi, cur.a[j], y, cur.c[j]);
            for (int p = cur.p0 + kPre; p < cur.p1; ++p) {     // long rows (well fill): the rest on demand
                TF a[9];
#pragma unroll
                for (int e = 0; e < 9; ++e) a[e] = __ldg(Lv + size_t(p) * 9 + e);
                sub_block(yi, a, y, __ldg(Lcol + p));
            }
            const int li = k - row0;
            y[li * 3 + 0] = yi[0]; y[li * 3 + 1] = yi[1]; y[li * 3 + 2] = yi[2];
            cur = nxt;
        }
        __syncthreads();
    }
    // ---- backward: z_i = U_ii^-1 (y_i - sum_{j>i} U_ij z_j) (engine/src/bsr.cpp:577-587), levels in reverse
    RowPreB<TF> bc, bn;
    {
        const int a = nl > 0 ? __ldg(lvlStart + l0 + nl - 1) + tid : -1;
        prefetch_bwd(bc, (nl > 0 && a < __ldg(lvlStart + l0 + nl)) ? a : -1, Uptr, Ucol, Uv, Dv);
    }
    for (int L = nl - 1; L >= 0; --L) {
        const int k1 = __ldg(lvlStart + l0 + L + 1);
        for (int k = __ldg(lvlStart + l0 + L) + tid; k < k1; k += blockDim.x) {
            if (bc.k != k) prefetch_bwd(bc, k, Uptr, Ucol, Uv, Dv);
            prefetch_bwd(bn, next_row(k, k1, L, nl, l0, lvlStart, 0), Uptr, Ucol, Uv, Dv);
            const int li = k - row0;
            TV yi[3] = {y[li * 3 + 0], y[li * 3 + 1], y[li * 3 + 2]};
#pragma unroll
            for (int j = 0; j < kPre; ++j)
                if (bc.p0 + j < bc.p1) sub_block(yi, bc.a[j], y, bc.c[j]);
            for (int p = bc.p0 + kPre; p < bc.p1; ++p) {
                TF a[9];
#pragma unroll
                for (int e = 0; e < 9; ++e) a[e] = __ldg(Uv + size_t(p) * 9 + e);
                sub_block(yi, a, y, __ldg(Ucol + p));
            }
            const TV t0 = rdot(bc.d, yi), t1 = rdot(bc.d + 3, yi), t2 = rdot(bc.d + 6, yi);
            y[li * 3 + 0] = t0; y[li * 3 + 1] = t1; y[li * 3 + 2] = t2;
            if (writeZ) {
                z[size_t(k) * 3 + 0] = double(t0);
                z[size_t(k) * 3 + 1] = double(t1);
                z[size_t(k) * 3 + 2] = double(t2);
            }
            bc = bn;
        }
        __syncthreads();
    }
}

template <class TF, class TV, int MODE>
__global__ void __launch_bounds__(kCtaThreads) k_ilu_cta(const int* __restrict__ sysRow0, const int* __restrict__ sysLvl0,
                                                        const int* __restrict__ lvlStart, const int* __restrict__ Lptr,
                                                        const int* __restrict__ Lcol, const TF* __restrict__ Lv,
                                                        const int* __restrict__ Uptr, const int* __restrict__ Ucol,
                                                        const TF* __restrict__ Uv, const TF* __restrict__ Dv, const double* r, double* pv,
                                                        const double* v, double* z, TV* yglob, size_t smemBytes, const KScal* ks) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int s = blockIdx.x;
    const int row0 = __ldg(sysRow0 + s), ns = __ldg(sysRow0 + s + 1) - row0;
    double beta = 0, omega = 0, alpha = 0;
    if (ks) {
        const KScal& K = ks[s];
        if (K.status != ST_RUNNING) return;                // whole block: uniform
        beta = K.beta; omega = K.omega; alpha = K.alpha;
    }
    // sweep vector: on chip when it fits, else global (yglob: z itself for TV = double)
    const bool onchip = size_t(ns) * 3 * sizeof(TV) <= smemBytes;
    TV* y = onchip ? reinterpret_cast<TV*>(smraw) : yglob + size_t(row0) * 3;
    const int l0 = __ldg(sysLvl0 + s), nl = __ldg(sysLvl0 + s + 1) - l0 - 1;
    ilu_body<TF, TV, MODE>(row0, l0, nl, lvlStart, Lptr, Lcol, Lv, Uptr, Ucol, Uv, Dv, r, pv, v, z, y,
                           onchip || sizeof(TV) != sizeof(double), beta, omega, alpha);
}

// ------------------------------------------------------------------ CPR (BlockCPR::apply, engine/src/bsr.cpp:1061-1084)
struct AmgArgs {
    const AmgSysLv* lv;
    int maxL;
    const int *rp, *ci, *diag, *lvl, *agg, *memPtr, *mem, *luPerm, *piv;
};

// V-cycle arithmetic type: FP64 explicitly rounded (bitwise the reference) or FP32
__device__ __forceinline__ double amul(double a, double b) { return dm(a, b); }
__device__ __forceinline__ double aadd(double a, double b) { return da(a, b); }
__device__ __forceinline__ double asub(double a, double b) { return ds(a, b); }
__device__ __forceinline__ double adiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float amul(float a, float b) { return a * b; }
__device__ __forceinline__ float aadd(float a, float b) { return a + b; }
__device__ __forceinline__ float asub(float a, float b) { return a - b; }
__device__ __forceinline__ float adiv(float a, float b) { return a / b; }

// Gauss-Seidel sweep of one level (engine/src/amg.cpp:98-113) over its GS levels: forward from x = 0 (only the
// lower entries contribute, bitwise the full sum), or forward / backward from the current x (full rows: entries of
// later rows still hold the old x). Rows of one GS level are independent.
template <class TA>
__device__ void gs_sweep(const AmgSysLv& A, const AmgArgs& G, const TA* __restrict__ val, TA* x, const TA* b, bool forward, bool fromZero) {
    const int* rp = G.rp + A.rpOff;
    const int* ci = G.ci + A.entOff;
    const int* dg = G.diag + A.rowOff;
    const int* lv = G.lvl + A.lvlOff;
    const TA* v = val + A.entOff;
    for (int g = 0; g < A.nl; ++g) {
        const int L = forward ? g : A.nl - 1 - g;
        const int k1 = __ldg(lv + L + 1);
        for (int k = __ldg(lv + L) + int(threadIdx.x); k < k1; k += blockDim.x) {
            const int d = __ldg(dg + k);
            const int pe = fromZero ? d : __ldg(rp + k + 1);
            TA s = b[k];
            for (int p = __ldg(rp + k); p < pe; ++p)
                if (p != d) s = asub(s, amul(v[p], x[__ldg(ci + p)]));
            x[k] = adiv(s, v[d]);
        }
        __syncthreads();
    }
}

// coarsest level: x = LU^-1 b with the dense LU of the natural numbering (engine/src/amg.cpp:306-312), one warp;
// work = the level's residual vector, used in natural order
template <class TA>
__device__ void coarse_solve(const AmgSysLv& A, const AmgArgs& G, const TA* __restrict__ luAll, TA* x, const TA* b, TA* work) {
    const int m = A.n;
    const TA* lu = luAll + A.luOff;
    const int* nat = G.luPerm + A.luRowOff;
    const int* piv = G.piv + A.luRowOff;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        for (int k = lane; k < m; k += 32) work[__ldg(nat + k)] = b[k];
        __syncwarp();
        if (lane == 0)
            for (int k = 0; k < m; ++k) {
                const int pk = __ldg(piv + k);
                if (pk != k) { const TA t = work[k]; work[k] = work[pk]; work[pk] = t; }
            }
        __syncwarp();
        for (int j = 0; j < m; ++j) {                    // unit lower: every row gets its terms in ascending j
            const TA xj = work[j];
            for (int i = j + 1 + lane; i < m; i += 32) work[i] = asub(work[i], amul(lu[size_t(i) * m + j], xj));
            __syncwarp();
        }
        for (int j = m - 1; j >= 0; --j) {               // upper
            if (lane == 0) work[j] = adiv(work[j], lu[size_t(j) * m + j]);
            __syncwarp();
            const TA xj = work[j];
            for (int i = lane; i < j; i += 32) work[i] = asub(work[i], amul(lu[size_t(i) * m + j], xj));
            __syncwarp();
        }
        for (int k = lane; k < m; k += 32) x[k] = work[__ldg(nat + k)];
    }
    __syncthreads();
}

// AMG::cycle (engine/src/amg.cpp:303-329) for system s, level 0 rhs in b + lv[0].rowOff
template <class TA>
__device__ void vcycle(int s, const AmgArgs& G, const TA* __restrict__ val, const TA* __restrict__ lu, TA* x, TA* b, TA* r) {
    int nlev = 0;
    while (nlev < G.maxL && G.lv[s * G.maxL + nlev].n > 0) ++nlev;
    int l = 0;
    for (; l < nlev; ++l) {
        const AmgSysLv A = G.lv[s * G.maxL + l];
        TA* xl = x + A.rowOff;
        TA* bl = b + A.rowOff;
        TA* rl = r + A.rowOff;
        if (A.coarse) {
            if (A.dense) {
                coarse_solve(A, G, lu, xl, bl, rl);
            } else {                                      // 20 symmetric GS sweeps from x = 0 (amg.cpp:313-315)
                for (int k = threadIdx.x; k < A.n; k += blockDim.x) xl[k] = TA(0);
                __syncthreads();
                for (int it = 0; it < 20; ++it) {
                    gs_sweep(A, G, val, xl, bl, true, false);
                    gs_sweep(A, G, val, xl, bl, false, false);
                }
            }
            break;
        }
        gs_sweep(A, G, val, xl, bl, true, true);
        // residual r = b - A x (amg.cpp:321-322)
        {
            const int* rp = G.rp + A.rpOff;
            const int* ci = G.ci + A.entOff;
            const TA* v = val + A.entOff;
            for (int k = threadIdx.x; k < A.n; k += blockDim.x) {
                TA t = TA(0);
                for (int p = __ldg(rp + k); p < __ldg(rp + k + 1); ++p) t = aadd(t, amul(v[p], xl[__ldg(ci + p)]));
                rl[k] = asub(bl[k], t);
            }
        }
        __syncthreads();
        // restriction b_{l+1} = R r: members in ascending natural order (amg.cpp:324)
        {
            const AmgSysLv C = G.lv[s * G.maxL + l + 1];
            const int* mp = G.memPtr + C.rpOff;
            const int* mem = G.mem + C.memOff;
            TA* bc = b + C.rowOff;
            for (int I = threadIdx.x; I < C.n; I += blockDim.x) {
                TA t = TA(0);
                for (int q = __ldg(mp + I); q < __ldg(mp + I + 1); ++q) t = aadd(t, rl[__ldg(mem + q)]);
                bc[I] = t;
            }
        }
        __syncthreads();
    }
    for (l = l - 1; l >= 0; --l) {                          // prolongation and post-smoothing (amg.cpp:326-327)
        const AmgSysLv A = G.lv[s * G.maxL + l];
        const AmgSysLv C = G.lv[s * G.maxL + l + 1];
        TA* xl = x + A.rowOff;
        const TA* xc = x + C.rowOff;
        const int* agg = G.agg + A.rowOff;
        for (int k = threadIdx.x; k < A.n; k += blockDim.x) xl[k] = aadd(xl[k], xc[__ldg(agg + k)]);
        __syncthreads();
        gs_sweep(A, G, val, xl, b + A.rowOff, false, false);
    }
}

template <class TF, class TV, class TA, int MODE>
__global__ void __launch_bounds__(kCtaThreads) k_cpr_cta(const int* __restrict__ sysRow0, const int* __restrict__ sysLvl0,
                                                        const int* __restrict__ lvlStart, const int* __restrict__ Lptr,
                                                        const int* __restrict__ Lcol, const TF* __restrict__ Lv,
                                                        const int* __restrict__ Uptr, const int* __restrict__ Ucol,
                                                        const TF* __restrict__ Uv, const TF* __restrict__ Dv,
                                                        const int* __restrict__ rowPtr, const int* __restrict__ col,
                                                        const double* __restrict__ val, const double* __restrict__ w, double* T,
                                                        AmgArgs G, const TA* __restrict__ aval, const TA* __restrict__ alu, TA* ax, TA* ab,
                                                        TA* ar, const double* r, double* pv, const double* v, double* z, TV* yglob,
                                                        size_t smemBytes, const KScal* ks) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int s = blockIdx.x;
    const int row0 = __ldg(sysRow0 + s), ns = __ldg(sysRow0 + s + 1) - row0;
    double beta = 0, omega = 0, alpha = 0;
    if (ks) {
        const KScal& K = ks[s];
        if (K.status != ST_RUNNING) return;
        beta = K.beta; omega = K.omega; alpha = K.alpha;
    }
    const AmgSysLv A0 = G.lv[s * G.maxL];
    TA* b0 = ab + A0.rowOff;
    const TA* xp = ax + A0.rowOff;
    // input (fused Krylov update) and pressure restriction rp = w . r (bsr.cpp:1064-1067)
    for (int k = row0 + int(threadIdx.x); k < row0 + ns; k += blockDim.x) {
        double in[3];
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            const size_t q = size_t(k) * 3 + e;
            if (MODE == IN_PUPDATE) { in[e] = da(r[q], dm(beta, ds(pv[q], dm(omega, v[q])))); pv[q] = in[e]; }
            else if (MODE == IN_SUPDATE) { in[e] = ds(r[q], dm(alpha, v[q])); pv[q] = in[e]; }
            else in[e] = r[q];
            T[q] = in[e];
        }
        const double* wk = w + size_t(k) * 3;
        b0[k - row0] = TA(da(da(dm(wk[0], in[0]), dm(wk[1], in[1])), dm(wk[2], in[2])));
    }
    __syncthreads();
    vcycle<TA>(s, G, aval, alu, ax, ab, ar);
    // second stage on t = r - S[:,p] xp (pressure column only, bsr.cpp:1071-1081)
    for (int k = row0 + int(threadIdx.x); k < row0 + ns; k += blockDim.x) {
        double acc[3] = {T[size_t(k) * 3], T[size_t(k) * 3 + 1], T[size_t(k) * 3 + 2]};
        for (int p = __ldg(rowPtr + k); p < __ldg(rowPtr + k + 1); ++p) {
            const double xk = double(xp[__ldg(col + p) - row0]);
            const double* B = val + size_t(p) * 9;
            acc[0] = ds(acc[0], dm(__ldg(B), xk));
            acc[1] = ds(acc[1], dm(__ldg(B + 3), xk));
            acc[2] = ds(acc[2], dm(__ldg(B + 6), xk));
        }
        T[size_t(k) * 3] = acc[0]; T[size_t(k) * 3 + 1] = acc[1]; T[size_t(k) * 3 + 2] = acc[2];
    }
    __syncthreads();
    const bool onchip = size_t(ns) * 3 * sizeof(TV) <= smemBytes;
    TV* y = onchip ? reinterpret_cast<TV*>(smraw) : yglob + size_t(row0) * 3;
    const int l0 = __ldg(sysLvl0 + s), nl = __ldg(sysLvl0 + s + 1) - l0 - 1;
    ilu_body<TF, TV, IN_PLAIN>(row0, l0, nl, lvlStart, Lptr, Lcol, Lv, Uptr, Ucol, Uv, Dv, T, nullptr, nullptr, z, y,
                               onchip || sizeof(TV) != sizeof(double), 0, 0, 0);
    // z_p += xp (bsr.cpp:1083)
    for (int k = row0 + int(threadIdx.x); k < row0 + ns; k += blockDim.x) z[size_t(k) * 3] = da(z[size_t(k) * 3], double(xp[k - row0]));
}



template <class T>
__global__ void k_pack(int n, int nL, int nU, const int* __restrict__ Lsrc, const int* __restrict__ Usrc, const int* __restrict__ Dsrc,
                       const T* __restrict__ lu, T* L, T* U, T* D) {
    const size_t total = (size_t(nL) + size_t(nU) + size_t(n)) * 9;
    for (size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x; q < total; q += size_t(gridDim.x) * blockDim.x) {
        const size_t b = q / 9, e = q % 9;
        if (b < size_t(nL)) L[q] = lu[size_t(__ldg(Lsrc + b)) * 9 + e];
        else if (b < size_t(nL) + size_t(nU)) { const size_t bb = b - nL; U[bb * 9 + e] = lu[size_t(__ldg(Usrc + bb)) * 9 + e]; }
        else { const size_t bb = b - nL - nU; D[bb * 9 + e] = lu[size_t(__ldg(Dsrc + bb)) * 9 + e]; }
    }
}

int max_smem_optin() {
    static int v = 0;
    if (!v) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (v <= 0) v = 48 * 1024;
    }
    return v;
}

template <class TF, class TV, int MODE>
void launch_cta(const DevPlan& P, const TF* L, const TF* U, const TF* D, size_t smem, const double* r, double* pv, const double* v,
                double* z, TV* yglob, const KScal* ks, cudaStream_t st) {
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaFuncSetAttribute(k_ilu_cta<TF, TV, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        configured = smem;
    }
    k_ilu_cta<TF, TV, MODE><<<P.nsys, kCtaThreads, smem, st>>>(P.sysRow0, P.sysLvl0, P.lvlStart, P.Lptr, P.Lcol, L, P.Uptr, P.Ucol, U, D,
                                                               r, pv, v, z, yglob, smem, ks);
}

template <int MODE>
void dispatch(const DevPlan& P, const PrecDev& M, const double* r, double* pv, const double* v, double* z, const KScal* ks,
              cudaStream_t st) {
    if (M.kind == 0) launch_cta<double, double, MODE>(P, M.s64.L, M.s64.U, M.s64.D, M.smem, r, pv, v, z, z, ks, st);
    else if (M.kind == 1) launch_cta<float, double, MODE>(P, M.s32.L, M.s32.U, M.s32.D, M.smem, r, pv, v, z, z, ks, st);
    else launch_cta<float, float, MODE>(P, M.s32.L, M.s32.U, M.s32.D, M.smem, r, pv, v, z, M.y32, ks, st);
}

}  // namespace

size_t cta_sweep_smem(const DevPlan& P, bool vec32) {
    // the largest system's vector if it fits, else all the opt-in shared memory (systems that fit use it)
    const size_t need = size_t(P.maxSysRows) * 3 * (vec32 ? sizeof(float) : sizeof(double));
    const size_t cap = size_t(max_smem_optin());
    return need <= cap ? need : cap;
}

bool cta_sweep_supported(const DevPlan& P, const HostPlan& H) {
    // structurally symmetric (reversed forward levels are backward levels) and small enough for one SM
    return H.symmetric && P.maxSysRows > 0 && P.maxSysRows <= 65536;
}

void launch_pack_f64(const DevPlan& P, const double* lu, SplitFactors<double>& F, cudaStream_t st) {
    const size_t total = (size_t(P.nL) + size_t(P.nU) + size_t(P.n)) * 9;
    const int grid = int(std::min<size_t>((total + 255) / 256, size_t(device_sm_count()) * 16));
    k_pack<double><<<grid, 256, 0, st>>>(P.n, P.nL, P.nU, P.Lsrc, P.Usrc, P.Dsrc, lu, F.L, F.U, F.D);
}
void launch_pack_f32(const DevPlan& P, const float* luf, SplitFactors<float>& F, cudaStream_t st) {
    const size_t total = (size_t(P.nL) + size_t(P.nU) + size_t(P.n)) * 9;
    const int grid = int(std::min<size_t>((total + 255) / 256, size_t(device_sm_count()) * 16));
    k_pack<float><<<grid, 256, 0, st>>>(P.n, P.nL, P.nU, P.Lsrc, P.Usrc, P.Dsrc, luf, F.L, F.U, F.D);
}

void launch_ilu_cta_apply(const DevPlan& P, const PrecDev& M, const double* r, double* z, cudaStream_t st) {
    dispatch<IN_PLAIN>(P, M, r, nullptr, nullptr, z, nullptr, st);
}

void launch_ilu_cta_fused(const DevPlan& P, const PrecDev& M, bool pupdate, const double* r, double* pv, const double* v, double* z,
                          const KScal* ks, cudaStream_t st) {
    if (pupdate) dispatch<IN_PUPDATE>(P, M, r, pv, v, z, ks, st);
    else dispatch<IN_SUPDATE>(P, M, r, pv, v, z, ks, st);
}

}  // namespace rsg

namespace rsg {
namespace {
template <class TF, class TV, class TA, int MODE>
void launch_cpr_t(const DevPlan& P, const double* Sval, const TF* Lf, const TF* Uf, const TF* Df, size_t smem, const DevAmg& G, const TA* aval, const TA* alu,
                  TA* ax, TA* ab, TA* ar, const double* r, double* pv, const double* v, double* z, TV* yglob, const KScal* ks,
                  cudaStream_t st) {
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaFuncSetAttribute(k_cpr_cta<TF, TV, TA, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        configured = smem;
    }
    AmgArgs A{G.lv, G.maxL, G.rp, G.ci, G.diag, G.lvl, G.agg, G.memPtr, G.mem, G.luPerm, G.piv};
    k_cpr_cta<TF, TV, TA, MODE><<<P.nsys, kCtaThreads, smem, st>>>(P.sysRow0, P.sysLvl0, P.lvlStart, P.Lptr, P.Lcol, Lf, P.Uptr, P.Ucol, Uf,
                                                                  Df, P.rowPtr, P.col, Sval, G.w, G.T, A, aval, alu, ax, ab, ar, r,
                                                                  pv, v, z, yglob, smem, ks);
}
}  // namespace

void launch_cpr_cta(const DevPlan& P, const PrecDev& M, const DevAmg& G, int mode, bool amgFp32, const double* r, double* pv,
                    const double* v, double* z, const KScal* ks, cudaStream_t st) {
    (void)amgFp32;
    const double* S = M.val;
    auto go = [&](auto tag_mode) {
        constexpr int MODE = decltype(tag_mode)::value;
        if (M.kind == 0)
            launch_cpr_t<double, double, double, MODE>(P, S, M.s64.L, M.s64.U, M.s64.D, M.smem, G, G.val, G.lu, G.x, G.b, G.r, r, pv, v, z, z,
                                                      ks, st);
        else if (M.kind == 1)
            launch_cpr_t<float, double, float, MODE>(P, S, M.s32.L, M.s32.U, M.s32.D, M.smem, G, G.valf, G.luf, G.xf, G.bf, G.rf, r, pv, v, z,
                                                    z, ks, st);
        else
            launch_cpr_t<float, float, float, MODE>(P, S, M.s32.L, M.s32.U, M.s32.D, M.smem, G, G.valf, G.luf, G.xf, G.bf, G.rf, r, pv, v, z,
                                                   M.y32, ks, st);
    };
    (void)S;
    if (mode == IN_PUPDATE) go(std::integral_constant<int, IN_PUPDATE>());
    else if (mode == IN_SUPDATE) go(std::integral_constant<int, IN_SUPDATE>());
    else go(std::integral_constant<int, IN_PLAIN>());
}

}  // namespace rsg
