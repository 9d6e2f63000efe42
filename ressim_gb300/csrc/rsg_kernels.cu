// Device kernels of the rsg solver (sm_103a).
//
// * BILU0 factorisation and the forward / backward sweeps are exact natural-order ILU(0): rows are processed in
//   a level order (a topological order of the L, resp. U, dependencies) by a persistent grid whose warps claim
//   32 rows at a time from an atomic counter; a row waits for the rows it depends on through per-row flags
//   (relaxed polls, one acquire fence, a release store when the row is done: rsg_sync.cuh). Claiming in order
//   guarantees that every awaited row belongs to a warp that is already running, so the waits always end; each
//   wait is additionally bounded and reports RSG_ETIMEOUT.
// * FP64 block arithmetic uses explicitly rounded multiplies and adds in the reference's loop order
//   (engine/src/bsr.cpp:13-64), so factors, sweeps and SpMV are bitwise those of the reference's serial code.
// * Tile kernels (SpMV, vector updates) cover TILE_ROWS block rows of one system with 3 threads per block row;
//   inner products are reduced per tile and then, in the last tile to finish, per system in a fixed order
//   (deterministic), and the BiCGSTAB scalar recurrences are evaluated on the device.
#include "rsg_impl.h"
#include "rsg_block3.cuh"
#include "rsg_reduce.cuh"
#include "rsg_sync.cuh"

#include <cuda_runtime.h>
#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>

namespace rsg {

namespace {

constexpr int kSweepThreads = 128;

// ------------------------------------------------------------------ BILU0 factorisation (sync-free, level order)
// engine/src/bsr.cpp:183-215 row by row; rows of a system claimed in forward level order.
__global__ void __launch_bounds__(kSweepThreads) k_factor_f64(int n, const int* __restrict__ rowPtr, const int* __restrict__ col,
                                                             const int* __restrict__ diag, const int* __restrict__ ford,
                                                             const int* __restrict__ elimPtr, const int* __restrict__ elimT,
                                                             const int* __restrict__ elimQ, double* lu, int* flagL, int epoch,
                                                             unsigned* ctr, int* nreg, int* err) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        __syncwarp();
        const int base = warp_claim(ctr);
        if (base >= n) break;
        const int idx = base + lane;
        if (idx < n) {
            const int i = __ldg(ford + idx);
            const int r0 = __ldg(rowPtr + i), d = __ldg(diag + i);
            wait_cols(flagL, col, r0, d, epoch, err);
            for (int p = r0; p < d; ++p) {
                const int k = __ldg(col + p);
                double a[9], u[9], L[9];
                load9(lu + size_t(p) * 9, a);
                load9(lu + size_t(__ldg(diag + k)) * 9, u);
                gemm3(a, u, L);                                   // L_ik = A_ik U_kk^-1
                store9(lu + size_t(p) * 9, L);
                for (int e = __ldg(elimPtr + p); e < __ldg(elimPtr + p + 1); ++e) {
                    const int t = __ldg(elimT + e), q = __ldg(elimQ + e);
                    double U[9], Cb[9];
                    load9(lu + size_t(q) * 9, U);
                    load9(lu + size_t(t) * 9, Cb);
                    gemm3_sub(L, U, Cb);                          // A_ij -= L_ik U_kj
                    store9(lu + size_t(t) * 9, Cb);
                }
            }
            double D[9];
            load9(lu + size_t(d) * 9, D);
            if (invert_pivot3(D)) atomicAdd(nreg, 1);
            store9(lu + size_t(d) * 9, D);
            st_release(flagL + i, epoch);
        }
    }
}

// C45 lean factorisation (engine/src/bsr.cpp:219-263): the row is eliminated in double (work) against the float
// factors of earlier rows, the pivot inverted in double, and the row stored rounded to float.
__global__ void __launch_bounds__(kSweepThreads) k_factor_lean(int n, const int* __restrict__ rowPtr, const int* __restrict__ col,
                                                              const int* __restrict__ diag, const int* __restrict__ ford,
                                                              const int* __restrict__ elimPtr, const int* __restrict__ elimT,
                                                              const int* __restrict__ elimQ, const double* __restrict__ val,
                                                              float* F, double* work, int* flagL, int epoch, unsigned* ctr,
                                                              int* nreg, int* err) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        __syncwarp();
        const int base = warp_claim(ctr);
        if (base >= n) break;
        const int idx = base + lane;
        if (idx < n) {
            const int i = __ldg(ford + idx);
            const int r0 = __ldg(rowPtr + i), r1 = __ldg(rowPtr + i + 1), d = __ldg(diag + i);
            for (int p = r0; p < r1; ++p)
                for (int e = 0; e < 9; ++e) work[size_t(p) * 9 + e] = double(float(__ldg(val + size_t(p) * 9 + e)));
            wait_cols(flagL, col, r0, d, epoch, err);
            for (int p = r0; p < d; ++p) {
                const int k = __ldg(col + p);
                double a[9], u[9], L[9];
                load9(work + size_t(p) * 9, a);
                const float* fk = F + size_t(__ldg(diag + k)) * 9;
                for (int e = 0; e < 9; ++e) u[e] = double(fk[e]);
                gemm3(a, u, L);
                store9(work + size_t(p) * 9, L);
                for (int e = __ldg(elimPtr + p); e < __ldg(elimPtr + p + 1); ++e) {
                    const int t = __ldg(elimT + e), q = __ldg(elimQ + e);
                    double U[9], Cb[9];
                    const float* fq = F + size_t(q) * 9;
                    for (int j = 0; j < 9; ++j) U[j] = double(fq[j]);
                    load9(work + size_t(t) * 9, Cb);
                    gemm3_sub(L, U, Cb);
                    store9(work + size_t(t) * 9, Cb);
                }
            }
            double D[9];
            load9(work + size_t(d) * 9, D);
            if (invert_pivot3(D)) atomicAdd(nreg, 1);
            store9(work + size_t(d) * 9, D);
            for (int p = r0; p < r1; ++p)
                for (int e = 0; e < 9; ++e) F[size_t(p) * 9 + e] = float(work[size_t(p) * 9 + e]);
            st_release(flagL + i, epoch);
        }
    }
}

// ------------------------------------------------------------------ sweeps
// Input modes of the forward sweep (fusions of the BiCGSTAB vector updates, engine/src/linsolve.cpp:172-186):
enum { IN_PLAIN = 0, IN_PUPDATE = 1, IN_SUPDATE = 2 };

__device__ __forceinline__ bool sys_running(const KScal* ks, const int* rowSys, int i) {
    return ks == nullptr || ks[__ldg(rowSys + i)].status == ST_RUNNING;
}

// y_i = in_i - sum_{k<i} L_ik y_k   (engine/src/bsr.cpp:568-575)
// IN_PUPDATE: in = p = r + beta (p - omega v) (p stored); IN_SUPDATE: in = s = r - alpha v (s stored in pv)
// factor blocks in FP64 or FP32 storage, read as double (the float-factor sweeps, engine/src/bsr.cpp:500-522)
__device__ __forceinline__ void ldf9(const double* p, double* a) { load9_ro(p, a); }
__device__ __forceinline__ void ldf9(const float* p, double* a) {
#pragma unroll
    for (int e = 0; e < 9; ++e) a[e] = double(__ldg(p + e));
}

// yi -= sum_p B_p y_col(p) over the entries [p0, p1) of a row, in order (FP64 explicitly rounded, the reference's
// sweep arithmetic). Four blocks at a time: their factor blocks are loaded before the wait (read-only: they need
// not wait for anything), the four dependency flags are polled together, then one acquire fence and the values.
template <class TF>
__device__ __forceinline__ void sub_flagged(double (&yi)[3], const int* __restrict__ col, const TF* __restrict__ lu, int p0, int p1,
                                            const double* y, const int* flag, int* err) {
    for (int q = p0; q < p1; q += 4) {
        const int q1 = q + 4 < p1 ? q + 4 : p1;
        double a[4][9];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (q + u < q1) ldf9(lu + size_t(q + u) * 9, a[u]);
        wait_cols(flag, col, q, q1, 1, err);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (q + u >= q1) break;
            const int k = __ldg(col + q + u);
            const double yk[3] = {y[size_t(k) * 3 + 0], y[size_t(k) * 3 + 1], y[size_t(k) * 3 + 2]};
            yi[0] = ds(yi[0], dot3(a[u], yk));
            yi[1] = ds(yi[1], dot3(a[u] + 3, yk));
            yi[2] = ds(yi[2], dot3(a[u] + 6, yk));
        }
    }
}

template <class TF, int MODE>
__global__ void __launch_bounds__(kSweepThreads) k_fwd_f64(int n, const int* __restrict__ rowPtr, const int* __restrict__ col,
                                                          const int* __restrict__ diag, const int* __restrict__ ford,
                                                          const TF* __restrict__ lu, const double* r, double* pv,
                                                          const double* v, double* y, const int* __restrict__ rowSys,
                                                          const KScal* ks, int* flagF, int* flagB, unsigned* ctr, int* err) {
    if (blockIdx.x == 0 && threadIdx.x == 0) ctr[1] = 0u;   // backward claim counter for the next sweep
    const int lane = threadIdx.x & 31;
    for (;;) {
        __syncwarp();
        const int base = warp_claim(ctr);
        if (base >= n) break;
        const int idx = base + lane;
        if (idx < n) {
            const int i = __ldg(ford + idx);
            const bool run = sys_running(ks, rowSys, i);
            double yi[3];
            if (MODE == IN_PUPDATE) {
                const KScal& K = ks[__ldg(rowSys + i)];
                const double beta = K.beta, omega = K.omega;
#pragma unroll
                for (int e = 0; e < 3; ++e) {
                    const size_t q = size_t(i) * 3 + e;
                    double pe = pv[q];
                    if (run) { pe = da(r[q], dm(beta, ds(pe, dm(omega, v[q])))); pv[q] = pe; }
                    yi[e] = pe;
                }
            } else if (MODE == IN_SUPDATE) {
                const KScal& K = ks[__ldg(rowSys + i)];
                const double alpha = K.alpha;
#pragma unroll
                for (int e = 0; e < 3; ++e) {
                    const size_t q = size_t(i) * 3 + e;
                    const double se = ds(r[q], dm(alpha, v[q]));
                    if (run) pv[q] = se;
                    yi[e] = se;
                }
            } else {
#pragma unroll
                for (int e = 0; e < 3; ++e) yi[e] = r[size_t(i) * 3 + e];
            }
            if (run) {
                sub_flagged(yi, col, lu, __ldg(rowPtr + i), __ldg(diag + i), y, flagF, err);
            }
            y[size_t(i) * 3 + 0] = yi[0]; y[size_t(i) * 3 + 1] = yi[1]; y[size_t(i) * 3 + 2] = yi[2];
            flagB[i] = 0;
            st_release(flagF + i, 1);
        }
    }
}

// z_i = U_ii^-1 (y_i - sum_{j>i} U_ij z_j), in place   (engine/src/bsr.cpp:577-587)
template <class TF>
__global__ void __launch_bounds__(kSweepThreads) k_bwd_f64(int n, const int* __restrict__ rowPtr, const int* __restrict__ col,
                                                          const int* __restrict__ diag, const int* __restrict__ bord,
                                                          const TF* __restrict__ lu, double* y, const int* __restrict__ rowSys,
                                                          const KScal* ks, int* flagF, int* flagB, unsigned* ctr, int* err) {
    if (blockIdx.x == 0 && threadIdx.x == 0) ctr[0] = 0u;
    const int lane = threadIdx.x & 31;
    for (;;) {
        __syncwarp();
        const int base = warp_claim(ctr + 1);
        if (base >= n) break;
        const int idx = base + lane;
        if (idx < n) {
            const int i = __ldg(bord + idx);
            if (sys_running(ks, rowSys, i)) {
                double yi[3] = {y[size_t(i) * 3 + 0], y[size_t(i) * 3 + 1], y[size_t(i) * 3 + 2]};
                const int d = __ldg(diag + i);
                double D[9];
                ldf9(lu + size_t(d) * 9, D);
                sub_flagged(yi, col, lu, d + 1, __ldg(rowPtr + i + 1), y, flagB, err);
                y[size_t(i) * 3 + 0] = dot3(D, yi);
                y[size_t(i) * 3 + 1] = dot3(D + 3, yi);
                y[size_t(i) * 3 + 2] = dot3(D + 6, yi);
            }
            flagF[i] = 0;
            st_release(flagB + i, 1);
        }
    }
}

// FP32 factors, FP32 vectors and accumulation (BILU0f, engine/src/bsr.cpp:1100-1121), the result written to z in
// double. The sweep vector is a tagged word per component: {float value, sweep tag} in 64 bits (tag 1 once the
// forward sweep wrote it, 2 once the backward sweep did). A 64-bit access is single-copy atomic, so a poll that
// sees the tag already holds the value: a dependency costs one round trip, with no flag, no fence and no second
// load. Every row is written by both sweeps (rows of systems that are not running carry their value along), so
// the tags alternate and a word never shows the awaited tag before its new value.
constexpr unsigned kTagF = 1u, kTagB = 2u;
__device__ __forceinline__ unsigned long long ld_word(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_word(unsigned long long* p, float v, unsigned tag) {
    const unsigned long long w = (static_cast<unsigned long long>(tag) << 32) | __float_as_uint(v);
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(w) : "memory");
}
__device__ __forceinline__ float word_val(unsigned long long w) { return __uint_as_float(unsigned(w & 0xffffffffull)); }
__device__ __forceinline__ bool word_has(unsigned long long w, unsigned tag) { return unsigned(w >> 32) == tag; }
// yi -= sum_p B_p y_col(p) over the entries [p0, p1) of a row (in order). The y words of four blocks are awaited
// together: every poll round re-issues the loads of all words still without the tag (one round trip per round),
// a short busy phase, then back-off up to 256 ns, bounded (ERR_TIMEOUT).
__device__ __forceinline__ void sub_tagged(float (&yi)[3], const int* __restrict__ col, const float* __restrict__ lu, int p0, int p1,
                                           const unsigned long long* y, unsigned tag, int* err) {
    for (int q = p0; q < p1; q += 4) {
        int k[4];
        unsigned long long w[4][3];
        float a[4][9];                                            // the factor blocks, loaded before the wait
        unsigned pending = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            k[u] = q + u < p1 ? __ldg(col + q + u) : -1;
            if (k[u] >= 0) pending |= 7u << (3 * u);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int e = 0; e < 9; ++e) a[u][e] = k[u] >= 0 ? __ldg(lu + size_t(q + u) * 9 + e) : 0.f;
        unsigned ns = 0;
        for (unsigned it = 0; pending; ++it) {
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int e = 0; e < 3; ++e)
                    if ((pending >> (3 * u + e)) & 1u) w[u][e] = ld_word(y + size_t(k[u]) * 3 + e);
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int e = 0; e < 3; ++e)
                    if (((pending >> (3 * u + e)) & 1u) && word_has(w[u][e], tag)) pending &= ~(1u << (3 * u + e));
            if (!pending) break;
            if (it >= 64) {
                __nanosleep(ns);
                ns = ns < 32 ? 32 : (ns < 256 ? 2 * ns : 256);
                if (it >= 64 + kSpinLimit) { atomicOr(err, ERR_TIMEOUT); break; }
                if ((it & 255u) == 255u && *(volatile int*)err != 0) break;
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (k[u] < 0) break;
            const float y0 = word_val(w[u][0]), y1 = word_val(w[u][1]), y2 = word_val(w[u][2]);
#pragma unroll
            for (int e = 0; e < 3; ++e) {
                float s = 0.f;
                s += a[u][e * 3 + 0] * y0;
                s += a[u][e * 3 + 1] * y1;
                s += a[u][e * 3 + 2] * y2;
                yi[e] -= s;
            }
        }
    }
}

template <int MODE>
__global__ void __launch_bounds__(kSweepThreads) k_fwd_f32(int n, const int* __restrict__ rowPtr, const int* __restrict__ col,
                                                          const int* __restrict__ diag, const int* __restrict__ ford,
                                                          const float* __restrict__ lu, const double* r, double* pv,
                                                          const double* v, unsigned long long* y, const int* __restrict__ rowSys,
                                                          const KScal* ks, unsigned* ctr, int* err) {
    if (blockIdx.x == 0 && threadIdx.x == 0) ctr[1] = 0u;
    const int lane = threadIdx.x & 31;
    for (;;) {
        __syncwarp();
        const int base = warp_claim(ctr);
        if (base >= n) break;
        const int idx = base + lane;
        if (idx < n) {
            const int i = __ldg(ford + idx);
            const bool run = sys_running(ks, rowSys, i);
            float yi[3];
            if (MODE == IN_PUPDATE) {
                const KScal& K = ks[__ldg(rowSys + i)];
                const double beta = K.beta, omega = K.omega;
#pragma unroll
                for (int e = 0; e < 3; ++e) {
                    const size_t q = size_t(i) * 3 + e;
                    double pe = pv[q];
                    if (run) { pe = da(r[q], dm(beta, ds(pe, dm(omega, v[q])))); pv[q] = pe; }
                    yi[e] = float(pe);
                }
            } else if (MODE == IN_SUPDATE) {
                const KScal& K = ks[__ldg(rowSys + i)];
                const double alpha = K.alpha;
#pragma unroll
                for (int e = 0; e < 3; ++e) {
                    const size_t q = size_t(i) * 3 + e;
                    const double se = ds(r[q], dm(alpha, v[q]));
                    if (run) pv[q] = se;
                    yi[e] = float(se);
                }
            } else {
#pragma unroll
                for (int e = 0; e < 3; ++e) yi[e] = float(r[size_t(i) * 3 + e]);
            }
            if (run) sub_tagged(yi, col, lu, __ldg(rowPtr + i), __ldg(diag + i), y, kTagF, err);
#pragma unroll
            for (int e = 0; e < 3; ++e) st_word(y + size_t(i) * 3 + e, yi[e], kTagF);
        }
    }
}

__global__ void __launch_bounds__(kSweepThreads) k_bwd_f32(int n, const int* __restrict__ rowPtr, const int* __restrict__ col,
                                                          const int* __restrict__ diag, const int* __restrict__ bord,
                                                          const float* __restrict__ lu, unsigned long long* y, double* z,
                                                          const int* __restrict__ rowSys, const KScal* ks, unsigned* ctr, int* err) {
    if (blockIdx.x == 0 && threadIdx.x == 0) ctr[0] = 0u;
    const int lane = threadIdx.x & 31;
    for (;;) {
        __syncwarp();
        const int base = warp_claim(ctr + 1);
        if (base >= n) break;
        const int idx = base + lane;
        if (idx < n) {
            const int i = __ldg(bord + idx);
            float yi[3] = {word_val(ld_word(y + size_t(i) * 3 + 0)), word_val(ld_word(y + size_t(i) * 3 + 1)),
                           word_val(ld_word(y + size_t(i) * 3 + 2))};
            if (sys_running(ks, rowSys, i)) {
                const int d = __ldg(diag + i);
                sub_tagged(yi, col, lu, d + 1, __ldg(rowPtr + i + 1), y, kTagB, err);
                const float* D = lu + size_t(d) * 9;
                float t[3];
#pragma unroll
                for (int e = 0; e < 3; ++e) {
                    float s = 0.f;
                    s += __ldg(D + e * 3 + 0) * yi[0];
                    s += __ldg(D + e * 3 + 1) * yi[1];
                    s += __ldg(D + e * 3 + 2) * yi[2];
                    t[e] = s;
                }
#pragma unroll
                for (int e = 0; e < 3; ++e) {
                    yi[e] = t[e];
                    z[size_t(i) * 3 + e] = double(t[e]);
                }
            }
#pragma unroll
            for (int e = 0; e < 3; ++e) st_word(y + size_t(i) * 3 + e, yi[e], kTagB);
        }
    }
}

// ------------------------------------------------------------------ tile kernels with fused reductions (rsg_reduce.cuh)
// SpMV epilogues / fused dot products
enum { SP_PLAIN = 0, SP_RV = 1, SP_OMEGA = 2, SP_TRUERES = 3 };

// y = A x on one tile (3 threads per block row). SP_RV: partial <rh, y>; then alpha = rho / <rh, v>. SP_OMEGA:
// partials <t,t>, <t,s>, <s,s>; then omega or the early exit on ||s||. SP_TRUERES: y = b - A x, partials <y,y>,
// <b,b>, result sqrt ratio into out[s].
//
// Arithmetic (FMA): false = the reference's order and rounding per block (engine/src/bsr.cpp:109-117: row sum of
// the block from zero, then added; bitwise the reference), true = one fused multiply-add per term.
// On GB300 the FP64 unit runs at 1/64 of the FP32 rate, and the 9 multiply-adds of a block bound this kernel
// rather than HBM: the FMA form keeps the FP64 pipe about 90 % busy at 70 % of the HBM copy rate, the unfused
// form needs twice the FP64 instructions. Hence direct read-only loads (the values stream once, the x gather
// hits L2), 128 block rows per pass so the SM holds enough loads in flight, and a reduction that spends as few
// FP64 adds as possible (rsg_reduce.cuh).
constexpr int kSpmvThreads = 384;

template <bool FMA>
__device__ __forceinline__ double block_row_term(double yv, const double* a, const double* xc) {
    if (FMA) return fma(a[2], __ldg(xc + 2), fma(a[1], __ldg(xc + 1), fma(a[0], __ldg(xc), yv)));
    return da(yv, da(da(dm(a[0], __ldg(xc)), dm(a[1], __ldg(xc + 1))), dm(a[2], __ldg(xc + 2))));
}

template <int MODE>
__device__ __forceinline__ void spmv_out(size_t q, double yv, double* y, const double* __restrict__ a1, double (&acc)[MAX_DOTS]) {
    if (MODE == SP_TRUERES) {
        const double bq = __ldg(a1 + q);
        const double rq = ds(bq, yv);
        if (y) y[q] = rq;
        acc[0] += rq * rq;
        acc[1] += bq * bq;
    } else {
        y[q] = yv;
        if (MODE == SP_RV) acc[0] += __ldg(a1 + q) * yv;
        if (MODE == SP_OMEGA) {
            const double sq = __ldg(a1 + q);
            acc[0] += yv * yv;
            acc[1] += yv * sq;
            acc[2] += sq * sq;
        }
    }
}

template <int MODE, bool FMA>
__global__ void __launch_bounds__(kSpmvThreads) k_spmv_tile(int ntiles, int nsys, const int* __restrict__ tileRow0,
                                                           const int* __restrict__ tileSys, const int* __restrict__ sysTile0,
                                                           const int* __restrict__ rowPtr, const int* __restrict__ col,
                                                           const double* __restrict__ val, const double* __restrict__ x, double* y,
                                                           const double* __restrict__ a1, KScal* ks, double* part, unsigned* done,
                                                           double* sysdot, int* active, double* out) {
    __shared__ double sh[MAX_DOTS * kSpmvThreads];
    const int tile = blockIdx.x;
    const int s = __ldg(tileSys + tile);
    const bool run = (MODE == SP_PLAIN || MODE == SP_TRUERES) || ks[s].status == ST_RUNNING;
    double acc[MAX_DOTS] = {0, 0, 0, 0};
    if (run) {
        const int r0 = __ldg(tileRow0 + tile), r1 = __ldg(tileRow0 + tile + 1);
        const int e = threadIdx.x % 3;
        for (int row = r0 + int(threadIdx.x) / 3; row < r1; row += kSpmvThreads / 3) {
            double yv = 0;
            const int p1 = __ldg(rowPtr + row + 1);
            for (int p = __ldg(rowPtr + row); p < p1; ++p) {
                const double* a = val + size_t(p) * 9 + e * 3;
                const double av[3] = {__ldg(a), __ldg(a + 1), __ldg(a + 2)};
                yv = block_row_term<FMA>(yv, av, x + size_t(__ldg(col + p)) * 3);
            }
            spmv_out<MODE>(size_t(row) * 3 + e, yv, y, a1, acc);
        }
    }
    if (MODE == SP_PLAIN) return;
    constexpr int ND = MODE == SP_RV ? 1 : (MODE == SP_OMEGA ? 3 : 2);
    block_reduce<ND>(acc, sh);
    if (threadIdx.x == 0)
#pragma unroll
        for (int j = 0; j < ND; ++j) part[size_t(tile) * MAX_DOTS + j] = acc[j];
    if (!last_tile_reduce<ND>(ntiles, nsys, sysTile0, part, done, sysdot, sh)) return;
    for (int q = threadIdx.x; q < nsys; q += blockDim.x) {
        const double* dd = sysdot + size_t(q) * MAX_DOTS;
        if (MODE == SP_TRUERES) {
            out[q] = dd[1] > 0 ? sqrt(dd[0]) / sqrt(dd[1]) : 0.0;
            continue;
        }
        KScal& K = ks[q];
        if (K.status != ST_RUNNING) continue;
        if (MODE == SP_RV) {
            const double rv = dd[0];
            if (fabs(rv) < 1e-300 || !isfinite(rv)) {   // engine/src/linsolve.cpp:179
                K.status = ST_BREAKDOWN;
                atomicSub(active, 1);
            } else {
                K.alpha = K.rho / rv;
            }
        } else if (MODE == SP_OMEGA) {
            const double tt = dd[0], ts = dd[1], ss = dd[2];
            K.sn = sqrt(ss);
            K.omega = tt > 0 ? ts / tt : 0.0;             // engine/src/linsolve.cpp:196
        }
    }
}

// BiCGSTAB initial state: x = 0, r = rh = b, p = v = 0; rho = <b,b>, alpha = omega = 1 (engine/src/linsolve.cpp:162-168)
__global__ void __launch_bounds__(kTileThreads) k_bicg_init(int ntiles, int nsys, const int* __restrict__ tileRow0,
                                                           const int* __restrict__ tileSys, const int* __restrict__ sysTile0,
                                                           const double* __restrict__ b, double* x, double* r, double* rh, double* p,
                                                           double* v, KScal* ks, double tol, int maxit, int guard, int onlyFailed,
                                                           double* part, unsigned* done, double* sysdot, int* active) {
    __shared__ double sh[MAX_DOTS * kTileThreads];
    const int tile = blockIdx.x;
    const size_t q0 = size_t(__ldg(tileRow0 + tile)) * 3, q1 = size_t(__ldg(tileRow0 + tile + 1)) * 3;
    double acc[MAX_DOTS] = {0, 0, 0, 0};
    // onlyFailed: the systems that converged keep their solution and status (a restart of the others)
    if (!onlyFailed || ks[__ldg(tileSys + tile)].status != ST_CONV)
        for (size_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
            const double bq = __ldg(b + q);
            x[q] = 0; r[q] = bq; rh[q] = bq; p[q] = 0; v[q] = 0;
            acc[0] += bq * bq;
        }
    block_reduce<1>(acc, sh);
    if (threadIdx.x == 0) part[size_t(tile) * MAX_DOTS] = acc[0];
    if (!last_tile_reduce<1>(ntiles, nsys, sysTile0, part, done, sysdot, sh)) return;
    if (threadIdx.x == 0) *active = 0;
    __syncthreads();
    int nact = 0;
    for (int s = threadIdx.x; s < nsys; s += blockDim.x) {
        KScal& K = ks[s];
        if (onlyFailed && K.status == ST_CONV) continue;
        const double bb = sysdot[size_t(s) * MAX_DOTS];
        K.guard = guard;
        K.hn = 1e300;           // the guard's best residual so far and its iteration
        K.gj = 0;
        K.bn = sqrt(bb);
        K.tol = tol; K.maxit = maxit; K.its = 0; K.relres = 0; K.sn = 0;
        K.alpha = 1; K.omega = 1; K.rho = bb; K.beta = bb;   // rhoN of iteration 1 = <rh, r> = <b, b>
        if (K.bn == 0) { K.status = ST_CONV; }                // engine/src/linsolve.cpp:165
        else if (fabs(bb) < 1e-300 || !isfinite(bb)) { K.status = ST_BREAKDOWN; }
        else if (maxit < 1) { K.status = ST_MAXIT; }
        else { K.status = ST_RUNNING; ++nact; }
    }
    if (nact) atomicAdd(active, nact);
}

// End of a BiCGSTAB iteration (engine/src/linsolve.cpp:183-213):
//   ||s|| small: x += alpha ph and stop; else x += alpha ph + omega sh, r = s - omega t, then ||r||, <rh, r>.
__global__ void __launch_bounds__(kTileThreads) k_bicg_update(int ntiles, int nsys, const int* __restrict__ tileRow0,
                                                             const int* __restrict__ tileSys, const int* __restrict__ sysTile0,
                                                             double* x, double* r, const double* __restrict__ rh,
                                                             const double* __restrict__ s, const double* __restrict__ t,
                                                             const double* __restrict__ ph, const double* __restrict__ sh_,
                                                             KScal* ks, double* part, unsigned* done, double* sysdot, int* active) {
    __shared__ double sh[MAX_DOTS * kTileThreads];
    const int tile = blockIdx.x;
    const int sy = __ldg(tileSys + tile);
    KScal K = ks[sy];
    double acc[MAX_DOTS] = {0, 0, 0, 0};
    if (K.status == ST_RUNNING) {
        const size_t q0 = size_t(__ldg(tileRow0 + tile)) * 3, q1 = size_t(__ldg(tileRow0 + tile + 1)) * 3;
        const bool sconv = K.sn / K.bn < K.tol;
        for (size_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
            if (sconv) {
                x[q] = da(x[q], dm(K.alpha, __ldg(ph + q)));
            } else {
                x[q] = da(x[q], da(dm(K.alpha, __ldg(ph + q)), dm(K.omega, __ldg(sh_ + q))));
                const double rq = ds(__ldg(s + q), dm(K.omega, __ldg(t + q)));
                r[q] = rq;
                acc[0] += rq * rq;
                acc[1] += __ldg(rh + q) * rq;
            }
        }
    }
    block_reduce<2>(acc, sh);
    if (threadIdx.x == 0) { part[size_t(tile) * MAX_DOTS] = acc[0]; part[size_t(tile) * MAX_DOTS + 1] = acc[1]; }
    if (!last_tile_reduce<2>(ntiles, nsys, sysTile0, part, done, sysdot, sh)) return;
    for (int q = threadIdx.x; q < nsys; q += blockDim.x) {
        KScal& k = ks[q];
        if (k.status != ST_RUNNING) continue;
        const int it = k.its + 1;
        k.its = it;
        if (k.sn / k.bn < k.tol) {                              // engine/src/linsolve.cpp:187-191
            k.relres = k.sn / k.bn;
            k.status = ST_CONV;
            atomicSub(active, 1);
            continue;
        }
        const double rn = sqrt(sysdot[size_t(q) * MAX_DOTS]);
        const double rhoN = sysdot[size_t(q) * MAX_DOTS + 1];
        k.relres = rn / k.bn;
        if (rn / k.bn < k.tol) { k.status = ST_CONV; atomicSub(active, 1); continue; }
        if (k.omega == 0 || !isfinite(rn)) { k.status = ST_BREAKDOWN; atomicSub(active, 1); continue; }
        if (fabs(rhoN) < 1e-300) { k.status = ST_BREAKDOWN; atomicSub(active, 1); continue; }   // next iteration's test
        if (it >= k.maxit) { k.status = ST_MAXIT; atomicSub(active, 1); continue; }
        if (k.guard) {          // FP32 preconditioner: diverging, or no new best residual for 40 iterations (stalled)
            if (k.relres < k.hn) { k.hn = k.relres; k.gj = it; }
            if ((it >= 8 && k.relres > 1e4) || it - k.gj >= 40) { k.status = ST_DIVERGED; atomicSub(active, 1); continue; }
        }
        k.beta = (rhoN / k.rho) * (k.alpha / k.omega);
        k.rho = rhoN;
    }
}

// ------------------------------------------------------------------ block Jacobi
__global__ void k_bj_setup(int n, const int* __restrict__ diag, const double* __restrict__ val, double* dinv, int* nreg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double D[9];
    load9_ro(val + size_t(__ldg(diag + i)) * 9, D);
    double B[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) B[e] = D[e];
    if (!invert3(B)) {   // DeviceCprAmg fallback: 1 / max(1e-30, |D_ee|) (engine/src/bsr.cpp:1305)
#pragma unroll
        for (int e = 0; e < 9; ++e) B[e] = 0;
        for (int e = 0; e < 3; ++e) B[e * 4] = 1.0 / fmax(1e-30, fabs(D[e * 4]));
        atomicAdd(nreg, 1);
    }
    store9(dinv + size_t(i) * 9, B);
}

template <int MODE>
__global__ void k_bj_apply(int n, const double* __restrict__ dinv, const double* r, double* pv, const double* v, double* z,
                           const int* __restrict__ rowSys, const KScal* ks) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool run = sys_running(ks, rowSys, i);
    if (!run) return;
    double yi[3];
    if (MODE == IN_PUPDATE) {
        const KScal& K = ks[__ldg(rowSys + i)];
        for (int e = 0; e < 3; ++e) {
            const size_t q = size_t(i) * 3 + e;
            const double pe = da(r[q], dm(K.beta, ds(pv[q], dm(K.omega, v[q]))));
            pv[q] = pe; yi[e] = pe;
        }
    } else if (MODE == IN_SUPDATE) {
        const KScal& K = ks[__ldg(rowSys + i)];
        for (int e = 0; e < 3; ++e) {
            const size_t q = size_t(i) * 3 + e;
            const double se = ds(r[q], dm(K.alpha, v[q]));
            pv[q] = se; yi[e] = se;
        }
    } else {
        for (int e = 0; e < 3; ++e) yi[e] = r[size_t(i) * 3 + e];
    }
    double D[9];
    load9_ro(dinv + size_t(i) * 9, D);
    z[size_t(i) * 3 + 0] = dot3(D, yi);
    z[size_t(i) * 3 + 1] = dot3(D + 3, yi);
    z[size_t(i) * 3 + 2] = dot3(D + 6, yi);
}

__global__ void k_gather_blocks(int nnzb, const int* __restrict__ src, const double* __restrict__ a, double* b) {
    const size_t total = size_t(nnzb) * 9;
    for (size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x; q < total; q += size_t(gridDim.x) * blockDim.x)
        b[q] = __ldg(a + size_t(__ldg(src + q / 9)) * 9 + q % 9);
}
__global__ void k_gather_vec(int n, const int* __restrict__ perm, const double* __restrict__ orig, double* lev) {
    const size_t total = size_t(n) * 3;
    for (size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x; q < total; q += size_t(gridDim.x) * blockDim.x)
        lev[q] = __ldg(orig + size_t(__ldg(perm + q / 3)) * 3 + q % 3);
}
__global__ void k_scatter_vec(int n, const int* __restrict__ perm, const double* __restrict__ lev, double* orig) {
    const size_t total = size_t(n) * 3;
    for (size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x; q < total; q += size_t(gridDim.x) * blockDim.x)
        orig[size_t(__ldg(perm + q / 3)) * 3 + q % 3] = __ldg(lev + q);
}

int g_sm_count = 0;
int stream_grid(size_t total) {
    const size_t g = (total + 255) / 256, cap = size_t(device_sm_count()) * 16;
    return int(g < cap ? (g > 0 ? g : 1) : cap);
}
int sweep_grid(int n) {
    const int sms = device_sm_count();
    // enough warps for several levels in flight, at most 8 blocks of 4 warps per SM
    const int warps = (n + 31) / 32;
    int blocks = (warps + 3) / 4;
    const int maxb = sms * 8;
    if (blocks > maxb) blocks = maxb;
    if (blocks < 1) blocks = 1;
    return blocks;
}

// the plan's grid when it was sized from the level widths, else one from n
int sweep_blocks(const DevPlan& P) { return P.sweepBlocks > 0 ? P.sweepBlocks : sweep_grid(P.n); }

}  // namespace

// Warps that poll flags of levels far ahead of the sweep front only add memory traffic to the critical path:
// keep about `inflight` levels' rows in flight (a warp per 32 rows), at most 8 blocks of 4 warps per SM.
int sweep_blocks_for(double avgRows, int inflight) {
    if (inflight <= 0) return 8 * device_sm_count();              // auto: the full grid (measured no slower)
    const double warps = double(inflight) * avgRows / 32.0;
    const long long blocks = (long long)((warps + 3.0) / 4.0);
    const long long cap = 8LL * device_sm_count();
    return int(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
}

int device_sm_count() {
    if (g_sm_count == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
        if (g_sm_count <= 0) g_sm_count = 1;
    }
    return g_sm_count;
}

void launch_gather_blocks(const DevPlan& P, const double* src, double* dst, cudaStream_t st) {
    k_gather_blocks<<<stream_grid(size_t(P.nnzb) * 9), 256, 0, st>>>(P.nnzb, P.valSrc, src, dst);
}
void launch_gather_vec(const DevPlan& P, const double* orig, double* lev, cudaStream_t st) {
    k_gather_vec<<<stream_grid(size_t(P.n) * 3), 256, 0, st>>>(P.n, P.perm, orig, lev);
}
void launch_scatter_vec(const DevPlan& P, const double* lev, double* orig, cudaStream_t st) {
    k_scatter_vec<<<stream_grid(size_t(P.n) * 3), 256, 0, st>>>(P.n, P.perm, lev, orig);
}

void launch_factor_f64(const DevPlan& P, const double* val, double* lu, SweepState& S, int epoch, int* nreg, int* err,
                       cudaStream_t st) {
    cudaMemcpyAsync(lu, val, size_t(P.nnzb) * 9 * sizeof(double), cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(S.ctr + 2, 0, sizeof(unsigned), st);
    k_factor_f64<<<sweep_blocks(P), kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.ford, P.elimPtr, P.elimT, P.elimQ, lu,
                                                           S.flagL, epoch, S.ctr + 2, nreg, err);
}

void launch_factor_lean(const DevPlan& P, const double* val, float* luf, double* work, SweepState& S, int epoch, int* nreg,
                        int* err, cudaStream_t st) {
    cudaMemsetAsync(S.ctr + 2, 0, sizeof(unsigned), st);
    k_factor_lean<<<sweep_blocks(P), kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.ford, P.elimPtr, P.elimT, P.elimQ,
                                                            val, luf, work, S.flagL, epoch, S.ctr + 2, nreg, err);
}

void launch_ilu_apply_f64(const DevPlan& P, const double* lu, const double* r, double* z, SweepState& S, int* err,
                          cudaStream_t st) {
    const int g = sweep_blocks(P);
    k_fwd_f64<double, IN_PLAIN><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.ford, lu, r, nullptr, nullptr, z, P.rowSys,
                                                     nullptr, S.flagF, S.flagB, S.ctr, err);
    k_bwd_f64<double><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.bord, lu, z, P.rowSys, nullptr, S.flagF, S.flagB, S.ctr,
                                          err);
}

void launch_ilu_apply_mixed(const DevPlan& P, const float* luf, const double* r, double* z, SweepState& S, int* err,
                            cudaStream_t st) {
    const int g = sweep_blocks(P);
    k_fwd_f64<float, IN_PLAIN><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.ford, luf, r, nullptr, nullptr, z, P.rowSys,
                                                           nullptr, S.flagF, S.flagB, S.ctr, err);
    k_bwd_f64<float><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.bord, luf, z, P.rowSys, nullptr, S.flagF, S.flagB, S.ctr,
                                                 err);
}

void launch_ilu_apply_f32(const DevPlan& P, const float* luf, const double* r, double* z, unsigned long long* y32, SweepState& S, int* err,
                          cudaStream_t st) {
    const int g = sweep_blocks(P);
    k_fwd_f32<IN_PLAIN><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.ford, luf, r, nullptr, nullptr, y32, P.rowSys,
                                                     nullptr, S.ctr, err);
    k_bwd_f32<<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.bord, luf, y32, z, P.rowSys, nullptr, S.ctr, err);
}

void launch_ilu_grid_ks(const DevPlan& P, const PrecDev& M, const double* r, double* z, const KScal* ks, SweepState& S, int* err,
                        cudaStream_t st) {
    const int g = sweep_blocks(P);
    if (M.kind == 0) {
        k_fwd_f64<double, IN_PLAIN><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.ford, M.lu, r, nullptr, nullptr, z,
                                                                 P.rowSys, ks, S.flagF, S.flagB, S.ctr, err);
        k_bwd_f64<double><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.bord, M.lu, z, P.rowSys, ks, S.flagF, S.flagB,
                                                       S.ctr, err);
    } else if (M.kind == 1) {
        k_fwd_f64<float, IN_PLAIN><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.ford, M.luf, r, nullptr, nullptr, z,
                                                                P.rowSys, ks, S.flagF, S.flagB, S.ctr, err);
        k_bwd_f64<float><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.bord, M.luf, z, P.rowSys, ks, S.flagF, S.flagB,
                                                      S.ctr, err);
    } else {
        k_fwd_f32<IN_PLAIN><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.ford, M.luf, r, nullptr, nullptr, M.yt,
                                                         P.rowSys, ks, S.ctr, err);
        k_bwd_f32<<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.bord, M.luf, M.yt, z, P.rowSys, ks, S.ctr, err);
    }
}

template <int MODE, bool FMA>
void spmv_go(const DevPlan& P, const double* val, const double* x, double* y, const double* a1, KScal* ks, ReduceState* R, int* active,
             double* out, cudaStream_t st) {
    k_spmv_tile<MODE, FMA><<<P.ntiles, kSpmvThreads, 0, st>>>(P.ntiles, P.nsys, P.tileRow0, P.tileSys, P.sysTile0, P.rowPtr, P.col, val,
                                                               x, y, a1, ks, R ? R->part : nullptr, R ? R->done : nullptr,
                                                               R ? R->sysdot : nullptr, active, out);
}
// SpMV tile kernel with the handle's arithmetic (P.spmvFma)
template <int MODE>
void spmv(const DevPlan& P, const double* val, const double* x, double* y, const double* a1, KScal* ks, ReduceState* R, int* active,
          double* out, cudaStream_t st) {
    if (P.spmvFma) spmv_go<MODE, true>(P, val, x, y, a1, ks, R, active, out, st);
    else spmv_go<MODE, false>(P, val, x, y, a1, ks, R, active, out, st);
}

// The dynamic shared-memory opt-in of a kernel is one process-wide value per device: handles on several threads
// (serving slots) with plans of different sizes only ever raise it, under one lock.
void raise_smem_limit(const void* fn, int bytes) {
    if (bytes <= 48 * 1024) return;
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, int> lim;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    int& cur = lim[{dev, fn}];
    if (bytes > cur) {
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        cur = bytes;
    }
}

__global__ void k_vec_add(size_t m, double* x, const double* __restrict__ d) {
    for (size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x; q < m; q += size_t(gridDim.x) * blockDim.x) x[q] += d[q];
}
void launch_vec_add(int n, double* x, const double* d, cudaStream_t st) {
    const size_t m = size_t(n) * 3;
    const int g = int(std::min<size_t>((m + 255) / 256, size_t(device_sm_count()) * 8));
    k_vec_add<<<std::max(g, 1), 256, 0, st>>>(m, x, d);
}

void launch_spmv_f64(const DevPlan& P, const double* val, const double* x, double* y, cudaStream_t st) {
    spmv<SP_PLAIN>(P, val, x, y, nullptr, nullptr, nullptr, nullptr, nullptr, st);
}

void launch_block_jacobi_setup(const DevPlan& P, const double* val, double* dinv, int* nreg, cudaStream_t st) {
    k_bj_setup<<<(P.n + 127) / 128, 128, 0, st>>>(P.n, P.diag, val, dinv, nreg);
}
void launch_block_jacobi_apply(const DevPlan& P, const double* dinv, const double* r, double* z, cudaStream_t st) {
    k_bj_apply<IN_PLAIN><<<(P.n + 127) / 128, 128, 0, st>>>(P.n, dinv, r, nullptr, nullptr, z, P.rowSys, nullptr);
}

void launch_bicg_init(const DevPlan& P, const double* b, BicgVecs& V, KScal* ks, ReduceState& R, double tol, int maxit,
                      int* active, bool guard, bool onlyFailed, cudaStream_t st) {
    k_bicg_init<<<P.ntiles, kTileThreads, 0, st>>>(P.ntiles, P.nsys, P.tileRow0, P.tileSys, P.sysTile0, b, V.x, V.r, V.rh, V.p, V.v,
                                                   ks, tol, maxit, guard ? 1 : 0, onlyFailed ? 1 : 0, R.part, R.done, R.sysdot, active);
}

// one iteration: (a) p-update fused into M p, (c) v = A ph + <rh,v>, (d) s-update fused into M s,
// (f) t = A sh + <t,t>, <t,s>, <s,s>, (g) x / r update + ||r||, <rh,r>
void launch_bicg_iteration(const DevPlan& P, const double* val, const PrecDev& M, BicgVecs& V, KScal* ks, ReduceState& R,
                           SweepState& S, int* active, int* err, cudaStream_t st) {
    const int g = sweep_blocks(P);
    auto prec = [&](bool pupd, double* out) {
        if (M.devcpr) {
            launch_devcpr(P, *M.amg, val, pupd ? 1 : 2, V.r, pupd ? V.p : V.s, V.v, out, ks, st);
        } else if (M.cpr && M.cta && !M.split) {
            launch_cpr_cta(P, M, *M.amg, pupd ? 1 : 2, M.kind != 0, V.r, pupd ? V.p : V.s, V.v, out, ks, st);
        } else if (M.cpr) {
            launch_cpr_grid(P, M, *M.amg, pupd ? 1 : 2, V.r, pupd ? V.p : V.s, V.v, out, ks, S, err, st);
        } else if (M.cta && M.kind != 2) {
            launch_ilu_cta_fused(P, M, pupd, V.r, pupd ? V.p : V.s, V.v, out, ks, st);
        } else if (M.kind == 0) {
            if (pupd)
                k_fwd_f64<double, IN_PUPDATE><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.ford, M.lu, V.r, V.p, V.v, out,
                                                                           P.rowSys, ks, S.flagF, S.flagB, S.ctr, err);
            else
                k_fwd_f64<double, IN_SUPDATE><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.ford, M.lu, V.r, V.s, V.v, out,
                                                                           P.rowSys, ks, S.flagF, S.flagB, S.ctr, err);
            k_bwd_f64<double><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.bord, M.lu, out, P.rowSys, ks, S.flagF,
                                                          S.flagB, S.ctr, err);
        } else if (M.kind == 1) {      // FP32 factors, FP64 sweep vector
            if (pupd)
                k_fwd_f64<float, IN_PUPDATE><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.ford, M.luf, V.r, V.p, V.v, out,
                                                                          P.rowSys, ks, S.flagF, S.flagB, S.ctr, err);
            else
                k_fwd_f64<float, IN_SUPDATE><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.ford, M.luf, V.r, V.s, V.v, out,
                                                                          P.rowSys, ks, S.flagF, S.flagB, S.ctr, err);
            k_bwd_f64<float><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.bord, M.luf, out, P.rowSys, ks, S.flagF,
                                                         S.flagB, S.ctr, err);
        } else if (M.kind == 3) {      // all-FP32 sweep
            if (pupd)
                k_fwd_f32<IN_PUPDATE><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.ford, M.luf, V.r, V.p, V.v, V.yt,
                                                                   P.rowSys, ks, S.ctr, err);
            else
                k_fwd_f32<IN_SUPDATE><<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.ford, M.luf, V.r, V.s, V.v, V.yt,
                                                                   P.rowSys, ks, S.ctr, err);
            k_bwd_f32<<<g, kSweepThreads, 0, st>>>(P.n, P.rowPtr, P.col, P.diag, P.bord, M.luf, V.yt, out, P.rowSys, ks, S.ctr, err);
        } else {
            const int gb = (P.n + 127) / 128;
            if (pupd)
                k_bj_apply<IN_PUPDATE><<<gb, 128, 0, st>>>(P.n, M.dinv, V.r, V.p, V.v, out, P.rowSys, ks);
            else
                k_bj_apply<IN_SUPDATE><<<gb, 128, 0, st>>>(P.n, M.dinv, V.r, V.s, V.v, out, P.rowSys, ks);
        }
    };
    prec(true, V.ph);
    spmv<SP_RV>(P, val, V.ph, V.v, V.rh, ks, &R, active, nullptr, st);
    prec(false, V.sh);
    spmv<SP_OMEGA>(P, val, V.sh, V.t, V.s, ks, &R, active, nullptr, st);
    k_bicg_update<<<P.ntiles, kTileThreads, 0, st>>>(P.ntiles, P.nsys, P.tileRow0, P.tileSys, P.sysTile0, V.x, V.r, V.rh, V.s, V.t,
                                                     V.ph, V.sh, ks, R.part, R.done, R.sysdot, active);
}

void launch_true_residual(const DevPlan& P, const double* val, const double* b, const double* x, double* tmp, ReduceState& R,
                          double* out, cudaStream_t st) {
    spmv<SP_TRUERES>(P, val, x, tmp, b, nullptr, &R, nullptr, out, st);
}

}  // namespace rsg
