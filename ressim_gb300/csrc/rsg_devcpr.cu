// The reference's GPU-shaped float CPR-AMG (DeviceCprAmg::build / apply, engine/src/bsr.cpp:1217-1371) as a
// preconditioner of the FP64 Krylov methods (RSG_PREC_CPR_DEVICE).
//
// The BlockCPR hierarchy (the device AMG of the CPR set-up, values rounded to float) smoothed by damped Jacobi
// (omega = 0.6667, one sweep before and one after, the first from x = 0), the coarsest level solved by an explicit
// inverse (Gauss-Jordan in double, rounded to float) or, without one, by 31 Jacobi sweeps, and a block-Jacobi
// second stage: z = z1 + D^-1 (r - S z1) with z1 = E x, the pressure correction in the first unknown of each block.
// Every step is row-parallel (no dependency chain: the reference designed it for a GPU), every float operation is
// rounded on its own in the reference's order, so the result equals the reference's bit for bit.
#include "rsg_impl.h"
#include "rsg_block3.cuh"

#include <cuda_runtime.h>

namespace rsg {

namespace {

constexpr float kOmega = 0.6667f;
enum { DC_PLAIN = 0, DC_PUPDATE = 1, DC_SUPDATE = 2 };

__device__ __forceinline__ float fmr(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float far(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsr(float a, float b) { return __fsub_rn(a, b); }

int grid_of(long long n, int threads) {
    const long long b = (n + threads - 1) / threads, cap = 16LL * device_sm_count();
    return int(b < 1 ? 1 : (b < cap ? b : cap));
}

__device__ __forceinline__ bool sys_ok(const KScal* ks, int s) { return ks == nullptr || ks[s].status == ST_RUNNING; }

// ------------------------------------------------------------------ set-up
// The coarsest level of every system, inverted by Gauss-Jordan in double on the natural-order dense matrix (the
// reference's loop: pivot = first strictly largest |a_ik|, row k scaled by 1 / pivot, every other row updated),
// rounded to float row by row: inv[i * m + j] (natural order). ok[s] = 0 when a pivot vanishes (Jacobi instead).
// One thread block per system; W is an m x 2m double work matrix per system.
__global__ void __launch_bounds__(256) k_dc_coarse_inverse(int maxL, const AmgSysLv* __restrict__ lv, const int* __restrict__ rp,
                                                           const int* __restrict__ ci, const double* __restrict__ val,
                                                           const int* __restrict__ luPerm, double* work, const size_t* workOff,
                                                           float* invAll, int* ok) {
    const int s = blockIdx.x;
    AmgSysLv L;
    bool found = false;
    for (int l = 0; l < maxL; ++l) {
        const AmgSysLv c = lv[s * maxL + l];
        if (c.n > 0 && c.coarse) { L = c; found = true; break; }
    }
    if (!found || !L.dense) {
        if (threadIdx.x == 0) ok[s] = 0;
        return;
    }
    const int m = L.n;
    const size_t w2 = 2 * size_t(m);
    double* M = work + workOff[s];
    const int* nat = luPerm + L.luRowOff;
    for (size_t q = threadIdx.x; q < size_t(m) * w2; q += blockDim.x) M[q] = 0.0;
    __syncthreads();
    if (threadIdx.x == 0)                                          // duplicates add up in entry order
        for (int k = 0; k < m; ++k) {
            const int I = __ldg(nat + k);
            for (int p = __ldg(rp + L.rpOff + k); p < __ldg(rp + L.rpOff + k + 1); ++p)
                M[size_t(I) * w2 + size_t(__ldg(nat + __ldg(ci + L.entOff + p)))] += val[L.entOff + p];
        }
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x) M[size_t(i) * w2 + size_t(m + i)] = 1.0;
    __shared__ double smax[256];
    __shared__ int sidx[256];
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int k = 0; k < m; ++k) {
        double best = -1.0;
        int bi = m;
        for (int i = k + int(threadIdx.x); i < m; i += blockDim.x) {
            const double a = fabs(M[size_t(i) * w2 + k]);
            if (a > best || (a == best && i < bi)) { best = a; bi = i; }
        }
        smax[threadIdx.x] = best;
        sidx[threadIdx.x] = bi;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if (int(threadIdx.x) < o) {
                const double b2 = smax[threadIdx.x + o];
                const int i2 = sidx[threadIdx.x + o];
                if (b2 > smax[threadIdx.x] || (b2 == smax[threadIdx.x] && i2 < sidx[threadIdx.x])) { smax[threadIdx.x] = b2; sidx[threadIdx.x] = i2; }
            }
            __syncthreads();
        }
        // the reference's scan starts at k and moves only on a strictly larger value: the first maximum
        const int pr = smax[0] > fabs(M[size_t(k) * w2 + k]) ? sidx[0] : k;
        if (fabs(M[size_t(pr) * w2 + k]) < 1e-300) {
            if (threadIdx.x == 0) bad = 1;
            __syncthreads();
            break;
        }
        __syncthreads();
        if (pr != k)
            for (size_t j = threadIdx.x; j < w2; j += blockDim.x) {
                const double t = M[size_t(k) * w2 + j];
                M[size_t(k) * w2 + j] = M[size_t(pr) * w2 + j];
                M[size_t(pr) * w2 + j] = t;
            }
        __syncthreads();
        const double piv = __ddiv_rn(1.0, M[size_t(k) * w2 + k]);
        __syncthreads();
        for (size_t j = threadIdx.x; j < w2; j += blockDim.x) M[size_t(k) * w2 + j] = dm(M[size_t(k) * w2 + j], piv);
        __syncthreads();
        for (size_t q = threadIdx.x; q < size_t(m) * w2; q += blockDim.x) {
            const int i = int(q / w2);
            if (i == k) continue;
            const double f = M[size_t(i) * w2 + k];
            if (f == 0) continue;
            const size_t j = q % w2;
            if (j == size_t(k)) continue;                            // column k last: the others read it
            M[q] = ds(M[q], dm(f, M[size_t(k) * w2 + j]));
        }
        __syncthreads();
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            if (i == k) continue;
            const double f = M[size_t(i) * w2 + k];
            if (f != 0) M[size_t(i) * w2 + k] = ds(f, dm(f, M[size_t(k) * w2 + k]));
        }
        __syncthreads();
    }
    float* inv = invAll + L.luOff;
    for (size_t q = threadIdx.x; q < size_t(m) * m; q += blockDim.x) {
        const size_t i = q / size_t(m), j = q % size_t(m);
        inv[q] = float(M[i * w2 + size_t(m) + j]);
    }
    if (threadIdx.x == 0) ok[s] = bad ? 0 : 1;
}

// float inverse diagonal of every AMG row (1 / d in double, rounded; 0 when |d| <= 1e-300)
__global__ void k_dc_dinv(int rows, const int* __restrict__ diagGlob, const double* __restrict__ val, float* dinv) {
    for (int i = int(blockIdx.x * blockDim.x + threadIdx.x); i < rows; i += int(gridDim.x * blockDim.x)) {
        const double d = val[__ldg(diagGlob + i)];
        dinv[i] = fabs(d) > 1e-300 ? float(__ddiv_rn(1.0, d)) : 0.0f;
    }
}

// block-Jacobi second stage: the inverse of every diagonal block (invertBlock, engine/src/bsr.cpp:67-87), else
// 1 / max(1e-30, |D_ee|) on the diagonal, rounded to float
__global__ void k_dc_bj(int n, const int* __restrict__ diag, const double* __restrict__ val, float* bj) {
    for (int i = int(blockIdx.x * blockDim.x + threadIdx.x); i < n; i += int(gridDim.x * blockDim.x)) {
        double D[9], B[9];
        load9_ro(val + size_t(__ldg(diag + i)) * 9, D);
#pragma unroll
        for (int e = 0; e < 9; ++e) B[e] = D[e];
        if (!invert3(B)) {
#pragma unroll
            for (int e = 0; e < 9; ++e) B[e] = 0;
            for (int e = 0; e < 3; ++e) B[e * 4] = __ddiv_rn(1.0, fmax(1e-30, fabs(D[e * 4])));
        }
#pragma unroll
        for (int e = 0; e < 9; ++e) bj[size_t(i) * 9 + e] = float(B[e]);
    }
}

// ------------------------------------------------------------------ application
// input (the fused Krylov update of the mode) rounded to float, kept in T; b0 = W r (float, from zero)
template <int MODE>
__global__ void __launch_bounds__(256) k_dc_in(int n, const int* __restrict__ rowSys, const double* r, double* pv, const double* v,
                                               const double* __restrict__ w, double* T, float* b0, const KScal* ks) {
    for (int k = int(blockIdx.x * blockDim.x + threadIdx.x); k < n; k += int(gridDim.x * blockDim.x)) {
        double beta = 0, omega = 0, alpha = 0;
        if (ks) {
            const KScal& K = ks[__ldg(rowSys + k)];
            if (K.status != ST_RUNNING) continue;
            beta = K.beta; omega = K.omega; alpha = K.alpha;
        }
        float acc = 0.f;
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            const size_t q = size_t(k) * 3 + e;
            double in;
            if (MODE == DC_PUPDATE) { in = da(r[q], dm(beta, ds(pv[q], dm(omega, v[q])))); pv[q] = in; }
            else if (MODE == DC_SUPDATE) { in = ds(r[q], dm(alpha, v[q])); pv[q] = in; }
            else in = r[q];
            const float rf = float(in);
            T[q] = double(rf);
            acc = far(acc, fmr(float(__ldg(w + q)), rf));
        }
        b0[k] = acc;
    }
}

// rows [q0, q1) of level l (systems whose level l is not the coarsest): x = (omega dinv) b, the first sweep from 0
__global__ void k_dc_smooth0(int q0, int q1, int maxL, const int* __restrict__ rowLv, const AmgSysLv* __restrict__ lv,
                             const float* __restrict__ dinv, const float* b, float* x, const KScal* ks) {
    for (int g = q0 + int(blockIdx.x * blockDim.x + threadIdx.x); g < q1; g += int(gridDim.x * blockDim.x)) {
        const int sl = __ldg(rowLv + g);
        if (__ldg(&lv[sl].coarse) || !sys_ok(ks, sl / maxL)) continue;
        x[g] = fmr(fmr(kOmega, __ldg(dinv + g)), b[g]);
    }
}

// b_{l+1} = R (b_l - A_l x_l) for the coarse rows [c0, c1): per member the row sum from zero in entry order, its
// residual, and the restriction sum (unit weights) from zero in restriction order
__global__ void k_dc_restrict(int c0, int c1, int maxL, const int* __restrict__ rowLv, const AmgSysLv* __restrict__ lv,
                              const int* __restrict__ rp, const int* __restrict__ gci, const float* __restrict__ valf,
                              const int* __restrict__ memPtr, const int* __restrict__ mem, float* b, const float* x, const KScal* ks) {
    for (int c = c0 + int(blockIdx.x * blockDim.x + threadIdx.x); c < c1; c += int(gridDim.x * blockDim.x)) {
        const int sl = __ldg(rowLv + c);
        if (!sys_ok(ks, sl / maxL)) continue;
        const AmgSysLv* Cl = lv + sl;
        const AmgSysLv* F = lv + sl - 1;
        const int I = c - __ldg(&Cl->rowOff);
        const int* mp = memPtr + __ldg(&Cl->rpOff);
        const int* mm = mem + __ldg(&Cl->memOff);
        const int fOff = __ldg(&F->rowOff), fEnt = __ldg(&F->entOff);
        const int* frp = rp + __ldg(&F->rpOff);
        float t = 0.f;
        for (int q = __ldg(mp + I); q < __ldg(mp + I + 1); ++q) {
            const int m = __ldg(mm + q);
            float acc = 0.f;
            for (int p = fEnt + __ldg(frp + m); p < fEnt + __ldg(frp + m + 1); ++p) acc = far(acc, fmr(__ldg(valf + p), x[__ldg(gci + p)]));
            t = far(t, fsr(b[fOff + m], acc));
        }
        b[c] = t;
    }
}

// coarsest level, one thread block per system: x = inv b (natural order, float from zero) with the explicit
// inverse, else 31 Jacobi sweeps from x = 0
__global__ void __launch_bounds__(256) k_dc_coarse(int maxL, const AmgSysLv* __restrict__ lv, const int* __restrict__ rp,
                                                   const int* __restrict__ gci, const float* __restrict__ valf,
                                                   const float* __restrict__ dinv, const int* __restrict__ luPerm,
                                                   const float* __restrict__ invAll, const int* __restrict__ ok, const float* b, float* x,
                                                   float* t, const KScal* ks) {
    const int s = blockIdx.x;
    if (!sys_ok(ks, s)) return;
    int nlev = 0;
    while (nlev < maxL && lv[s * maxL + nlev].n > 0) ++nlev;
    if (nlev == 0) return;
    const AmgSysLv L = lv[s * maxL + nlev - 1];
    const int m = L.n, r0 = L.rowOff;
    if (L.dense && ok[s]) {
        extern __shared__ float sm[];                              // b in natural order, natural -> level row
        float* bn = sm;
        int* lev = reinterpret_cast<int*>(sm + m);
        const int* nat = luPerm + L.luRowOff;
        for (int k = threadIdx.x; k < m; k += blockDim.x) {
            const int I = __ldg(nat + k);
            bn[I] = b[r0 + k];
            lev[I] = k;
        }
        __syncthreads();
        const float* inv = invAll + L.luOff;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            float acc = 0.f;
            for (int j = 0; j < m; ++j) acc = far(acc, fmr(__ldg(inv + size_t(i) * m + j), bn[j]));
            x[r0 + lev[i]] = acc;
        }
        return;
    }
    for (int k = threadIdx.x; k < m; k += blockDim.x) x[r0 + k] = fmr(fmr(kOmega, __ldg(dinv + r0 + k)), b[r0 + k]);
    __syncthreads();
    for (int sweep = 0; sweep < 30; ++sweep) {
        for (int k = threadIdx.x; k < m; k += blockDim.x) {
            float acc = 0.f;
            for (int p = L.entOff + __ldg(rp + L.rpOff + k); p < L.entOff + __ldg(rp + L.rpOff + k + 1); ++p)
                acc = far(acc, fmr(__ldg(valf + p), x[__ldg(gci + p)]));
            t[r0 + k] = acc;
        }
        __syncthreads();
        for (int k = threadIdx.x; k < m; k += blockDim.x)
            x[r0 + k] = far(x[r0 + k], fmr(fmr(kOmega, __ldg(dinv + r0 + k)), fsr(b[r0 + k], t[r0 + k])));
        __syncthreads();
    }
}

// rows of level l: x += P x_{l+1} (unit weights: the row sum from zero is the aggregate's value)
__global__ void k_dc_prolong(int q0, int q1, int maxL, const int* __restrict__ rowLv, const AmgSysLv* __restrict__ lv,
                             const int* __restrict__ agg, float* x, const KScal* ks) {
    for (int g = q0 + int(blockIdx.x * blockDim.x + threadIdx.x); g < q1; g += int(gridDim.x * blockDim.x)) {
        const int sl = __ldg(rowLv + g);
        if (__ldg(&lv[sl].coarse) || !sys_ok(ks, sl / maxL)) continue;
        const float t = far(0.f, fmr(1.0f, x[__ldg(&lv[sl + 1].rowOff) + __ldg(agg + g)]));
        x[g] = far(x[g], t);
    }
}

// rows of level l: t = A x (float, from zero in entry order)
__global__ void k_dc_spmv(int q0, int q1, int maxL, const int* __restrict__ rowLv, const AmgSysLv* __restrict__ lv, const int* __restrict__ rp,
                          const int* __restrict__ gci, const float* __restrict__ valf, const float* x, float* t, const KScal* ks) {
    for (int g = q0 + int(blockIdx.x * blockDim.x + threadIdx.x); g < q1; g += int(gridDim.x * blockDim.x)) {
        const int sl = __ldg(rowLv + g);
        const AmgSysLv* A = lv + sl;
        if (__ldg(&A->coarse) || !sys_ok(ks, sl / maxL)) continue;
        const int k = g - __ldg(&A->rowOff), e0 = __ldg(&A->entOff);
        const int* r = rp + __ldg(&A->rpOff);
        float acc = 0.f;
        for (int p = e0 + __ldg(r + k); p < e0 + __ldg(r + k + 1); ++p) acc = far(acc, fmr(__ldg(valf + p), x[__ldg(gci + p)]));
        t[g] = acc;
    }
}

// rows of level l: x += (omega dinv) (b - t), the sweep after the correction
__global__ void k_dc_jacobi(int q0, int q1, int maxL, const int* __restrict__ rowLv, const AmgSysLv* __restrict__ lv,
                            const float* __restrict__ dinv, const float* b, const float* t, float* x, const KScal* ks) {
    for (int g = q0 + int(blockIdx.x * blockDim.x + threadIdx.x); g < q1; g += int(gridDim.x * blockDim.x)) {
        const int sl = __ldg(rowLv + g);
        if (__ldg(&lv[sl].coarse) || !sys_ok(ks, sl / maxL)) continue;
        x[g] = far(x[g], fmr(fmr(kOmega, __ldg(dinv + g)), fsr(b[g], t[g])));
    }
}

// second stage per block row: z1 = E x0 (the pressure component), tt = r - S_f z1 (float, from zero over the
// row's blocks and their columns), z = z1 + D^-1 tt, written as double
__global__ void __launch_bounds__(256) k_dc_second(int n, const int* __restrict__ rowSys, const int* __restrict__ rowPtr,
                                                   const int* __restrict__ col, const double* __restrict__ val, const float* x0,
                                                   const double* T, const float* __restrict__ bj, double* z, const KScal* ks) {
    for (int i = int(blockIdx.x * blockDim.x + threadIdx.x); i < n; i += int(gridDim.x * blockDim.x)) {
        if (!sys_ok(ks, __ldg(rowSys + i))) continue;
        float acc[3] = {0.f, 0.f, 0.f};
        for (int p = __ldg(rowPtr + i); p < __ldg(rowPtr + i + 1); ++p) {
            const double* B = val + size_t(p) * 9;
            const float xk[3] = {far(0.f, fmr(1.0f, x0[__ldg(col + p)])), 0.f, 0.f};
#pragma unroll
            for (int e = 0; e < 3; ++e)
#pragma unroll
                for (int f = 0; f < 3; ++f) acc[e] = far(acc[e], fmr(float(__ldg(B + e * 3 + f)), xk[f]));
        }
        float tt[3];
#pragma unroll
        for (int e = 0; e < 3; ++e) tt[e] = fsr(float(T[size_t(i) * 3 + e]), acc[e]);
        const float z1[3] = {far(0.f, fmr(1.0f, x0[i])), 0.f, 0.f};
        const float* D = bj + size_t(i) * 9;
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            float s2 = 0.f;
#pragma unroll
            for (int f = 0; f < 3; ++f) s2 = far(s2, fmr(__ldg(D + e * 3 + f), tt[f]));
            z[size_t(i) * 3 + e] = double(far(z1[e], s2));
        }
    }
}

}  // namespace

int devcpr_launches(const DevAmg& G) { return 3 + 5 * (G.maxL > 1 ? G.maxL - 1 : 0); }

int launch_devcpr_setup(const DevPlan& P, const double* val, DevAmg& G, cudaStream_t st) {
    if (G.totLu > 0) {
        k_dc_coarse_inverse<<<G.nsys, 256, 0, st>>>(G.maxL, G.lv, G.rp, G.ci, G.val, G.luPerm, G.dcWork, G.dcWorkOff, G.invf, G.dcOk);
    } else {
        cudaMemsetAsync(G.dcOk, 0, sizeof(int) * size_t(G.nsys), st);
    }
    k_dc_dinv<<<grid_of(G.totRows, 256), 256, 0, st>>>(G.totRows, G.diagGlob, G.val, G.dinvf);
    k_dc_bj<<<grid_of(P.n, 256), 256, 0, st>>>(P.n, P.diag, val, G.bjf);
    return G.totLu > 0 ? 3 : 2;
}

int launch_devcpr(const DevPlan& P, const DevAmg& G, const double* val, int mode, const double* r, double* pv, const double* v, double* z,
                  const KScal* ks, cudaStream_t st) {
    const int n = P.n, gn = grid_of(n, 256);
    float *x = G.xf, *b = G.bf, *t = G.rf;
    if (mode == DC_PUPDATE) k_dc_in<DC_PUPDATE><<<gn, 256, 0, st>>>(n, P.rowSys, r, pv, v, G.w, G.T, b, ks);
    else if (mode == DC_SUPDATE) k_dc_in<DC_SUPDATE><<<gn, 256, 0, st>>>(n, P.rowSys, r, pv, v, G.w, G.T, b, ks);
    else k_dc_in<DC_PLAIN><<<gn, 256, 0, st>>>(n, P.rowSys, r, pv, v, G.w, G.T, b, ks);
    const auto& LB = G.levelRowBeg;
    for (int l = 0; l + 1 < G.maxL; ++l) {
        const int q0 = LB[size_t(l)], q1 = LB[size_t(l) + 1], c1 = LB[size_t(l) + 2];
        k_dc_smooth0<<<grid_of(q1 - q0, 256), 256, 0, st>>>(q0, q1, G.maxL, G.rowLv, G.lv, G.dinvf, b, x, ks);
        k_dc_restrict<<<grid_of(c1 - q1, 256), 256, 0, st>>>(q1, c1, G.maxL, G.rowLv, G.lv, G.rp, G.gci, G.valf, G.memPtr, G.mem, b, x, ks);
    }
    const size_t smem = size_t(G.maxCoarse) * (sizeof(float) + sizeof(int));
    k_dc_coarse<<<G.nsys, 256, smem, st>>>(G.maxL, G.lv, G.rp, G.gci, G.valf, G.dinvf, G.luPerm, G.invf, G.dcOk, b, x, t, ks);
    for (int l = G.maxL - 2; l >= 0; --l) {
        const int q0 = LB[size_t(l)], q1 = LB[size_t(l) + 1], g = grid_of(q1 - q0, 256);
        k_dc_prolong<<<g, 256, 0, st>>>(q0, q1, G.maxL, G.rowLv, G.lv, G.agg, x, ks);
        k_dc_spmv<<<g, 256, 0, st>>>(q0, q1, G.maxL, G.rowLv, G.lv, G.rp, G.gci, G.valf, x, t, ks);
        k_dc_jacobi<<<g, 256, 0, st>>>(q0, q1, G.maxL, G.rowLv, G.lv, G.dinvf, b, t, x, ks);
    }
    k_dc_second<<<gn, 256, 0, st>>>(n, P.rowSys, P.rowPtr, P.col, val, x, G.T, G.bjf, z, ks);
    return devcpr_launches(G);
}

}  // namespace rsg
