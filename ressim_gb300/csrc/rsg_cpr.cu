// CPR set-up on the device (BlockCPR::setup, engine/src/bsr.cpp:993-1059; AMG::refresh / factorCoarsest,
// engine/src/amg.cpp:257-295): decoupling weights, pressure matrix, Galerkin values of the coarse levels in the
// reference's summation order, and the dense LU of the coarsest level. All FP64 arithmetic explicitly rounded.
#include "rsg_impl.h"
#include "rsg_block3.cuh"

#include <cuda_runtime.h>

namespace rsg {

namespace {

int grid_for(size_t work) {
    const size_t g = (work + 255) / 256, cap = size_t(device_sm_count()) * 16;
    return int(g < cap ? (g > 0 ? g : 1) : cap);
}

__global__ void k_gather_acc(int n, const int* __restrict__ perm, const double* __restrict__ acc, double* out) {
    for (size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x; q < size_t(n) * 9; q += size_t(gridDim.x) * blockDim.x)
        out[q] = __ldg(acc + size_t(__ldg(perm + q / 9)) * 9 + q % 9);
}

// w_i = first row of D^-1, D = accumulation block when its 1-norm condition estimate is <= 1e10 (true IMPES),
// else the Jacobian diagonal block (quasi IMPES); fallbacks as engine/src/bsr.cpp:1000-1040
__global__ void k_cpr_weights(int n, const int* __restrict__ diag, const double* __restrict__ val, const double* __restrict__ acc,
                              double* w, int* nfallback) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double D[9];
    load9_ro(val + size_t(__ldg(diag + k)) * 9, D);
    bool inverted = false;
    if (acc) {
        double B[9], inv[9];
        load9_ro(acc + size_t(k) * 9, B);
        for (int e = 0; e < 9; ++e) inv[e] = B[e];
        if (invert3(inv)) {
            double n1 = 0, ni = 0;
            for (int j = 0; j < 3; ++j) {
                double c = 0, d = 0;
                for (int r = 0; r < 3; ++r) { c = da(c, fabs(B[r * 3 + j])); d = da(d, fabs(inv[r * 3 + j])); }
                n1 = fmax(n1, c);
                ni = fmax(ni, d);
            }
            if (dm(n1, ni) <= 1e10) { for (int e = 0; e < 9; ++e) D[e] = inv[e]; inverted = true; }
            else atomicAdd(nfallback, 1);
        } else {
            atomicAdd(nfallback, 1);
        }
    }
    double wk[3];
    if (inverted || invert3(D)) {
        wk[0] = D[0]; wk[1] = D[1]; wk[2] = D[2];
    } else {
        double s = 0;
        const double* A = val + size_t(__ldg(diag + k)) * 9;
        for (int e = 0; e < 3; ++e) s = da(s, __ldg(A + e * 3));
        for (int e = 0; e < 3; ++e) wk[e] = fabs(s) > 1e-300 ? __ddiv_rn(1.0, s) : 1.0;
    }
    double wm = 0;
    for (int e = 0; e < 3; ++e) wm = fmax(wm, fabs(wk[e]));
    if (!(wm > 0) || !isfinite(wm)) wk[0] = wk[1] = wk[2] = 1.0;
    w[size_t(k) * 3 + 0] = wk[0]; w[size_t(k) * 3 + 1] = wk[1]; w[size_t(k) * 3 + 2] = wk[2];
}

// Ap_ij = sum_e w_ie S_ij[e][0] on S's block pattern (engine/src/bsr.cpp:1044-1053), tiny diagonals -> 1
__global__ void k_cpr_pressure(int n, const int* __restrict__ rowPtr, const int* __restrict__ diag, const double* __restrict__ val,
                               const double* __restrict__ w, double* ap) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double w0 = w[size_t(k) * 3], w1 = w[size_t(k) * 3 + 1], w2 = w[size_t(k) * 3 + 2];
    for (int p = __ldg(rowPtr + k); p < __ldg(rowPtr + k + 1); ++p) {
        const double* a = val + size_t(p) * 9;
        ap[p] = da(da(dm(w0, __ldg(a)), dm(w1, __ldg(a + 3))), dm(w2, __ldg(a + 6)));
    }
    const int d = __ldg(diag + k);
    if (fabs(ap[d]) < 1e-300) ap[d] = 1.0;
}

// Galerkin refresh of one level: AP entries, then the level's entries, in the reference's order (first term
// assigned, the others added)
__global__ void k_gather_sum(int beg, int end, const int* __restrict__ ptr, const int* __restrict__ src, const double* __restrict__ in,
                             double* out) {
    for (int e = beg + int(blockIdx.x * blockDim.x + threadIdx.x); e < end; e += int(gridDim.x * blockDim.x)) {
        const int q0 = __ldg(ptr + e), q1 = __ldg(ptr + e + 1);
        double s = 0;
        if (q0 < q1) {
            s = in[__ldg(src + q0)];
            for (int q = q0 + 1; q < q1; ++q) s = da(s, in[__ldg(src + q)]);
        }
        out[e] = s;
    }
}
__global__ void k_diag_fix(int beg, int end, const int* __restrict__ diagGlob, double* val) {
    for (int i = beg + int(blockIdx.x * blockDim.x + threadIdx.x); i < end; i += int(gridDim.x * blockDim.x)) {
        const int d = __ldg(diagGlob + i);
        if (fabs(val[d]) < 1e-300) val[d] = 1.0;
    }
}

// dense LU with partial pivoting of every system's coarsest level in its natural numbering
// (engine/src/amg.cpp:273-295); one thread block per system. T = double (reference arithmetic) or float (the FP32
// hierarchy of the precision forms: same algorithm, float operations).
__device__ __forceinline__ double cmul(double a, double b) { return dm(a, b); }
__device__ __forceinline__ double csub(double a, double b) { return ds(a, b); }
__device__ __forceinline__ double cdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float cmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float csub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float cdiv(float a, float b) { return __fdiv_rn(a, b); }
template <class T> __device__ __forceinline__ T tiny_pivot();
template <> __device__ __forceinline__ double tiny_pivot<double>() { return 1e-300; }
template <> __device__ __forceinline__ float tiny_pivot<float>() { return 1.17549435e-38f; }   // smallest normal float

template <class T>
__global__ void __launch_bounds__(256) k_coarse_lu(int nsys, int maxL, const AmgSysLv* __restrict__ lv, const int* __restrict__ rp,
                                                   const int* __restrict__ ci, const double* __restrict__ val,
                                                   const int* __restrict__ luPerm, T* luAll, int* pivAll, int* cinAll,
                                                   int skipUpTo, const int* only) {
    const int s = blockIdx.x;
    if (only && !only[s]) return;                                 // only the systems flagged (FP64 coarse solve)
    AmgSysLv L;
    bool found = false;
    for (int l = 0; l < maxL; ++l) {
        const AmgSysLv c = lv[s * maxL + l];
        if (c.n > 0 && c.coarse) { L = c; found = true; break; }
    }
    if (!found || !L.dense || L.n <= skipUpTo) return;        // skipUpTo: levels inverted in shared memory
    const int m = L.n;
    T* lu = luAll + L.luOff;
    int* piv = pivAll + L.luRowOff;
    const int* nat = luPerm + L.luRowOff;
    for (size_t q = threadIdx.x; q < size_t(m) * m; q += blockDim.x) lu[q] = T(0);
    __syncthreads();
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        const int I = __ldg(nat + k);
        for (int p = __ldg(rp + L.rpOff + k); p < __ldg(rp + L.rpOff + k + 1); ++p)
            lu[size_t(I) * m + __ldg(nat + __ldg(ci + L.entOff + p))] = T(val[L.entOff + p]);
    }
    __syncthreads();
    __shared__ T smax[256];
    __shared__ int sidx[256];
    for (int k = 0; k < m; ++k) {
        // pivot: first row with the largest |a_ik|, i >= k
        T best = T(-1);
        int bi = m;
        for (int i = k + int(threadIdx.x); i < m; i += blockDim.x) {
            const T a = fabs(lu[size_t(i) * m + k]);
            if (a > best || (a == best && i < bi)) { best = a; bi = i; }
        }
        smax[threadIdx.x] = best;
        sidx[threadIdx.x] = bi;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if (int(threadIdx.x) < o) {
                const T b2 = smax[threadIdx.x + o];
                const int i2 = sidx[threadIdx.x + o];
                if (b2 > smax[threadIdx.x] || (b2 == smax[threadIdx.x] && i2 < sidx[threadIdx.x])) { smax[threadIdx.x] = b2; sidx[threadIdx.x] = i2; }
            }
            __syncthreads();
        }
        // reference: pr starts at k and moves only on a strictly larger value -> first maximum
        const int pr = (smax[0] > fabs(lu[size_t(k) * m + k])) ? sidx[0] : k;
        __syncthreads();
        if (threadIdx.x == 0) piv[k] = pr;
        if (pr != k)
            for (int j = threadIdx.x; j < m; j += blockDim.x) {
                const T t = lu[size_t(k) * m + j];
                lu[size_t(k) * m + j] = lu[size_t(pr) * m + j];
                lu[size_t(pr) * m + j] = t;
            }
        __syncthreads();
        if (threadIdx.x == 0 && fabs(lu[size_t(k) * m + k]) < tiny_pivot<T>()) lu[size_t(k) * m + k] = tiny_pivot<T>();
        __syncthreads();
        const T dk = lu[size_t(k) * m + k];
        for (int i = k + 1 + int(threadIdx.x); i < m; i += blockDim.x) lu[size_t(i) * m + k] = cdiv(lu[size_t(i) * m + k], dk);
        __syncthreads();
        const int w = m - k - 1;
        for (size_t q = threadIdx.x; q < size_t(w) * w; q += blockDim.x) {
            const int i = k + 1 + int(q / w), j = k + 1 + int(q % w);
            const T f = lu[size_t(i) * m + k];
            if (f != T(0)) lu[size_t(i) * m + j] = csub(lu[size_t(i) * m + j], cmul(f, lu[size_t(k) * m + j]));
        }
        __syncthreads();
    }
    // gather order of the solve: the level-space row whose value lands at position i once the natural-order
    // vector has gone through the row interchanges piv[0], piv[1], ... (engine/src/amg.cpp:306-308)
    int* cin = cinAll + L.luRowOff;
    for (int k = threadIdx.x; k < m; k += blockDim.x) cin[__ldg(nat + k)] = k;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < m; ++k) {
            const int pk = piv[k];
            if (pk != k) { const int t = cin[k]; cin[k] = cin[pk]; cin[pk] = t; }
        }
}

// Explicit inverse of every coarsest level for the FP32 precision forms (the reference's device-shaped CPR keeps an
// explicit coarse inverse, engine/src/bsr.cpp:1235-1317): column j = LU^-1 e_j of the level-space unit vector,
// stored in natural row order: inv[j * m + nat(k)] = (A^-1)_{k j} (k_coarse_perm then moves it to the V-cycle's
// level-space layout). All m columns are eliminated together by the
// block, column-oriented, in an m x m shared-memory work matrix (m <= kInvSmemRows), else one column per thread in
// global memory.
constexpr int kInvSmemRows = 224;
__global__ void __launch_bounds__(256) k_coarse_inv(int maxL, const AmgSysLv* __restrict__ lv, const int* __restrict__ cinAll,
                                                    const float* __restrict__ luAll, float* invAll, int skipUpTo) {
    extern __shared__ float W[];
    const int s = blockIdx.x;
    AmgSysLv L;
    bool found = false;
    for (int l = 0; l < maxL; ++l) {
        const AmgSysLv c = lv[s * maxL + l];
        if (c.n > 0 && c.coarse) { L = c; found = true; break; }
    }
    if (!found || !L.dense || L.n <= skipUpTo) return;
    const int m = L.n;
    const float* lu = luAll + L.luOff;
    const int* cin = cinAll + L.luRowOff;
    float* inv = invAll + L.luOff;
    if (m <= kInvSmemRows && m <= int(blockDim.x)) {
        // thread j owns column j of the work matrix W[i * m + j] (consecutive threads, consecutive banks); column k
        // of the factors is staged in shared memory for each elimination step and read by all threads
        float* lc = W + m * m;
        const int j = threadIdx.x;
        if (j < m)
            for (int i = 0; i < m; ++i) W[i * m + j] = __ldg(cin + i) == j ? 1.f : 0.f;   // pivoted e_j
        for (int k = 0; k + 1 < m; ++k) {                                         // unit lower
            __syncthreads();
            for (int i = threadIdx.x; i < m; i += blockDim.x) lc[i] = __ldg(lu + size_t(i) * m + k);
            __syncthreads();
            if (j < m) {
                const float wk = W[k * m + j];
                if (wk != 0.f)
                    for (int i = k + 1; i < m; ++i) W[i * m + j] = __fsub_rn(W[i * m + j], __fmul_rn(lc[i], wk));
            }
        }
        for (int k = m - 1; k >= 0; --k) {                                        // upper
            __syncthreads();
            for (int i = threadIdx.x; i < m; i += blockDim.x) lc[i] = __ldg(lu + size_t(i) * m + k);
            __syncthreads();
            if (j < m) {
                const float wk = __fdiv_rn(W[k * m + j], lc[k]);
                W[k * m + j] = wk;
                if (wk != 0.f)
                    for (int i = 0; i < k; ++i) W[i * m + j] = __fsub_rn(W[i * m + j], __fmul_rn(lc[i], wk));
            }
        }
        __syncthreads();
        for (int q = threadIdx.x; q < m * m; q += blockDim.x) {
            const int jj = q / m, i = q - jj * m;
            inv[q] = W[i * m + jj];
        }
        return;
    }
    for (int j = threadIdx.x; j < m; j += blockDim.x) {
        float* w = inv + size_t(j) * m;
        for (int i = 0; i < m; ++i) w[i] = __ldg(cin + i) == j ? 1.f : 0.f;
        for (int i = 1; i < m; ++i) {
            float t = w[i];
            for (int k = 0; k < i; ++k) t = __fsub_rn(t, __fmul_rn(__ldg(lu + size_t(i) * m + k), w[k]));
            w[i] = t;
        }
        for (int i = m - 1; i >= 0; --i) {
            float t = w[i];
            for (int k = i + 1; k < m; ++k) t = __fsub_rn(t, __fmul_rn(__ldg(lu + size_t(i) * m + k), w[k]));
            w[i] = __fdiv_rn(t, __ldg(lu + size_t(i) * m + i));
        }
    }
}

// FP32 forms: the coarsest inverse directly, by Gauss-Jordan elimination with partial pivoting on the dense matrix
// in its natural numbering (m <= kInvSmemRows); the inverse is written as inv[j * m + I] = (A^-1)[I][nat(j)], which
// k_coarse_perm turns into the V-cycle's layout. Larger levels take the LU (k_coarse_lu<float>) and k_coarse_inv.
// The work matrix lives in registers: 16 warps, row i in warp i % 16, column j in lane j % 32, so a thread holds
// a 14 x 7 tile and a step's rank-1 update is register arithmetic. Per step, the pivot column (staged in shared
// memory by its owning lane during the previous update) is searched by every warp on its own; the pivot row and
// row k go through shared memory for the interchange and the scaled pivot row. Every element gets the same
// separately rounded operations as a column-per-thread elimination in shared memory.
constexpr int kGjThreads = 512;
constexpr int kGjWarps = kGjThreads / 32;
constexpr int kGjRows = (kInvSmemRows + kGjWarps - 1) / kGjWarps;   // register rows per thread
constexpr int kGjCols = (kInvSmemRows + 31) / 32;                  // register columns per thread
__global__ void __launch_bounds__(kGjThreads, 1) k_coarse_gj(int maxL, const AmgSysLv* __restrict__ lv, const int* __restrict__ rp,
                                                            const int* __restrict__ ci, const double* __restrict__ val,
                                                            const int* __restrict__ luPerm, float* invAll) {
    extern __shared__ float W[];
    const int s = blockIdx.x, tid = int(threadIdx.x), nt = int(blockDim.x), lane = tid & 31, wg = tid >> 5;
    AmgSysLv L;
    bool found = false;
    for (int l = 0; l < maxL; ++l) {
        const AmgSysLv c = lv[s * maxL + l];
        if (c.n > 0 && c.coarse) { L = c; found = true; break; }
    }
    if (!found || !L.dense) return;
    const int m = L.n;
    if (m > kInvSmemRows || nt != kGjThreads) return;          // left to the LU path
    __shared__ float colk[2][kGjWarps * kGjRows];               // column k of the current step, then of the next
    __shared__ float rowK[32 * kGjCols], rowP[32 * kGjCols];   // rows k and p before the interchange
    __shared__ int perm[kInvSmemRows];
    const int* nat = luPerm + L.luRowOff;
    for (int q = tid; q < m * m; q += nt) W[q] = 0.f;
    __syncthreads();
    for (int k = tid; k < m; k += nt) {
        const int I = __ldg(nat + k);
        for (int p = __ldg(rp + L.rpOff + k); p < __ldg(rp + L.rpOff + k + 1); ++p)
            W[I * m + __ldg(nat + __ldg(ci + L.entOff + p))] = float(val[L.entOff + p]);
    }
    __syncthreads();
    float R[kGjRows][kGjCols];
#pragma unroll
    for (int r = 0; r < kGjRows; ++r)
#pragma unroll
        for (int c = 0; c < kGjCols; ++c) {
            const int i = wg + kGjWarps * r, j = lane + 32 * c;
            R[r][c] = (i < m && j < m) ? W[i * m + j] : 0.f;
        }
    for (int i = tid; i < kGjWarps * kGjRows; i += nt) colk[0][i] = i < m ? W[i * m] : 0.f;
    for (int k = 0; k < m; ++k) {
        const float* ck = colk[k & 1];
        __syncthreads();
        // pivot: largest |a_ik|, i >= k (first on ties), found by every warp
        float best = -1.f;
        int bi = m;
        for (int i = k + lane; i < m; i += 32) {
            const float a = fabsf(ck[i]);
            if (a > best) { best = a; bi = i; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float b2 = __shfl_xor_sync(0xffffffffu, best, o);
            const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
            if (b2 > best || (b2 == best && i2 < bi)) { best = b2; bi = i2; }
        }
        const int p = bi < m ? bi : k;                          // no comparable entry (NaN column): no interchange
        // (register rows and columns are picked by select chains: an indexed access would move the tile to local
        // memory)
        if (wg == k % kGjWarps) {
            const int rk = k / kGjWarps;
#pragma unroll
            for (int c = 0; c < kGjCols; ++c) {
                float v = R[0][c];
#pragma unroll
                for (int r = 1; r < kGjRows; ++r) v = rk == r ? R[r][c] : v;
                rowK[lane + 32 * c] = v;
            }
        }
        if (wg == p % kGjWarps) {
            const int rp = p / kGjWarps;
#pragma unroll
            for (int c = 0; c < kGjCols; ++c) {
                float v = R[0][c];
#pragma unroll
                for (int r = 1; r < kGjRows; ++r) v = rp == r ? R[r][c] : v;
                rowP[lane + 32 * c] = v;
            }
        }
        if (tid == 0) perm[k] = p;
        __syncthreads();
        float d = ck[p];
        if (fabsf(d) < 1.17549435e-38f) d = 1.17549435e-38f;                     // singular: smallest normal pivot
        float akj[kGjCols];                                                       // the scaled pivot row
#pragma unroll
        for (int c = 0; c < kGjCols; ++c) {
            const int j = lane + 32 * c;
            akj[c] = j == k ? __fdiv_rn(1.f, d) : __fdiv_rn(rowP[j], d);
        }
        if (p != k && wg == p % kGjWarps) {                                       // row p takes row k
            const int rp = p / kGjWarps;
#pragma unroll
            for (int c = 0; c < kGjCols; ++c) {
                const float v = rowK[lane + 32 * c];
#pragma unroll
                for (int r = 0; r < kGjRows; ++r) R[r][c] = rp == r ? v : R[r][c];
            }
        }
        const float ckk = ck[k];
#pragma unroll
        for (int r = 0; r < kGjRows; ++r) {
            const int i = wg + kGjWarps * r;
            const float cik = i == p ? ckk : ck[i];                              // column k after the interchange
#pragma unroll
            for (int c = 0; c < kGjCols; ++c) {
                const int j = lane + 32 * c;
                R[r][c] = i == k ? akj[c] : __fsub_rn(j == k ? 0.f : R[r][c], __fmul_rn(cik, akj[c]));
            }
        }
        const int kn = k + 1;                                   // the next pivot column, by its owning lane
        if (kn < m && lane == kn % 32) {
            float* cn = colk[kn & 1];
            const int kc = kn / 32;
#pragma unroll
            for (int r = 0; r < kGjRows; ++r) {
                float v = R[r][0];
#pragma unroll
                for (int c = 1; c < kGjCols; ++c) v = kc == c ? R[r][c] : v;
                cn[wg + kGjWarps * r] = v;
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kGjRows; ++r)
#pragma unroll
        for (int c = 0; c < kGjCols; ++c) {
            const int i = wg + kGjWarps * r, j = lane + 32 * c;
            if (i < m && j < m) W[i * m + j] = R[r][c];
        }
    __syncthreads();
    const int j = tid;
    // the row interchanges of the elimination become column interchanges of the inverse, in reverse order
    if (j < m)
        for (int k = m - 1; k >= 0; --k) {
            const int p = perm[k];
            if (p != k) { const float t = W[j * m + k]; W[j * m + k] = W[j * m + p]; W[j * m + p] = t; }
        }
    __syncthreads();
    float* inv = invAll + L.luOff;
    for (int q = threadIdx.x; q < m * m; q += blockDim.x) {
        const int jj = q / m, I = q - jj * m;
        inv[q] = W[I * m + __ldg(nat + jj)];
    }
}

// V-cycle row slots from the level values (zero padding), FP32 copies for the FP32 V-cycle
__global__ void k_amg_slots(int totSlots, int totRows, const int* __restrict__ slotSrc, const int* __restrict__ diagGlob,
                            const double* __restrict__ val, double* slotVal, float* slotValf, double* diagVal, float* diagValf) {
    const int total = totSlots + totRows;
    for (int q = int(blockIdx.x * blockDim.x + threadIdx.x); q < total; q += int(gridDim.x * blockDim.x)) {
        if (q < totSlots) {
            const int src = __ldg(slotSrc + q);
            const double v = src >= 0 ? val[src] : 0.0;
            slotVal[q] = v;
            if (slotValf) slotValf[q] = float(v);
        } else {
            const int g = q - totSlots;
            const double v = val[__ldg(diagGlob + g)];
            diagVal[g] = v;
            if (diagValf) diagValf[g] = float(v);
        }
    }
}

// pressure columns S_ij[e][0] of the second stage in the factors' slot order: per row SPREC values (L slots,
// diagonal, U slots, padding), overflow blocks 3 values each
template <class T>
__device__ __forceinline__ void put_sp(const double* __restrict__ val, int src, T* out) {
    for (int e = 0; e < 3; ++e) out[e] = src >= 0 ? T(val[size_t(src) * 9 + size_t(e) * 3]) : T(0);
}
__global__ void k_cpr_sp(int n, int nLov, int nUov, const int* __restrict__ LslotSrc, const int* __restrict__ UslotSrc,
                         const int* __restrict__ Dsrc, const int* __restrict__ LovSrc, const int* __restrict__ UovSrc,
                         const double* __restrict__ val, double* sp, float* spf, double* spLov, float* spLovf, double* spUov,
                         float* spUovf) {
    const int total = n + nLov + nUov;
    for (int q = int(blockIdx.x * blockDim.x + threadIdx.x); q < total; q += int(gridDim.x * blockDim.x)) {
        if (q < n) {
            const int k = q;
            int src[2 * SLOTS + 1];
            for (int j = 0; j < SLOTS; ++j) {
                src[j] = __ldg(LslotSrc + size_t(k) * SLOTS + j);
                src[SLOTS + 1 + j] = __ldg(UslotSrc + size_t(k) * SLOTS + j);
            }
            src[SLOTS] = __ldg(Dsrc + k);
            if (spf) {
                float* o = spf + size_t(k) * SPREC;
                for (int j = 0; j < 2 * SLOTS + 1; ++j) put_sp(val, src[j], o + 3 * j);
                for (int e = 3 * (2 * SLOTS + 1); e < SPREC; ++e) o[e] = 0.f;
            } else {
                double* o = sp + size_t(k) * SPREC;
                for (int j = 0; j < 2 * SLOTS + 1; ++j) put_sp(val, src[j], o + 3 * j);
                for (int e = 3 * (2 * SLOTS + 1); e < SPREC; ++e) o[e] = 0.0;
            }
        } else if (q < n + nLov) {
            const int i = q - n, src = __ldg(LovSrc + i);
            if (spLovf) put_sp(val, src, spLovf + size_t(i) * 3);
            else put_sp(val, src, spLov + size_t(i) * 3);
        } else {
            const int i = q - n - nLov, src = __ldg(UovSrc + i);
            if (spUovf) put_sp(val, src, spUovf + size_t(i) * 3);
            else put_sp(val, src, spUov + size_t(i) * 3);
        }
    }
}

__global__ void k_round(size_t n, const double* __restrict__ a, float* b) {
    for (size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x; q < n; q += size_t(gridDim.x) * blockDim.x) b[q] = float(a[q]);
}

}  // namespace

void launch_gather_acc(const DevPlan& P, const double* accOrig, double* accLev, cudaStream_t st) {
    k_gather_acc<<<grid_for(size_t(P.n) * 9), 256, 0, st>>>(P.n, P.perm, accOrig, accLev);
}
void launch_cpr_weights(const DevPlan& P, const double* val, const double* accLev, double* w, int* nfallback, cudaStream_t st) {
    k_cpr_weights<<<(P.n + 127) / 128, 128, 0, st>>>(P.n, P.diag, val, accLev, w, nfallback);
}
void launch_cpr_pressure(const DevPlan& P, const double* val, const double* w, double* ap, cudaStream_t st) {
    k_cpr_pressure<<<(P.n + 127) / 128, 128, 0, st>>>(P.n, P.rowPtr, P.diag, val, w, ap);
}
void launch_amg_refresh(const DevAmg& G, cudaStream_t st) {
    for (int l = 1; l < G.maxL; ++l) {
        const int a0 = G.levelApBeg[size_t(l)], a1 = G.levelApBeg[size_t(l) + 1];
        const int e0 = G.levelEntBeg[size_t(l)], e1 = G.levelEntBeg[size_t(l) + 1];
        const int r0 = G.levelRowBeg[size_t(l)], r1 = G.levelRowBeg[size_t(l) + 1];
        if (e1 <= e0) continue;
        if (a1 > a0) k_gather_sum<<<grid_for(size_t(a1 - a0)), 256, 0, st>>>(a0, a1, G.apPtr, G.apSrc, G.val, G.apVal);
        k_gather_sum<<<grid_for(size_t(e1 - e0)), 256, 0, st>>>(e0, e1, G.acPtr, G.acSrc, G.apVal, G.val);
        k_diag_fix<<<grid_for(size_t(r1 - r0)), 256, 0, st>>>(r0, r1, G.diagGlob, G.val);
    }
}
// FP32 forms: the explicit inverses from the natural-row layout inv[j * m + I] = (A^-1)[I][nat(j)] to the layout the
// V-cycle reads, inv[j * m + k] = (A^-1)[nat(k)][nat(j)] (k, j level-space): the threads of consecutive rows k then
// read consecutive words of a column. One column at a time through shared memory, in place.
__global__ void __launch_bounds__(256) k_coarse_perm(int maxL, const AmgSysLv* __restrict__ lv, const int* __restrict__ luPerm,
                                                     float* invAll) {
    extern __shared__ float colbuf[];
    const int s = blockIdx.x;
    AmgSysLv L;
    bool found = false;
    for (int l = 0; l < maxL; ++l) {
        const AmgSysLv c = lv[s * maxL + l];
        if (c.n > 0 && c.coarse) { L = c; found = true; break; }
    }
    if (!found || !L.dense) return;
    const int m = L.n;
    const int* nat = luPerm + L.luRowOff;
    float* inv = invAll + L.luOff;
    for (int j = 0; j < m; ++j) {
        float* col = inv + size_t(j) * m;
        for (int i = threadIdx.x; i < m; i += blockDim.x) colbuf[i] = col[i];
        __syncthreads();
        for (int k = threadIdx.x; k < m; k += blockDim.x) col[k] = colbuf[__ldg(nat + k)];
        __syncthreads();
    }
}

// FP32 forms: how well the explicit FP32 inverse solves the coarsest level. x_t deterministic in [-1, 1), b = A x_t
// in FP64, x = inv float(b) as the V-cycle applies it; a system whose relative error exceeds kCoarseTol (or is not
// finite) solves its coarsest level in FP64 with the LU instead: extreme permeability contrasts (sigma ln k ~ 3)
// leave coarse matrices too ill-conditioned for an FP32 inverse, and the preconditioner then stalls.
constexpr double kCoarseTol = 1e-2;
__global__ void __launch_bounds__(256) k_coarse_check(int maxL, const AmgSysLv* __restrict__ lv, const int* __restrict__ rp,
                                                      const int* __restrict__ ci, const double* __restrict__ val,
                                                      const int* __restrict__ luPerm, const float* __restrict__ invAll, double* xt,
                                                      double* bt, int* coarse64) {
    const int s = blockIdx.x;
    AmgSysLv L;
    bool found = false;
    for (int l = 0; l < maxL; ++l) {
        const AmgSysLv c = lv[s * maxL + l];
        if (c.n > 0 && c.coarse) { L = c; found = true; break; }
    }
    if (!found || !L.dense) {
        if (threadIdx.x == 0) coarse64[s] = 0;
        return;
    }
    const int m = L.n;
    double* x = xt + L.rowOff;
    double* b = bt + L.rowOff;
    for (int k = threadIdx.x; k < m; k += blockDim.x) x[k] = double((unsigned(k) * 2654435761u) >> 8) * (2.0 / 16777216.0) - 1.0;
    __syncthreads();
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        double t = 0;
        for (int p = __ldg(rp + L.rpOff + k); p < __ldg(rp + L.rpOff + k + 1); ++p) t += val[L.entOff + p] * x[__ldg(ci + L.entOff + p)];
        b[k] = t;
    }
    __syncthreads();
    const float* inv = invAll + L.luOff;
    const int* nat = luPerm + L.luRowOff;
    double e2 = 0, r2 = 0;
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        const float* col = inv + k;                              // the V-cycle's layout (k_coarse_perm)
        float acc = 0.f;
#pragma unroll 16
        for (int j = 0; j < m; ++j) acc = fmaf(col[size_t(j) * m], float(b[j]), acc);
        const double d = double(acc) - x[k];
        e2 += d * d;
        r2 += x[k] * x[k];
    }
    __shared__ double se[256], sr[256];
    se[threadIdx.x] = e2;
    sr[threadIdx.x] = r2;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (int(threadIdx.x) < o) { se[threadIdx.x] += se[threadIdx.x + o]; sr[threadIdx.x] += sr[threadIdx.x + o]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double rel = sqrt(se[0] / sr[0]);
        coarse64[s] = (rel <= kCoarseTol) ? 0 : 1;              // NaN lands here too
    }
}

void launch_amg_coarse_lu(const DevAmg& G, bool fp32, cudaStream_t st) {
    if (G.totLu <= 0) return;
    if (fp32) {
        const int smem = int(sizeof(float)) * (kInvSmemRows * kInvSmemRows + kInvSmemRows);
        raise_smem_limit(reinterpret_cast<const void*>(k_coarse_gj), smem);
        k_coarse_gj<<<G.nsys, kGjThreads, smem, st>>>(G.maxL, G.lv, G.rp, G.ci, G.val, G.luPerm, G.invf);
        if (G.maxCoarse > kInvSmemRows) {                        // levels too large for shared memory: LU, then columns
            raise_smem_limit(reinterpret_cast<const void*>(k_coarse_inv), smem);
            k_coarse_lu<float><<<G.nsys, 256, 0, st>>>(G.nsys, G.maxL, G.lv, G.rp, G.ci, G.val, G.luPerm, G.luf, G.piv, G.cin,
                                                       kInvSmemRows, nullptr);
            k_coarse_inv<<<G.nsys, 256, smem, st>>>(G.maxL, G.lv, G.cin, G.luf, G.invf, kInvSmemRows);
        }
        k_coarse_perm<<<G.nsys, 256, size_t(std::max(G.maxCoarse, 1)) * sizeof(float), st>>>(G.maxL, G.lv, G.luPerm, G.invf);
        // the FP32 inverse checked per system; the FP64 LU (after the FP32 one: pivots and gather order are its own)
        // only for the systems that need it
        k_coarse_check<<<G.nsys, 256, 0, st>>>(G.maxL, G.lv, G.rp, G.ci, G.val, G.luPerm, G.invf, G.x, G.b, G.coarse64);
        k_coarse_lu<double><<<G.nsys, 256, 0, st>>>(G.nsys, G.maxL, G.lv, G.rp, G.ci, G.val, G.luPerm, G.lu, G.piv, G.cin, 0, G.coarse64);
    } else {
        k_coarse_lu<double><<<G.nsys, 256, 0, st>>>(G.nsys, G.maxL, G.lv, G.rp, G.ci, G.val, G.luPerm, G.lu, G.piv, G.cin, 0, nullptr);
    }
}
void launch_amg_round(const DevAmg& G, cudaStream_t st) {
    k_round<<<grid_for(size_t(G.totEnt)), 256, 0, st>>>(size_t(G.totEnt), G.val, G.valf);
}
void launch_amg_slots(const DevAmg& G, bool fp32, cudaStream_t st) {
    k_amg_slots<<<grid_for(size_t(G.totSlots) + size_t(G.totRows)), 256, 0, st>>>(G.totSlots, G.totRows, G.slotSrc, G.diagGlob, G.val,
                                                                                   G.slotVal, fp32 ? G.slotValf : nullptr, G.diagVal,
                                                                                   fp32 ? G.diagValf : nullptr);
}
void launch_cpr_sp(const DevPlan& P, const double* val, const DevAmg& G, bool fp32, cudaStream_t st) {
    k_cpr_sp<<<grid_for(size_t(P.n) + size_t(P.nLov) + size_t(P.nUov)), 256, 0, st>>>(
        P.n, P.nLov, P.nUov, P.LslotSrc, P.UslotSrc, P.Dsrc, P.LovSrc, P.UovSrc, val, G.sp, fp32 ? G.spf : nullptr, G.spLov,
        fp32 ? G.spLovf : nullptr, G.spUov, fp32 ? G.spUovf : nullptr);
}

}  // namespace rsg
