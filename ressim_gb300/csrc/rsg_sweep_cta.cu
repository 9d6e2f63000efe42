// CTA-per-system BILU0 application: exact natural-order ILU(0) sweeps for systems that fit one SM.
//
// One thread block owns one system of the (block-diagonal) batch and walks its forward levels with a block
// barrier between levels, then the same levels in reverse for the backward sweep (valid for the structurally
// symmetric patterns of reservoir Jacobians; the plan falls back to the grid-wide sync-free sweeps otherwise).
// The sweep vector stays in shared memory between the two sweeps (FP32: up to ~19k block rows per system),
// so every dependency read is a shared-memory read and the two sweeps are one kernel. Factors are read from
// the level-ordered split storage (strict lower / strict upper / diagonal inverses, rows of a level contiguous).
//
// FP64 arithmetic follows the reference loop order with unfused multiply / add (engine/src/bsr.cpp:565-587),
// so the FP64 result is bitwise that of the reference's serial sweeps. FP32 follows BILU0f
// (engine/src/bsr.cpp:1100-1121): float factors, float vector, float accumulation.
#include "rsg_impl.h"

#include <cuda_runtime.h>

namespace rsg {

namespace {

constexpr int kCtaThreads = 256;

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

template <class T>
struct Ar;
template <>
struct Ar<double> {
    static __device__ __forceinline__ double dot3(const double* a, const double* x) {
        return da(da(dm(__ldg(a), x[0]), dm(__ldg(a + 1), x[1])), dm(__ldg(a + 2), x[2]));
    }
    static __device__ __forceinline__ double sub(double a, double b) { return ds(a, b); }
};
template <>
struct Ar<float> {
    static __device__ __forceinline__ float dot3(const float* a, const float* x) {
        float s = 0.f;
        s += __ldg(a) * x[0];
        s += __ldg(a + 1) * x[1];
        s += __ldg(a + 2) * x[2];
        return s;
    }
    static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
};

enum { IN_PLAIN = 0, IN_PUPDATE = 1, IN_SUPDATE = 2 };

// YSM: sweep vector in shared memory; otherwise (FP64 only) it lives in z itself.
template <class T, int MODE, bool YSM>
__global__ void __launch_bounds__(kCtaThreads) k_ilu_cta(const int* __restrict__ sysRow0, const int* __restrict__ sysLvl0,
                                                        const int* __restrict__ lvlStart, const int* __restrict__ lrow,
                                                        const int* __restrict__ Lptr, const int* __restrict__ Lcol,
                                                        const T* __restrict__ Lv, const int* __restrict__ Uptr,
                                                        const int* __restrict__ Ucol, const T* __restrict__ Uv,
                                                        const T* __restrict__ Dv, const double* r, double* pv, const double* v,
                                                        double* z, const KScal* ks) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int s = blockIdx.x;
    const int row0 = __ldg(sysRow0 + s);
    double beta = 0, omega = 0, alpha = 0;
    if (ks) {
        const KScal& K = ks[s];
        if (K.status != ST_RUNNING) return;                // whole block: uniform
        beta = K.beta; omega = K.omega; alpha = K.alpha;
    }
    T* y = YSM ? reinterpret_cast<T*>(smraw) : reinterpret_cast<T*>(z + size_t(row0) * 3);
    const int l0 = __ldg(sysLvl0 + s), nl = __ldg(sysLvl0 + s + 1) - l0 - 1;
    // forward: y_i = in_i - sum_{k<i} L_ik y_k, level by level
    for (int L = 0; L < nl; ++L) {
        const int k0 = __ldg(lvlStart + l0 + L), k1 = __ldg(lvlStart + l0 + L + 1);
        for (int k = k0 + int(threadIdx.x); k < k1; k += blockDim.x) {
            const int i = __ldg(lrow + k);
            const int li = i - row0;
            T yi[3];
#pragma unroll
            for (int e = 0; e < 3; ++e) {
                const size_t q = size_t(i) * 3 + e;
                if (MODE == IN_PUPDATE) {
                    const double pe = da(r[q], dm(beta, ds(pv[q], dm(omega, v[q]))));   // engine/src/linsolve.cpp:173
                    pv[q] = pe;
                    yi[e] = T(pe);
                } else if (MODE == IN_SUPDATE) {
                    const double se = ds(r[q], dm(alpha, v[q]));                         // engine/src/linsolve.cpp:183
                    pv[q] = se;
                    yi[e] = T(se);
                } else {
                    yi[e] = T(r[q]);
                }
            }
            const int p1 = __ldg(Lptr + k + 1);
            for (int p = __ldg(Lptr + k); p < p1; ++p) {
                const int c = __ldg(Lcol + p);
                const T yc[3] = {y[c * 3 + 0], y[c * 3 + 1], y[c * 3 + 2]};
                const T* a = Lv + size_t(p) * 9;
                yi[0] = Ar<T>::sub(yi[0], Ar<T>::dot3(a, yc));
                yi[1] = Ar<T>::sub(yi[1], Ar<T>::dot3(a + 3, yc));
                yi[2] = Ar<T>::sub(yi[2], Ar<T>::dot3(a + 6, yc));
            }
            y[li * 3 + 0] = yi[0]; y[li * 3 + 1] = yi[1]; y[li * 3 + 2] = yi[2];
        }
        __syncthreads();
    }
    // backward: z_i = U_ii^-1 (y_i - sum_{j>i} U_ij z_j), levels in reverse
    for (int L = nl - 1; L >= 0; --L) {
        const int k0 = __ldg(lvlStart + l0 + L), k1 = __ldg(lvlStart + l0 + L + 1);
        for (int k = k0 + int(threadIdx.x); k < k1; k += blockDim.x) {
            const int i = __ldg(lrow + k);
            const int li = i - row0;
            T yi[3] = {y[li * 3 + 0], y[li * 3 + 1], y[li * 3 + 2]};
            const int p1 = __ldg(Uptr + k + 1);
            for (int p = __ldg(Uptr + k); p < p1; ++p) {
                const int c = __ldg(Ucol + p);
                const T yc[3] = {y[c * 3 + 0], y[c * 3 + 1], y[c * 3 + 2]};
                const T* a = Uv + size_t(p) * 9;
                yi[0] = Ar<T>::sub(yi[0], Ar<T>::dot3(a, yc));
                yi[1] = Ar<T>::sub(yi[1], Ar<T>::dot3(a + 3, yc));
                yi[2] = Ar<T>::sub(yi[2], Ar<T>::dot3(a + 6, yc));
            }
            const T* d = Dv + size_t(k) * 9;
            const T t0 = Ar<T>::dot3(d, yi), t1 = Ar<T>::dot3(d + 3, yi), t2 = Ar<T>::dot3(d + 6, yi);
            y[li * 3 + 0] = t0; y[li * 3 + 1] = t1; y[li * 3 + 2] = t2;
            if (YSM) {
                z[size_t(i) * 3 + 0] = double(t0);
                z[size_t(i) * 3 + 1] = double(t1);
                z[size_t(i) * 3 + 2] = double(t2);
            }
        }
        __syncthreads();
    }
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

template <class T, int MODE, bool YSM>
void launch_cta(const DevPlan& P, const SplitFactors<T>& F, size_t smem, const double* r, double* pv, const double* v, double* z,
                const KScal* ks, cudaStream_t st) {
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaFuncSetAttribute(k_ilu_cta<T, MODE, YSM>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        configured = smem;
    }
    k_ilu_cta<T, MODE, YSM><<<P.nsys, kCtaThreads, smem, st>>>(P.sysRow0, P.sysLvl0, P.lvlStart, P.lrow, P.Lptr, P.Lcol, F.L, P.Uptr,
                                                               P.Ucol, F.U, F.D, r, pv, v, z, ks);
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

}  // namespace

size_t cta_sweep_smem(const DevPlan& P, bool fp32) {
    const size_t need = size_t(P.maxSysRows) * 3 * (fp32 ? sizeof(float) : sizeof(double));
    return need <= size_t(max_smem_optin()) ? need : 0;
}

bool cta_sweep_supported(const DevPlan& P, const HostPlan& H) {
    // structurally symmetric (reversed forward levels are backward levels) and small enough for one SM
    return H.symmetric && P.maxSysRows > 0 && P.maxSysRows <= 32768;
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

// z = M^-1 r (plain input) -- the fused BiCGSTAB variants are launched by launch_ilu_cta_fused
void launch_ilu_cta_apply(const DevPlan& P, const PrecDev& M, const double* r, double* z, cudaStream_t st) {
    if (M.kind == 1) launch_cta<float, IN_PLAIN, true>(P, M.s32, M.smem, r, nullptr, nullptr, z, nullptr, st);
    else if (M.smem) launch_cta<double, IN_PLAIN, true>(P, M.s64, M.smem, r, nullptr, nullptr, z, nullptr, st);
    else launch_cta<double, IN_PLAIN, false>(P, M.s64, 0, r, nullptr, nullptr, z, nullptr, st);
}

void launch_ilu_cta_fused(const DevPlan& P, const PrecDev& M, bool pupdate, const double* r, double* pv, const double* v, double* z,
                          const KScal* ks, cudaStream_t st) {
    if (M.kind == 1) {
        if (pupdate) launch_cta<float, IN_PUPDATE, true>(P, M.s32, M.smem, r, pv, v, z, ks, st);
        else launch_cta<float, IN_SUPDATE, true>(P, M.s32, M.smem, r, pv, v, z, ks, st);
    } else if (M.smem) {
        if (pupdate) launch_cta<double, IN_PUPDATE, true>(P, M.s64, M.smem, r, pv, v, z, ks, st);
        else launch_cta<double, IN_SUPDATE, true>(P, M.s64, M.smem, r, pv, v, z, ks, st);
    } else {
        if (pupdate) launch_cta<double, IN_PUPDATE, false>(P, M.s64, 0, r, pv, v, z, ks, st);
        else launch_cta<double, IN_SUPDATE, false>(P, M.s64, 0, r, pv, v, z, ks, st);
    }
}

}  // namespace rsg
