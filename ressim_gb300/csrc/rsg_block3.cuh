// FP64 3x3 block helpers shared by the device translation units (internal linkage in each).
// Multiplies and adds are explicitly rounded (never fused) and follow the reference's loop order
// (engine/src/bsr.cpp:13-87), so results are bitwise those of the reference's serial code.
#pragma once
#include <cuda_runtime.h>

namespace rsg {
namespace {

// ------------------------------------------------------------------ FP64 block arithmetic, reference order, unfused
__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

// c = a b   (engine/src/bsr.cpp:26-32: row accumulator, k outer, j inner)
__device__ __forceinline__ void gemm3(const double* a, const double* b, double* c) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        double r0 = 0, r1 = 0, r2 = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double f = a[i * 3 + k];
            r0 = da(r0, dm(f, b[k * 3 + 0]));
            r1 = da(r1, dm(f, b[k * 3 + 1]));
            r2 = da(r2, dm(f, b[k * 3 + 2]));
        }
        c[i * 3 + 0] = r0; c[i * 3 + 1] = r1; c[i * 3 + 2] = r2;
    }
}
// c -= a b  (engine/src/bsr.cpp:33-39)
__device__ __forceinline__ void gemm3_sub(const double* a, const double* b, double* c) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        double r0 = 0, r1 = 0, r2 = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double f = a[i * 3 + k];
            r0 = da(r0, dm(f, b[k * 3 + 0]));
            r1 = da(r1, dm(f, b[k * 3 + 1]));
            r2 = da(r2, dm(f, b[k * 3 + 2]));
        }
        c[i * 3 + 0] = ds(c[i * 3 + 0], r0); c[i * 3 + 1] = ds(c[i * 3 + 1], r1); c[i * 3 + 2] = ds(c[i * 3 + 2], r2);
    }
}
// one row of a 3x3 block times a 3-vector, accumulated from zero left to right
__device__ __forceinline__ double dot3(const double* a, const double* x) {
    return da(da(dm(a[0], x[0]), dm(a[1], x[1])), dm(a[2], x[2]));
}

// engine/src/bsr.cpp:67-87 for nb = 3: Gauss-Jordan on [A | I], partial pivoting, singular below 1e-14 max|a|
__device__ bool invert3(double* a) {
    double m[3][6];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) { m[i][j] = a[i * 3 + j]; m[i][3 + j] = (i == j) ? 1.0 : 0.0; }
    double scale = 0;
#pragma unroll
    for (int i = 0; i < 9; ++i) scale = fmax(scale, fabs(a[i]));
    if (!(scale > 0) || !isfinite(scale)) return false;
    for (int k = 0; k < 3; ++k) {
        int pr = k;
        for (int i = k + 1; i < 3; ++i)
            if (fabs(m[i][k]) > fabs(m[pr][k])) pr = i;
        if (fabs(m[pr][k]) <= dm(1e-14, scale)) return false;
        if (pr != k)
            for (int j = 0; j < 6; ++j) { const double t = m[k][j]; m[k][j] = m[pr][j]; m[pr][j] = t; }
        const double inv = __ddiv_rn(1.0, m[k][k]);
        for (int j = 0; j < 6; ++j) m[k][j] = dm(m[k][j], inv);
        for (int i = 0; i < 3; ++i) {
            if (i == k || m[i][k] == 0.0) continue;
            const double f = m[i][k];
            for (int j = 0; j < 6; ++j) m[i][j] = ds(m[i][j], dm(f, m[k][j]));
        }
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) a[i * 3 + j] = m[i][3 + j];
    return true;
}
// pivot inversion with the reference's regularisation of singular blocks (engine/src/bsr.cpp:204-212);
// returns 1 when the block had to be regularised
__device__ int invert_pivot3(double* d) {
    double tmp[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) tmp[e] = d[e];
    if (invert3(d)) return 0;
    double sc = 0;
#pragma unroll
    for (int e = 0; e < 9; ++e) sc = fmax(sc, fabs(tmp[e]));
    if (!(sc > 0) || !isfinite(sc)) sc = 1.0;
#pragma unroll
    for (int e = 0; e < 9; ++e) d[e] = tmp[e];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const double de = d[e * 4];
        d[e * 4] = da(de, da(dm(de >= 0 ? 1e-8 : -1e-8, sc), de == 0 ? dm(sc, 1e-8) : 0.0));
    }
    if (!invert3(d)) {
#pragma unroll
        for (int e = 0; e < 9; ++e) d[e] = 0;
        const double inv = __ddiv_rn(1.0, sc);
        d[0] = inv; d[4] = inv; d[8] = inv;
    }
    return 1;
}

__device__ __forceinline__ void load9(const double* p, double* a) {
#pragma unroll
    for (int e = 0; e < 9; ++e) a[e] = p[e];
}
__device__ __forceinline__ void store9(double* p, const double* a) {
#pragma unroll
    for (int e = 0; e < 9; ++e) p[e] = a[e];
}
__device__ __forceinline__ void load9_ro(const double* p, double* a) {
#pragma unroll
    for (int e = 0; e < 9; ++e) a[e] = __ldg(p + e);
}


}  // namespace
}  // namespace rsg
