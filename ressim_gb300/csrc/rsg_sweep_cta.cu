// Thread-block-per-system BILU0 and CPR application: exact natural-order ILU(0) sweeps and the CPR V-cycle for
// systems that fit one SM.
//
// One thread block owns one system of the (block-diagonal) batch and walks its forward levels with a block
// barrier between levels, then the same levels in reverse for the backward sweep (valid for the structurally
// symmetric patterns of reservoir Jacobians; otherwise the plan uses the grid-wide sync-free sweeps). Rows are
// in level space, so a level is a contiguous range of rows, of input vector entries and of factor records.
//
// Latency is the whole game in these sweeps (one level = one barrier and one dependent step), so:
// * factors are stored in slot records: per row a fixed 16-byte-multiple record of its first SLOTS blocks of L
//   (resp. U and the inverted diagonal) and a vector of their columns. A row's data sits at an address computed
//   from its index -- no pointer chasing -- and comes in as a few 16-byte loads;
// * every thread holds two register buffers and loads its next row into one while it works on the other, so a
//   row's loads are issued a whole level (work + barrier) before they are used;
// * thread 0 asks the bulk-copy unit to prefetch the records of the level kAhead levels ahead into L2
//   (cp.async.bulk.prefetch.L2), so the register loads above hit L2, not HBM;
// * the sweep vector y and the V-cycle vectors stay in shared memory when they fit (chosen per system).
// TF = factor storage type, TV = sweep vector type. FP64 (double, double) and mixed (float factors, double
// vector: the reference's float-factor sweeps, engine/src/bsr.cpp:500-522) use unfused multiply / add in the
// reference loop order, so their results are bitwise those of the reference's serial sweeps on the same
// factors. (float, float) is the all-FP32 BILU0f sweep (engine/src/bsr.cpp:1100-1121).
#include "rsg_impl.h"
#include "rsg_block3.cuh"
#include "rsg_sync.cuh"

#include <cuda_runtime.h>
#include <type_traits>

namespace rsg {

namespace {

constexpr int kCtaThreads = 256;
// threads per block of a sweep / CPR kernel (a template parameter of the kernels). 512 threads for the all-FP32
// forms measured slower on the 64-system ensemble (the V-cycle phases spill at 128 registers), so all forms use 256.
template <class TF, class TV>
__host__ __device__ constexpr int cta_threads() { return 256; }
constexpr int kAhead = 4;                  // levels prefetched into L2 ahead of the sweep front

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

// L2 prefetch of bytes [b, e) of base by the bulk-copy unit. The bulk unit wants a 16-byte aligned address and
// a 16-byte multiple size: the range is rounded inward on the absolute addresses, so it never leaves [b, e)
// whatever the alignment of base. A hint: nothing waits for it.
__device__ __forceinline__ void l2_prefetch(const void* base, size_t b, size_t e) {
    const unsigned long long a = reinterpret_cast<unsigned long long>(base);
    const unsigned long long a0 = (a + b + 15) & ~15ull, a1 = (a + e) & ~15ull;
    if (a1 > a0) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a0), "r"(unsigned(a1 - a0)) : "memory");
}

// N values from a 16-byte aligned record (read-only data)
template <int N>
__device__ __forceinline__ void ldrec(float (&a)[N], const float* p) {
    static_assert(N % 4 == 0, "record of whole float4s");
    const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
    for (int i = 0; i < N / 4; ++i) {
        const float4 t = __ldg(q + i);
        a[4 * i] = t.x; a[4 * i + 1] = t.y; a[4 * i + 2] = t.z; a[4 * i + 3] = t.w;
    }
}
template <int N>
__device__ __forceinline__ void ldrec(double (&a)[N], const double* p) {
    static_assert(N % 2 == 0, "record of whole double2s");
    const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
    for (int i = 0; i < N / 2; ++i) {
        const double2 t = __ldg(q + i);
        a[2 * i] = t.x; a[2 * i + 1] = t.y;
    }
}
template <int N>
__device__ __forceinline__ void ldrec(int (&a)[N], const int* p) {
    static_assert(N % 4 == 0, "record of whole int4s");
    const int4* q = reinterpret_cast<const int4*>(p);
#pragma unroll
    for (int i = 0; i < N / 4; ++i) {
        const int4 t = __ldg(q + i);
        a[4 * i] = t.x; a[4 * i + 1] = t.y; a[4 * i + 2] = t.z; a[4 * i + 3] = t.w;
    }
}
// N values of a row record stored component-major with stride w (the rows of its level): coalesced across the
// threads of consecutive rows
template <class T, int N>
__device__ __forceinline__ void ldrec_cm(T (&a)[N], const T* p, int w) {
#pragma unroll
    for (int i = 0; i < N; ++i) a[i] = __ldg(p + size_t(i) * size_t(w));
}
__device__ __forceinline__ int slot_col(const int4& c, int j) { return j == 0 ? c.x : (j == 1 ? c.y : c.z); }

// ------------------------------------------------------------------ BILU0 sweeps on slot records
template <class TF>
struct IluArgs {
    const int *sysRow0, *sysLvl0, *lvlStart;
    const int4 *Lslot, *Uslot;
    const int *LovCol, *UovCol;
    const TF *L, *UD, *Lov, *Uov;
};

// Registers of one row: slot columns, factor record, input (TI: the sweep input's storage type)
template <class TF, class TI, int MODE>
struct FwdRow {
    int k;
    int4 c;
    TF a[LREC];
    TI in[MODE == IN_PUPDATE ? 9 : (MODE == IN_SUPDATE ? 6 : 3)];
};
template <class TF>
struct BwdRow {
    int k;
    int4 c;
    TF a[UREC];
    double xp;
};

// row k of the level [ls, ls + lw) (component-major records)
template <class TF, class TI, int MODE>
__device__ __forceinline__ void load_fwd(FwdRow<TF, TI, MODE>& R, int k, int ls, int lw, const IluArgs<TF>& F, const TI* r,
                                         const double* pv, const double* v) {
    R.k = k;
    if (k < 0) return;
    R.c = __ldg(F.Lslot + k);
    ldrec_cm(R.a, F.L + size_t(ls) * LREC + size_t(k - ls), lw);
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const size_t q = size_t(k) * 3 + e;
        R.in[e] = r[q];
        if (MODE == IN_PUPDATE) { R.in[3 + e] = pv[q]; R.in[6 + e] = v[q]; }
        if (MODE == IN_SUPDATE) R.in[3 + e] = v[q];
    }
}
template <class TF, class TX>
__device__ __forceinline__ void load_bwd(BwdRow<TF>& R, int k, int ls, int lw, const IluArgs<TF>& F, const TX* xp, int row0) {
    R.k = k;
    if (k < 0) return;
    R.c = __ldg(F.Uslot + k);
    ldrec_cm(R.a, F.UD + size_t(ls) * UREC + size_t(k - ls), lw);
    if (xp) R.xp = double(xp[k - row0]);
}

template <class TF, class TV>
__device__ __forceinline__ void sub_block(TV (&yi)[3], const TF* a, const TV* y, int c) {
    const TV yc[3] = {y[c * 3 + 0], y[c * 3 + 1], y[c * 3 + 2]};
    yi[0] = vsub(yi[0], rdot(a, yc));
    yi[1] = vsub(yi[1], rdot(a + 3, yc));
    yi[2] = vsub(yi[2], rdot(a + 6, yc));
}

// yi -= sum over the overflow list from position q (columns oc, blocks ov) in list order. The entries come in
// chunks of OV_CHUNK whose columns and blocks are all loaded before the first is used: a row with many
// couplings (a well cell) costs one memory latency per chunk, not two per entry. Entries past a row's
// terminator are read but not used (the lists are padded so that they exist).
template <class TF, class TV>
__device__ __forceinline__ void ov_sub(TV (&yi)[3], const int* __restrict__ oc, const TF* __restrict__ ov, int q, const TV* y) {
    for (;; q += OV_CHUNK) {
        int c[OV_CHUNK];
        TF a[OV_CHUNK][9];
#pragma unroll
        for (int u = 0; u < OV_CHUNK; ++u) c[u] = __ldg(oc + q + u);
#pragma unroll
        for (int u = 0; u < OV_CHUNK; ++u)
#pragma unroll
            for (int e = 0; e < 9; ++e) a[u][e] = __ldg(ov + size_t(q + u) * 9 + e);
#pragma unroll
        for (int u = 0; u < OV_CHUNK; ++u) {
            if (c[u] < 0) return;
            sub_block(yi, a[u], y, c[u]);
        }
    }
}

// y_i = in_i - sum_{k<i} L_ik y_k (engine/src/bsr.cpp:568-575): slots, then the overflow list, in row order
template <class TF, class TV, class TI, int MODE>
__device__ __forceinline__ void fwd_step(const FwdRow<TF, TI, MODE>& R, const IluArgs<TF>& F, int row0, TV* y, double* pv, double beta,
                                         double omega, double alpha) {
    const int k = R.k;
    TV yi[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const size_t q = size_t(k) * 3 + e;
        if (MODE == IN_PUPDATE) {
            const double pe = da(R.in[e], dm(beta, ds(R.in[3 + e], dm(omega, R.in[6 + e]))));   // linsolve.cpp:173
            pv[q] = pe;
            yi[e] = TV(pe);
        } else if (MODE == IN_SUPDATE) {
            const double se = ds(R.in[e], dm(alpha, R.in[3 + e]));                              // linsolve.cpp:183
            pv[q] = se;
            yi[e] = TV(se);
        } else {
            yi[e] = TV(R.in[e]);
        }
    }
#pragma unroll
    for (int j = 0; j < SLOTS; ++j) {
        const int c = slot_col(R.c, j);
        if (c >= 0) sub_block(yi, R.a + 9 * j, y, c);
    }
    if (R.c.w >= 0) ov_sub(yi, F.LovCol, F.Lov, R.c.w, y);
    const int li = k - row0;
    y[li * 3 + 0] = yi[0]; y[li * 3 + 1] = yi[1]; y[li * 3 + 2] = yi[2];
}

// z_i = U_ii^-1 (y_i - sum_{j>i} U_ij z_j) (engine/src/bsr.cpp:577-587); with XP the CPR correction z_p += xp
// (bsr.cpp:1083) is applied to the stored z
template <class TF, class TV, bool XP>
__device__ __forceinline__ void bwd_step(const BwdRow<TF>& R, const IluArgs<TF>& F, int row0, TV* y, double* z, bool writeZ) {
    const int k = R.k, li = k - row0;
    TV yi[3] = {y[li * 3 + 0], y[li * 3 + 1], y[li * 3 + 2]};
#pragma unroll
    for (int j = 0; j < SLOTS; ++j) {
        const int c = slot_col(R.c, j);
        if (c >= 0) sub_block(yi, R.a + 9 * j, y, c);
    }
    if (R.c.w >= 0) ov_sub(yi, F.UovCol, F.Uov, R.c.w, y);
    const TF* d = R.a + 9 * SLOTS;
    const TV t0 = rdot(d, yi), t1 = rdot(d + 3, yi), t2 = rdot(d + 6, yi);
    y[li * 3 + 0] = t0; y[li * 3 + 1] = t1; y[li * 3 + 2] = t2;
    if (writeZ) {
        z[size_t(k) * 3 + 0] = XP ? da(double(t0), R.xp) : double(t0);
        z[size_t(k) * 3 + 1] = double(t1);
        z[size_t(k) * 3 + 2] = double(t2);
    }
}

template <class TF, class TI, int MODE>
__device__ __forceinline__ void prefetch_fwd_level(const IluArgs<TF>& F, const int* lv, int L, const TI* r, const double* pv,
                                                   const double* v) {
    const size_t s = size_t(lv[L]), e = size_t(lv[L + 1]);
    l2_prefetch(F.L, s * LREC * sizeof(TF), e * LREC * sizeof(TF));
    l2_prefetch(F.Lslot, s * sizeof(int4), e * sizeof(int4));
    l2_prefetch(r, s * 3 * sizeof(TI), e * 3 * sizeof(TI));
    if (MODE == IN_PUPDATE) l2_prefetch(pv, s * 24, e * 24);
    if (MODE != IN_PLAIN) l2_prefetch(v, s * 24, e * 24);
}
template <class TF>
__device__ __forceinline__ void prefetch_bwd_level(const IluArgs<TF>& F, const int* lv, int L) {
    const size_t s = size_t(lv[L]), e = size_t(lv[L + 1]);
    l2_prefetch(F.UD, s * UREC * sizeof(TF), e * UREC * sizeof(TF));
    l2_prefetch(F.Uslot, s * sizeof(int4), e * sizeof(int4));
}

// The level loops below run levels in pairs with fixed register roles (cur, nxt) = (A, B) then (B, A): a level
// works on the rows in cur while the same threads' rows of the next level load into nxt, so every row's loads
// are in flight for a whole level. NSET row sets cover levels of up to NSET x blockDim rows this way; further
// rows of a level load when they are reached.
template <int NSET>
__device__ __forceinline__ int row_of(int s, int e, int j) {
    const int k = s + int(threadIdx.x) + j * int(blockDim.x);
    return k < e ? k : -1;
}

template <class TF, class TV, class TI, int MODE, int NSET>
__device__ __forceinline__ void fwd_level(const IluArgs<TF>& F, const int* lv, int L, int nl, FwdRow<TF, TI, MODE>* cur,
                                          FwdRow<TF, TI, MODE>* nxt, int row0, const TI* r, double* pv, const double* v, TV* y,
                                          double beta, double omega, double alpha) {
    const int s = lv[L], e = lv[L + 1];
    if (threadIdx.x == 0 && L + kAhead < nl) prefetch_fwd_level<TF, TI, MODE>(F, lv, L + kAhead, r, pv, v);
    if (L + 1 < nl) {
        const int e1 = lv[L + 2];
#pragma unroll
        for (int j = 0; j < NSET; ++j) load_fwd(nxt[j], row_of<NSET>(e, e1, j), e, e1 - e, F, r, pv, v);
    }
#pragma unroll
    for (int j = 0; j < NSET; ++j) {
        const int k = row_of<NSET>(s, e, j);
        if (k >= 0) {
            if (cur[j].k != k) load_fwd(cur[j], k, s, e - s, F, r, pv, v);
            fwd_step<TF, TV, TI, MODE>(cur[j], F, row0, y, pv, beta, omega, alpha);
        }
    }
    for (int k = s + int(threadIdx.x) + NSET * int(blockDim.x); k < e; k += blockDim.x) {
        load_fwd(cur[0], k, s, e - s, F, r, pv, v);
        fwd_step<TF, TV, TI, MODE>(cur[0], F, row0, y, pv, beta, omega, alpha);
    }
    __syncthreads();
}

template <class TF, class TV, bool XP, int NSET, class TX>
__device__ __forceinline__ void bwd_level(const IluArgs<TF>& F, const int* lv, int L, BwdRow<TF>* cur, BwdRow<TF>* nxt, int row0,
                                          const TX* xp, TV* y, double* z, bool writeZ) {
    const int s = lv[L], e = lv[L + 1];
    if (threadIdx.x == 0 && L - kAhead >= 0) prefetch_bwd_level(F, lv, L - kAhead);
    if (L > 0) {
        const int s1 = lv[L - 1];
#pragma unroll
        for (int j = 0; j < NSET; ++j) load_bwd(nxt[j], row_of<NSET>(s1, s, j), s1, s - s1, F, xp, row0);
    }
#pragma unroll
    for (int j = 0; j < NSET; ++j) {
        const int k = row_of<NSET>(s, e, j);
        if (k >= 0) {
            if (cur[j].k != k) load_bwd(cur[j], k, s, e - s, F, xp, row0);
            bwd_step<TF, TV, XP>(cur[j], F, row0, y, z, writeZ);
        }
    }
    for (int k = s + int(threadIdx.x) + NSET * int(blockDim.x); k < e; k += blockDim.x) {
        load_bwd(cur[0], k, s, e - s, F, xp, row0);
        bwd_step<TF, TV, XP>(cur[0], F, row0, y, z, writeZ);
    }
    __syncthreads();
}

// The level starts of a system are read at every level step by every thread. The streaming factor records keep the
// small L1 of these kernels (most of the SM's memory is shared memory) from holding them, so each step would
// begin with an L2 round trip: a block copies them to shared memory when they fit.
constexpr int kLvCache = 512;
constexpr size_t kCtaStaticSmem = 4096;    // static shared memory of the sweep kernels (level starts), off the dynamic cap
__device__ __forceinline__ const int* level_starts(const int* g, int nl, int* cache) {
    if (nl + 1 > kLvCache) return g;
    for (int i = int(threadIdx.x); i <= nl; i += int(blockDim.x)) cache[i] = __ldg(g + i);
    __syncthreads();
    return cache;
}

// Both sweeps of one system by the calling thread block (y: the sweep vector of this system, on chip or in z;
// xp: with XP, the CPR pressure correction added to z_p as z is written)
template <class TF, class TV, class TI, int MODE, bool XP, class TX, int NT>
__device__ void ilu_body(const IluArgs<TF>& F, int row0, const int* lv, int nl, const TI* r, double* pv, const double* v, double* z, TV* y,
                         bool writeZ, double beta, double omega, double alpha, const TX* xp) {
    constexpr int NSET = (NT < 512 && sizeof(TF) == 4 && MODE == IN_PLAIN) ? 2 : 1;
    if (threadIdx.x == 0)
        for (int L = 0; L < kAhead && L < nl; ++L) prefetch_fwd_level<TF, TI, MODE>(F, lv, L, r, pv, v);
    {
        FwdRow<TF, TI, MODE> A[NSET], B[NSET];
        if (nl > 0) {
            const int s = lv[0], e = lv[1];
#pragma unroll
            for (int j = 0; j < NSET; ++j) load_fwd(A[j], row_of<NSET>(s, e, j), s, e - s, F, r, pv, v);
        }
        for (int L = 0; L < nl; L += 2) {
            fwd_level<TF, TV, TI, MODE, NSET>(F, lv, L, nl, A, B, row0, r, pv, v, y, beta, omega, alpha);
            if (L + 1 < nl) fwd_level<TF, TV, TI, MODE, NSET>(F, lv, L + 1, nl, B, A, row0, r, pv, v, y, beta, omega, alpha);
        }
    }
    if (threadIdx.x == 0)
        for (int L = nl - 1; L >= 0 && L >= nl - kAhead; --L) prefetch_bwd_level(F, lv, L);
    {
        const TX* xq = XP ? xp : nullptr;
        BwdRow<TF> A[NSET], B[NSET];
        if (nl > 0) {
            const int s = lv[nl - 1], e = lv[nl];
#pragma unroll
            for (int j = 0; j < NSET; ++j) load_bwd(A[j], row_of<NSET>(s, e, j), s, e - s, F, xq, row0);
        }
        for (int L = nl - 1; L >= 0; L -= 2) {
            bwd_level<TF, TV, XP, NSET>(F, lv, L, A, B, row0, xq, y, z, writeZ);
            if (L - 1 >= 0) bwd_level<TF, TV, XP, NSET>(F, lv, L - 1, B, A, row0, xq, y, z, writeZ);
        }
    }
}

// The same sweeps with three register buffers and one row per thread per buffer: a level's rows are loaded two
// levels ahead (at the start of level L, the rows of level L + 2), so a load has two level steps to arrive. Rows past
// blockDim in a level load when they are reached. For FP32 factor records (three FP64 records do not fit the
// registers of a 256-thread block).
template <class TF, class TV, class TI, bool XP, class TX>
__device__ void ilu_body3(const IluArgs<TF>& F, int row0, const int* lv, int nl, const TI* r, double* z, TV* y, bool writeZ, const TX* xp) {
    const int nt = int(blockDim.x);
    if (threadIdx.x == 0)
        for (int L = 0; L < kAhead && L < nl; ++L) prefetch_fwd_level<TF, TI, IN_PLAIN>(F, lv, L, r, nullptr, nullptr);
    {
        FwdRow<TF, TI, IN_PLAIN> R[3];
#pragma unroll
        for (int b = 0; b < 2; ++b)
            if (b < nl) load_fwd(R[b], row_of<1>(lv[b], lv[b + 1], 0), lv[b], lv[b + 1] - lv[b], F, r, nullptr, nullptr);
        for (int L0 = 0; L0 < nl; L0 += 3) {
#pragma unroll
            for (int b = 0; b < 3; ++b) {                    // level L0 + b works on R[b], loads level + 2 into R[(b + 2) % 3]
                const int L = L0 + b;
                if (L >= nl) break;
                const int s = lv[L], e = lv[L + 1];
                if (threadIdx.x == 0 && L + kAhead < nl) prefetch_fwd_level<TF, TI, IN_PLAIN>(F, lv, L + kAhead, r, nullptr, nullptr);
                if (L + 2 < nl) load_fwd(R[(b + 2) % 3], row_of<1>(lv[L + 2], lv[L + 3], 0), lv[L + 2], lv[L + 3] - lv[L + 2], F, r, nullptr, nullptr);
                const int k = row_of<1>(s, e, 0);
                if (k >= 0) {
                    if (R[b].k != k) load_fwd(R[b], k, s, e - s, F, r, nullptr, nullptr);
                    fwd_step<TF, TV, TI, IN_PLAIN>(R[b], F, row0, y, nullptr, 0, 0, 0);
                }
                for (int k2 = s + int(threadIdx.x) + nt; k2 < e; k2 += nt) {
                    load_fwd(R[b], k2, s, e - s, F, r, nullptr, nullptr);
                    fwd_step<TF, TV, TI, IN_PLAIN>(R[b], F, row0, y, nullptr, 0, 0, 0);
                }
                __syncthreads();
            }
        }
    }
    if (threadIdx.x == 0)
        for (int L = nl - 1; L >= 0 && L >= nl - kAhead; --L) prefetch_bwd_level(F, lv, L);
    {
        const TX* xq = XP ? xp : nullptr;
        BwdRow<TF> R[3];
#pragma unroll
        for (int b = 0; b < 2; ++b)
            if (b < nl) load_bwd(R[b], row_of<1>(lv[nl - 1 - b], lv[nl - b], 0), lv[nl - 1 - b], lv[nl - b] - lv[nl - 1 - b], F, xq, row0);
        for (int g0 = 0; g0 < nl; g0 += 3) {
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                const int g = g0 + b;
                if (g >= nl) break;
                const int L = nl - 1 - g;
                const int s = lv[L], e = lv[L + 1];
                if (threadIdx.x == 0 && L - kAhead >= 0) prefetch_bwd_level(F, lv, L - kAhead);
                if (L - 2 >= 0) load_bwd(R[(b + 2) % 3], row_of<1>(lv[L - 2], lv[L - 1], 0), lv[L - 2], lv[L - 1] - lv[L - 2], F, xq, row0);
                const int k = row_of<1>(s, e, 0);
                if (k >= 0) {
                    if (R[b].k != k) load_bwd(R[b], k, s, e - s, F, xq, row0);
                    bwd_step<TF, TV, XP>(R[b], F, row0, y, z, writeZ);
                }
                for (int k2 = s + int(threadIdx.x) + nt; k2 < e; k2 += nt) {
                    load_bwd(R[b], k2, s, e - s, F, xq, row0);
                    bwd_step<TF, TV, XP>(R[b], F, row0, y, z, writeZ);
                }
                __syncthreads();
            }
        }
    }
}

// ------------------------------------------------------------------ BILU0 sweeps with records staged by cp.async
// A CTA barrier waits for the register loads its threads have in flight, so register lookahead cannot carry a row's
// loads across the level barriers; asynchronous copies into shared memory (cp.async) are not waited for by the
// barrier. Here every thread stages the record of its row of the next level (slot columns, factor record, input or
// the CPR correction) into its own slot of a shared-memory stage while the current level computes, and waits for its
// own copies (cp.async.wait_group) at the start of the next level: a level step no longer waits for its rows' data
// to come in from L2. The stage holds one row per thread (kStageWords words each, component-major over the threads:
// conflict-free); rows past blockDim in a level load directly when they are reached. FP32 records, vector on chip.
constexpr int kStageWords = 4 + UREC + 1;     // slot columns, the larger record (U with the diagonal), input / correction
constexpr int kStageSlots = 256;               // threads with a stage slot; further threads (512-thread blocks) load directly

__device__ __forceinline__ void cpa4(unsigned* dst, const void* src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cpa_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <class TX>
__device__ void ilu_body_async(const IluArgs<float>& F, int row0, const int* lv, int nl, const float* r, double* z, float* y,
                               const TX* xp, unsigned* stage) {
    static_assert(sizeof(TX) == 4, "the CPR correction is staged as one 32-bit word");
    const int t = int(threadIdx.x), nt = int(blockDim.x);
    const int nsl = min(nt, kStageSlots);          // slots: the stage's stride
    const bool slotted = t < nsl;                  // threads past the slots load their rows directly
    unsigned* st = stage + t;
    auto word = [&](int f) { return st[size_t(f) * size_t(nsl)]; };
    // the copies of this thread's row of forward level L / backward level L (none if the level is narrower)
    auto stage_fwd = [&](int L) {
        const int s0 = lv[L], w = lv[L + 1] - s0, k = s0 + t;
        if (slotted && t < w) {
            const int* sl = reinterpret_cast<const int*>(F.Lslot + k);
#pragma unroll
            for (int j = 0; j < 4; ++j) cpa4(st + j * nsl, sl + j);
            const float* rec = F.L + size_t(s0) * LREC + size_t(t);
#pragma unroll
            for (int j = 0; j < LREC; ++j) cpa4(st + (4 + j) * nsl, rec + size_t(j) * size_t(w));
#pragma unroll
            for (int e = 0; e < 3; ++e) cpa4(st + (4 + UREC - 3 + e) * nsl, r + size_t(k) * 3 + e);
        }
        cpa_commit();
    };
    auto stage_bwd = [&](int L) {
        const int s0 = lv[L], w = lv[L + 1] - s0, k = s0 + t;
        if (slotted && t < w) {
            const int* sl = reinterpret_cast<const int*>(F.Uslot + k);
#pragma unroll
            for (int j = 0; j < 4; ++j) cpa4(st + j * nsl, sl + j);
            const float* rec = F.UD + size_t(s0) * UREC + size_t(t);
#pragma unroll
            for (int j = 0; j < UREC; ++j) cpa4(st + (4 + j) * nsl, rec + size_t(j) * size_t(w));
            cpa4(st + (4 + UREC) * nsl, xp + (k - row0));
        }
        cpa_commit();
    };
    // the levels' records are also brought into L2 kAhead levels ahead (one thread), so the staged copies hit L2
    if (t == 0)
        for (int L = 0; L < kAhead && L < nl; ++L) prefetch_fwd_level<float, float, IN_PLAIN>(F, lv, L, r, nullptr, nullptr);
    if (nl > 0) stage_fwd(0);
    for (int L = 0; L < nl; ++L) {
        const int s0 = lv[L], e = lv[L + 1], k = s0 + t;
        if (t == 0) {
            if (L + kAhead < nl) prefetch_fwd_level<float, float, IN_PLAIN>(F, lv, L + kAhead, r, nullptr, nullptr);
            else if (nl - 1 - (L + kAhead - nl) >= 0) prefetch_bwd_level(F, lv, nl - 1 - (L + kAhead - nl));
        }
        cpa_wait_all();
        FwdRow<float, float, IN_PLAIN> R;
        R.k = -1;
        if (k < e && slotted) {
            R.k = k;
            R.c = make_int4(int(word(0)), int(word(1)), int(word(2)), int(word(3)));
#pragma unroll
            for (int j = 0; j < LREC; ++j) R.a[j] = __uint_as_float(word(4 + j));
#pragma unroll
            for (int q = 0; q < 3; ++q) R.in[q] = __uint_as_float(word(4 + UREC - 3 + q));
        } else if (k < e) {
            load_fwd(R, k, s0, e - s0, F, r, nullptr, nullptr);
        }
        if (L + 1 < nl) stage_fwd(L + 1);       // this thread's slot is free again: its values are in registers
        else stage_bwd(nl - 1);                  // the first backward level comes in during the last forward one
        if (k < e) fwd_step<float, float, float, IN_PLAIN>(R, F, row0, y, nullptr, 0, 0, 0);
        for (int k2 = k + nt; k2 < e; k2 += nt) {
            load_fwd(R, k2, s0, e - s0, F, r, nullptr, nullptr);
            fwd_step<float, float, float, IN_PLAIN>(R, F, row0, y, nullptr, 0, 0, 0);
        }
        __syncthreads();
    }
    for (int g = 0; g < nl; ++g) {
        const int L = nl - 1 - g;
        const int s0 = lv[L], e = lv[L + 1], k = s0 + t;
        if (t == 0 && L - kAhead >= 0) prefetch_bwd_level(F, lv, L - kAhead);
        cpa_wait_all();
        BwdRow<float> R;
        R.k = -1;
        if (k < e && slotted) {
            R.k = k;
            R.c = make_int4(int(word(0)), int(word(1)), int(word(2)), int(word(3)));
#pragma unroll
            for (int j = 0; j < UREC; ++j) R.a[j] = __uint_as_float(word(4 + j));
            R.xp = double(__uint_as_float(word(4 + UREC)));
        } else if (k < e) {
            load_bwd(R, k, s0, e - s0, F, xp, row0);
        }
        if (L > 0) stage_bwd(L - 1);
        if (k < e) bwd_step<float, float, true>(R, F, row0, y, z, true);
        for (int k2 = k + nt; k2 < e; k2 += nt) {
            load_bwd(R, k2, s0, e - s0, F, xp, row0);
            bwd_step<float, float, true>(R, F, row0, y, z, true);
        }
        __syncthreads();
    }
}

template <class TF, class TV, int MODE, int NT = cta_threads<TF, TV>()>
__global__ void __launch_bounds__(NT) k_ilu_cta(IluArgs<TF> F, const double* r, double* pv, const double* v, double* z,
                                                        TV* yglob, size_t smemBytes, const KScal* ks) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int s = blockIdx.x;
    const int row0 = __ldg(F.sysRow0 + s), ns = __ldg(F.sysRow0 + s + 1) - row0;
    double beta = 0, omega = 0, alpha = 0;
    if (ks) {
        const KScal& K = ks[s];
        if (K.status != ST_RUNNING) return;                // whole block: uniform
        beta = K.beta; omega = K.omega; alpha = K.alpha;
    }
    // sweep vector: on chip when it fits, else global (yglob: z itself for TV = double)
    const bool onchip = size_t(ns) * 3 * sizeof(TV) <= smemBytes;
    TV* y = onchip ? reinterpret_cast<TV*>(smraw) : yglob + size_t(row0) * 3;
    const int l0 = __ldg(F.sysLvl0 + s), nl = __ldg(F.sysLvl0 + s + 1) - l0 - 1;
    __shared__ int lvc[kLvCache];
    const int* lv = level_starts(F.lvlStart + l0, nl, lvc);
    ilu_body<TF, TV, double, MODE, false, double, NT>(F, row0, lv, nl, r, pv, v, z, y, onchip || sizeof(TV) != sizeof(double), beta, omega,
                                                  alpha, nullptr);
}

// ------------------------------------------------------------------ CPR (BlockCPR::apply, engine/src/bsr.cpp:1061-1084)
template <class TA>
struct CprArgs {
    const AmgSysLv* lv;
    int maxL;
    const int* lvl;                   // GS schedule boundaries of every (system, level): forward levels or colours
    const int* gsRows;                // rows in schedule order
    const int* ci;                    // level CSR columns / values (entries beyond the row slots)
    const TA* val;
    const int* slotCol;
    const TA* slotVal;
    const TA* diagVal;
    const int4* rowMeta;
    const int *agg, *memPtr, *mem;
    const TA* lu;                     // coarsest dense LU
    const float* inv;                 // FP32 forms: coarsest explicit inverse (columns, natural row order)
    const int *luPerm, *cin;
    TA *x, *b, *r;                    // V-cycle vectors in global memory (levels that do not fit on chip)
    const double* w;
    double* T;
    const TA *sp, *spLov, *spUov;     // pressure columns of S in slot order
    const int* coarse64;              // FP32 forms: per system, coarsest level solved in FP64 with the LU below
    const double* lu64;
    double *x64, *b64, *r64;          // FP64 vectors of that solve (every level's rows; only the coarsest used)
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

// one row of an AMG level in registers: W slot values / columns, diagonal, {entries before the diagonal,
// off-diagonal entries, continuation position, diagonal position}
template <class TA, int W>
struct GsRow {
    int k;
    int4 m;
    TA v[W];
    int c[W];
    TA d;
};
template <class TA, int W>
__device__ __forceinline__ void load_gs(GsRow<TA, W>& R, int k, const AmgSysLv& A, const CprArgs<TA>& C) {
    R.k = k;
    if (k < 0) return;
    R.m = __ldg(C.rowMeta + A.rowOff + k);
    ldrec(R.v, C.slotVal + size_t(A.slotOff) + size_t(k) * W);
    ldrec(R.c, C.slotCol + size_t(A.slotOff) + size_t(k) * W);
    R.d = __ldg(C.diagVal + A.rowOff + k);
}
// Gauss-Seidel update of row k (engine/src/amg.cpp:98-113): s = b_k - sum_{p != diag} a_p x_col(p), in row order;
// from x = 0 only the entries before the diagonal (the others multiply zeros)
template <class TA, int W>
__device__ __forceinline__ void gs_step(const GsRow<TA, W>& R, const AmgSysLv& A, const CprArgs<TA>& C, TA* x, const TA* b, bool fromZero) {
    TA s = b[R.k];
    const int lim = fromZero ? R.m.x : R.m.y;
#pragma unroll
    for (int j = 0; j < W; ++j)
        if (j < lim) s = asub(s, amul(R.v[j], x[R.c[j]]));
    if (lim > W) {                    // entries after the slots, in chunks as ov_sub (the arrays are padded)
        const int* ci = C.ci + A.entOff;
        const TA* val = C.val + A.entOff;
        int jo = W;
        for (int p = R.m.z; jo < lim; p += OV_CHUNK) {
            int c[OV_CHUNK];
            TA a[OV_CHUNK];
#pragma unroll
            for (int u = 0; u < OV_CHUNK; ++u) { c[u] = __ldg(ci + p + u); a[u] = val[p + u]; }
#pragma unroll
            for (int u = 0; u < OV_CHUNK; ++u)
                if (jo < lim && p + u != R.m.w) {
                    s = asub(s, amul(a[u], x[c[u]]));
                    ++jo;
                }
        }
    }
    x[R.k] = adiv(s, R.d);
}

template <class TA, int W>
__device__ __forceinline__ void prefetch_gs_level(const AmgSysLv& A, const CprArgs<TA>& C, const int* lv, int L, const TA* bg) {
    const size_t s = size_t(__ldg(lv + L)), e = size_t(__ldg(lv + L + 1));
    l2_prefetch(C.slotVal + A.slotOff, s * W * sizeof(TA), e * W * sizeof(TA));
    l2_prefetch(C.slotCol + A.slotOff, s * W * sizeof(int), e * W * sizeof(int));
    l2_prefetch(C.rowMeta + A.rowOff, s * sizeof(int4), e * sizeof(int4));
    if (bg) l2_prefetch(bg, s * sizeof(TA), e * sizeof(TA));
}

// row of schedule position pos (-1 stays -1): the colour order for colours; forward levels are the identity (no
// lookup: it would add a dependent load to every level step)
__device__ __forceinline__ int sched_row(const int* __restrict__ rw, int pos, bool mc) { return pos >= 0 && mc ? __ldg(rw + pos) : pos; }

template <class TA, int W, int NSET>
__device__ __forceinline__ void gs_level(const AmgSysLv& A, const CprArgs<TA>& C, const int* lv, const int* rw, int L, int Lnext, int g,
                                         int dir, GsRow<TA, W>* cur, GsRow<TA, W>* nxt, TA* x, const TA* b, const TA* bg, bool fromZero) {
    const int s = __ldg(lv + L), e = __ldg(lv + L + 1);
    if (threadIdx.x == 0 && !A.mc && g + kAhead < A.nl) prefetch_gs_level<TA, W>(A, C, lv, L + dir * kAhead, bg);
    if (Lnext >= 0 && Lnext < A.nl) {
        const int s1 = __ldg(lv + Lnext), e1 = __ldg(lv + Lnext + 1);
#pragma unroll
        for (int j = 0; j < NSET; ++j) load_gs(nxt[j], sched_row(rw, row_of<NSET>(s1, e1, j), A.mc), A, C);
    }
#pragma unroll
    for (int j = 0; j < NSET; ++j) {
        const int k = sched_row(rw, row_of<NSET>(s, e, j), A.mc);
        if (k >= 0) {
            if (cur[j].k != k) load_gs(cur[j], k, A, C);
            gs_step(cur[j], A, C, x, b, fromZero);
        }
    }
    for (int pos = s + int(threadIdx.x) + NSET * int(blockDim.x); pos < e; pos += blockDim.x) {
        load_gs(cur[0], sched_row(rw, pos, A.mc), A, C);
        gs_step(cur[0], A, C, x, b, fromZero);
    }
    __syncthreads();
}

// Rows a thread takes at once in the parallel passes: their loads are all issued before any is used, so a batch
// costs about one memory latency (about a microsecond under this load) instead of one per row.
template <class TA, int W>
__host__ __device__ constexpr int row_batch() { return sizeof(TA) == 8 ? 1 : (W <= 8 ? 4 : 2); }   // FP64: registers

// One colour of the multicolour sweep: a colour's rows are independent; every thread takes its rows in batches.
template <class TA, int W>
__device__ __forceinline__ void gs_colour(const AmgSysLv& A, const CprArgs<TA>& C, const int* __restrict__ rw, int s, int e, TA* x,
                                          const TA* b) {
    constexpr int RB = row_batch<TA, W>();
    const int nt = int(blockDim.x);
    for (int base = s + int(threadIdx.x); base < e; base += RB * nt) {
        // named row buffers (an array of row structs would live in local memory)
        const int k0 = __ldg(rw + base), k1 = RB > 1 && base + nt < e ? __ldg(rw + base + nt) : -1;
        int k2 = -1, k3 = -1;
        if (RB > 2) {
            k2 = base + 2 * nt < e ? __ldg(rw + base + 2 * nt) : -1;
            k3 = base + 3 * nt < e ? __ldg(rw + base + 3 * nt) : -1;
        }
        GsRow<TA, W> R0, R1, R2, R3;
        load_gs(R0, k0, A, C);
        if (RB > 1) load_gs(R1, k1, A, C);
        if (RB > 2) { load_gs(R2, k2, A, C); load_gs(R3, k3, A, C); }
        gs_step(R0, A, C, x, b, false);
        if (RB > 1 && k1 >= 0) gs_step(R1, A, C, x, b, false);
        if (RB > 2) {
            if (k2 >= 0) gs_step(R2, A, C, x, b, false);
            if (k3 >= 0) gs_step(R3, A, C, x, b, false);
        }
    }
    __syncthreads();
}

// one Gauss-Seidel sweep of a level over its GS levels (forward, or backward for the post-smoothing: valid on the
// structurally symmetric levels), rows of one GS level in parallel; levels in pairs as the BILU0 sweeps
template <class TA, int W, int NT>
__device__ __forceinline__ void gs_sweep_body(const AmgSysLv& A, const CprArgs<TA>& C, TA* x, const TA* b, bool bGlobal, bool forward,
                                              bool fromZero) {
    constexpr int NSET = NT >= 512 ? 1 : ((sizeof(TA) == 4 || W == AMG_W0) ? 2 : 1);
    const int* lv = C.lvl + A.lvlOff;
    const int* rw = C.gsRows + A.rowOff;
    const int nl = A.nl, dir = forward ? 1 : -1;
    const TA* bg = bGlobal ? b : nullptr;
    const int Lfirst = forward ? 0 : nl - 1;
    if constexpr (sizeof(TA) == 4) {                  // the multicolour schedule exists only in the FP32 forms
        if (A.mc) {                                   // colours: each a batched pass over independent rows
            if (threadIdx.x == 0) {                   // a colour gathers rows from the whole level: prefetch it once
                l2_prefetch(C.slotVal + A.slotOff, 0, size_t(A.n) * W * sizeof(TA));
                l2_prefetch(C.slotCol + A.slotOff, 0, size_t(A.n) * W * sizeof(int));
                l2_prefetch(C.rowMeta + A.rowOff, 0, size_t(A.n) * sizeof(int4));
            }
            for (int g = 0; g < nl; ++g) {
                const int L = Lfirst + dir * g;
                gs_colour<TA, W>(A, C, rw, __ldg(lv + L), __ldg(lv + L + 1), x, b);
            }
            return;
        }
    }
    if (threadIdx.x == 0)
        for (int g = 0; g < kAhead && g < nl; ++g) prefetch_gs_level<TA, W>(A, C, lv, Lfirst + dir * g, bg);
    GsRow<TA, W> P[NSET], Q[NSET];
    if (nl > 0) {
        const int s = __ldg(lv + Lfirst), e = __ldg(lv + Lfirst + 1);
#pragma unroll
        for (int j = 0; j < NSET; ++j) load_gs(P[j], sched_row(rw, row_of<NSET>(s, e, j), A.mc), A, C);
    }
    for (int g = 0; g < nl; g += 2) {
        const int L = Lfirst + dir * g;
        gs_level<TA, W, NSET>(A, C, lv, rw, L, L + dir, g, dir, P, Q, x, b, bg, fromZero);
        if (g + 1 < nl) gs_level<TA, W, NSET>(A, C, lv, rw, L + dir, L + 2 * dir, g + 1, dir, Q, P, x, b, bg, fromZero);
    }
}

// r = b - A x (engine/src/amg.cpp:321-322: the row sum from zero in entry order, diagonal at its place)
template <class TA, int W>
__device__ __forceinline__ void residual_row(const GsRow<TA, W>& R, const AmgSysLv& A, const CprArgs<TA>& C, const TA* x, const TA* b,
                                             TA* r) {
    {
        const int k = R.k;
        const int nlow = R.m.x, noff = R.m.y;
        TA t = TA(0);
#pragma unroll
        for (int j = 0; j < W; ++j) {
            if (j == nlow) t = aadd(t, amul(R.d, x[k]));
            if (j < noff) t = aadd(t, amul(R.v[j], x[R.c[j]]));
        }
        // entries after the slots (the diagonal among them when it comes after W off-diagonal entries)
        int rem = noff + 1 - (noff < W ? noff : W) - (nlow < W ? 1 : 0);
        if (rem > 0) {
            const int* ci = C.ci + A.entOff;
            const TA* val = C.val + A.entOff;
            for (int p = R.m.z; rem > 0; ++p, --rem) t = aadd(t, amul(val[p], x[__ldg(ci + p)]));
        }
        r[k] = asub(b[k], t);
    }
}
template <class TA, int W>
__device__ __forceinline__ void residual_body(const AmgSysLv& A, const CprArgs<TA>& C, const TA* x, const TA* b, TA* r) {
    constexpr int RB = row_batch<TA, W>();
    const int nt = int(blockDim.x);
    for (int base = threadIdx.x; base < A.n; base += RB * nt) {
        GsRow<TA, W> R0, R1, R2, R3;                           // named row buffers (see gs_colour)
        load_gs(R0, base, A, C);
        if (RB > 1) load_gs(R1, base + nt < A.n ? base + nt : -1, A, C);
        if (RB > 2) {
            load_gs(R2, base + 2 * nt < A.n ? base + 2 * nt : -1, A, C);
            load_gs(R3, base + 3 * nt < A.n ? base + 3 * nt : -1, A, C);
        }
        residual_row(R0, A, C, x, b, r);
        if (RB > 1 && R1.k >= 0) residual_row(R1, A, C, x, b, r);
        if (RB > 2) {
            if (R2.k >= 0) residual_row(R2, A, C, x, b, r);
            if (R3.k >= 0) residual_row(R3, A, C, x, b, r);
        }
    }
}

// coarsest level: x = LU^-1 b with the dense LU of the natural numbering (engine/src/amg.cpp:306-312). 32-column
// panels: warp 0 solves the panel's triangle with shuffles, then every thread updates its rows below (forward)
// or above (backward) with the panel. The forward substitution subtracts every row's terms in ascending column
// order, as the reference; the backward one takes the panels last to first (rounding-level differences).
template <class TA>
__device__ __forceinline__ void coarse_dense_body(const AmgSysLv& A, const CprArgs<TA>& C, TA* x, const TA* b, TA* work) {
    const int m = A.n, tid = int(threadIdx.x), nt = int(blockDim.x), lane = tid & 31;
    const TA* lu = C.lu + A.luOff;
    const int* nat = C.luPerm + A.luRowOff;
    const int* cin = C.cin + A.luRowOff;
    for (int i = tid; i < m; i += nt) work[i] = b[__ldg(cin + i)];
    __syncthreads();
    for (int j0 = 0; j0 < m; j0 += 32) {
        const int jb = min(32, m - j0);
        if (tid < 32) {
            const int i = j0 + lane;
            TA a[32];
#pragma unroll
            for (int jj = 0; jj < 32; ++jj) a[jj] = (lane < jb && jj < lane) ? __ldg(lu + size_t(i) * m + j0 + jj) : TA(0);
            TA s = lane < jb ? work[i] : TA(0);
#pragma unroll
            for (int jj = 0; jj < 31; ++jj) {
                const TA xj = __shfl_sync(0xffffffffu, s, jj);
                if (jj < lane && lane < jb) s = asub(s, amul(a[jj], xj));
            }
            if (lane < jb) work[i] = s;
        }
        __syncthreads();
        for (int i = j0 + jb + tid; i < m; i += nt) {
            const TA* row = lu + size_t(i) * m + j0;
            TA s = work[i];
#pragma unroll 8
            for (int jj = 0; jj < jb; ++jj) s = asub(s, amul(__ldg(row + jj), work[j0 + jj]));
            work[i] = s;
        }
        __syncthreads();
    }
    for (int j0 = ((m - 1) / 32) * 32; j0 >= 0; j0 -= 32) {
        const int jb = min(32, m - j0);
        if (tid < 32) {
            const int i = j0 + lane;
            TA a[32];
#pragma unroll
            for (int jj = 0; jj < 32; ++jj) a[jj] = (lane < jb && jj > lane && jj < jb) ? __ldg(lu + size_t(i) * m + j0 + jj) : TA(0);
            const TA dg = lane < jb ? __ldg(lu + size_t(i) * m + i) : TA(1);
            TA s = lane < jb ? work[i] : TA(0);
#pragma unroll
            for (int jj = 31; jj >= 0; --jj) {
                if (jj < jb) {
                    if (lane == jj) s = adiv(s, dg);
                    const TA xj = __shfl_sync(0xffffffffu, s, jj);
                    if (lane < jj) s = asub(s, amul(a[jj], xj));
                }
            }
            if (lane < jb) work[i] = s;
        }
        __syncthreads();
        for (int i = tid; i < j0; i += nt) {
            const TA* row = lu + size_t(i) * m + j0;
            TA s = work[i];
#pragma unroll 8
            for (int jj = 0; jj < jb; ++jj) s = asub(s, amul(__ldg(row + jj), work[j0 + jj]));
            work[i] = s;
        }
        __syncthreads();
    }
    for (int k = tid; k < m; k += nt) x[k] = work[__ldg(nat + k)];
    __syncthreads();
}

// The phases above run out of line: inlined into one kernel they would share its register budget (255 at 256
// threads, 128 at 512) and spill heavily.
template <class TA, int W, int NT>
__device__ __noinline__ void gs_sweep_call(const AmgSysLv& A, const CprArgs<TA>& C, TA* x, const TA* b, bool bGlobal, bool forward,
                                           bool fromZero) {
    gs_sweep_body<TA, W, NT>(A, C, x, b, bGlobal, forward, fromZero);
}
template <class TA, int W, int NT>
__device__ __forceinline__ void gs_sweep(const AmgSysLv& A, const CprArgs<TA>& C, TA* x, const TA* b, bool bGlobal, bool forward,
                                         bool fromZero) {
    gs_sweep_call<TA, W, NT>(A, C, x, b, bGlobal, forward, fromZero);
}
template <class TA, int W>
__device__ __noinline__ void residual_call(const AmgSysLv& A, const CprArgs<TA>& C, const TA* x, const TA* b, TA* r) {
    residual_body<TA, W>(A, C, x, b, r);
}
template <class TA, int W, int NT>
__device__ __forceinline__ void residual(const AmgSysLv& A, const CprArgs<TA>& C, const TA* x, const TA* b, TA* r) {
    residual_call<TA, W>(A, C, x, b, r);
}
// FP32 forms: x = A^-1 b with the explicit inverse in the level-space layout inv[j * m + k] = (A^-1)[nat(k)][nat(j)];
// thread k accumulates row k over the columns (consecutive k: consecutive words), many loads in flight
__device__ __noinline__ void coarse_inverse(const AmgSysLv& A, const CprArgs<float>& C, float* x, const float* b) {
    const int m = A.n;
    const float* inv = C.inv + A.luOff;
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        const float* col = inv + k;
        float acc = 0.f;
#pragma unroll 32
        for (int j = 0; j < m; ++j) acc = fmaf(__ldg(col + size_t(j) * m), b[j], acc);
        x[k] = acc;
    }
    __syncthreads();
}
// the same product for the rows [k0, min(k1, m)) only (no block barrier: rows are independent)
__device__ __noinline__ void coarse_inverse_rows(const AmgSysLv& A, const CprArgs<float>& C, float* x, const float* b, int k0, int k1) {
    const int m = A.n;
    const float* inv = C.inv + A.luOff;
    for (int k = k0 + int(threadIdx.x); k < min(k1, m); k += blockDim.x) {
        const float* col = inv + k;
        float acc = 0.f;
#pragma unroll 32
        for (int j = 0; j < m; ++j) acc = fmaf(__ldg(col + size_t(j) * m), b[j], acc);
        x[k] = acc;
    }
}

// FP32 forms, systems flagged at set-up: the coarsest level in FP64 (dense LU, as the FP64 form), from and back to
// the FP32 V-cycle vectors
__device__ __noinline__ void coarse_fp64(const AmgSysLv& A, const CprArgs<float>& C, float* x, const float* b) {
    CprArgs<double> D{};
    D.lu = C.lu64;
    D.luPerm = C.luPerm;
    D.cin = C.cin;
    double* x64 = C.x64 + A.rowOff;
    double* b64 = C.b64 + A.rowOff;
    for (int k = threadIdx.x; k < A.n; k += blockDim.x) b64[k] = double(b[k]);
    __syncthreads();
    coarse_dense_body<double>(A, D, x64, b64, C.r64 + A.rowOff);
    for (int k = threadIdx.x; k < A.n; k += blockDim.x) x[k] = float(x64[k]);
    __syncthreads();
}

template <class TA>
__device__ __noinline__ void coarse_dense_call(const AmgSysLv& A, const CprArgs<TA>& C, TA* x, const TA* b, TA* work) {
    coarse_dense_body<TA>(A, C, x, b, work);
}
template <class TA, int NT>
__device__ __forceinline__ void coarse_dense(const AmgSysLv& A, const CprArgs<TA>& C, TA* x, const TA* b, TA* work) {
    coarse_dense_call<TA>(A, C, x, b, work);
}

// where the V-cycle vectors of system s live: shared memory (x, then b, then r, as far as they fit) or global
template <class TA>
struct VVecs {
    TA *xs, *bs, *rs;                 // on-chip bases (null when global)
    bool bGlobal;
    int loc0 = 0;                     // offset of the first level held on chip (the on-chip vectors start at that level)
    __device__ TA* x(const AmgSysLv& A, const CprArgs<TA>& C) const { return xs ? xs + (A.locOff - loc0) : C.x + A.rowOff; }
    __device__ TA* b(const AmgSysLv& A, const CprArgs<TA>& C) const { return bs ? bs + (A.locOff - loc0) : C.b + A.rowOff; }
    __device__ TA* r(const AmgSysLv& A, const CprArgs<TA>& C) const { return rs ? rs + (A.locOff - loc0) : C.r + A.rowOff; }
};

template <class TA, int W, int NT>
__device__ void gs_sweep_w(const AmgSysLv& A, const CprArgs<TA>& C, const VVecs<TA>& V, bool forward, bool fromZero) {
    gs_sweep<TA, W, NT>(A, C, V.x(A, C), V.b(A, C), V.bGlobal, forward, fromZero);
}
template <class TA, int NT>
__device__ void gs_any(const AmgSysLv& A, const CprArgs<TA>& C, const VVecs<TA>& V, bool forward, bool fromZero) {
    if (A.W == AMG_W0) gs_sweep_w<TA, AMG_W0, NT>(A, C, V, forward, fromZero);
    else gs_sweep_w<TA, AMG_W1, NT>(A, C, V, forward, fromZero);
}

// AMG::cycle (engine/src/amg.cpp:303-329) for system s from level lstart down and back (lstart 0: the whole V-cycle,
// level-0 right-hand side already in place; lstart 1: the coarse part under a level 0 smoothed by the grid passes,
// level-1 right-hand side in place, level-1 solution left for the grid prolongation)
template <class TA, int NT>
__device__ __forceinline__ void vcycle_body(int s, const CprArgs<TA>& C, const VVecs<TA>& V, int lstart) {
    int nlev = 0;
    while (nlev < C.maxL && C.lv[s * C.maxL + nlev].n > 0) ++nlev;
    if (lstart >= nlev) lstart = nlev > 0 ? nlev - 1 : 0;   // a system whose level 0 is its coarsest
    int l = lstart;
    for (; l < nlev; ++l) {
        const AmgSysLv A = C.lv[s * C.maxL + l];
        if (A.coarse) {
            if (A.dense) {
                if constexpr (sizeof(TA) == 4) {
                    if (C.coarse64[s]) coarse_fp64(A, C, V.x(A, C), V.b(A, C));
                    else coarse_inverse(A, C, V.x(A, C), V.b(A, C));
                } else {
                    coarse_dense<TA, NT>(A, C, V.x(A, C), V.b(A, C), V.r(A, C));
                }
            } else {                                      // 20 symmetric GS sweeps from x = 0 (amg.cpp:313-315)
                TA* xl = V.x(A, C);
                for (int k = threadIdx.x; k < A.n; k += blockDim.x) xl[k] = TA(0);
                __syncthreads();
                for (int it = 0; it < 20; ++it) {
                    gs_any<TA, NT>(A, C, V, true, false);
                    gs_any<TA, NT>(A, C, V, false, false);
                }
            }
            break;
        }
        if (A.mc) {                                     // colours: from x = 0 with full rows (x of later colours is 0)
            TA* xl = V.x(A, C);
            for (int k = threadIdx.x; k < A.n; k += blockDim.x) xl[k] = TA(0);
            __syncthreads();
        }
        gs_any<TA, NT>(A, C, V, true, !A.mc);
        if (A.W == AMG_W0) residual<TA, AMG_W0, NT>(A, C, V.x(A, C), V.b(A, C), V.r(A, C));
        else residual<TA, AMG_W1, NT>(A, C, V.x(A, C), V.b(A, C), V.r(A, C));
        __syncthreads();
        // restriction b_{l+1} = R r: members in ascending natural order (amg.cpp:324)
        {
            const AmgSysLv Cl = C.lv[s * C.maxL + l + 1];
            const int* mp = C.memPtr + Cl.rpOff;
            const int* mem = C.mem + Cl.memOff;
            const TA* rl = V.r(A, C);
            TA* bc = V.b(Cl, C);
            for (int I = threadIdx.x; I < Cl.n; I += blockDim.x) {
                const int q0 = __ldg(mp + I), q1 = __ldg(mp + I + 1);
                TA t = TA(0);
                for (int q = q0; q < q1; ++q) t = aadd(t, rl[__ldg(mem + q)]);
                bc[I] = t;
            }
        }
        __syncthreads();
    }
    for (l = l - 1; l >= lstart; --l) {                     // prolongation and post-smoothing (amg.cpp:326-327)
        const AmgSysLv A = C.lv[s * C.maxL + l];
        const AmgSysLv Cl = C.lv[s * C.maxL + l + 1];
        TA* xl = V.x(A, C);
        const TA* xc = V.x(Cl, C);
        const int* agg = C.agg + A.rowOff;
        for (int k = threadIdx.x; k < A.n; k += blockDim.x) xl[k] = aadd(xl[k], xc[__ldg(agg + k)]);
        __syncthreads();
        gs_any<TA, NT>(A, C, V, false, false);
    }
}

template <class TA, int NT>
__device__ __noinline__ void vcycle_call(int s, const CprArgs<TA>& C, const VVecs<TA>& V, int lstart) {
    vcycle_body<TA, NT>(s, C, V, lstart);
}
template <class TA, int NT>
__device__ __forceinline__ void vcycle(int s, const CprArgs<TA>& C, const VVecs<TA>& V, int lstart = 0) {
    vcycle_call<TA, NT>(s, C, V, lstart);
}

// t -= S_kj[:,p] xp_j for the pressure column of one block (TT: the arithmetic of the second-stage input)
__device__ __forceinline__ void sub_p(double (&acc)[3], const double* s3, double xk) {
#pragma unroll
    for (int e = 0; e < 3; ++e) acc[e] = ds(acc[e], dm(s3[e], xk));
}
__device__ __forceinline__ void sub_p(double (&acc)[3], const float* s3, double xk) {
#pragma unroll
    for (int e = 0; e < 3; ++e) acc[e] = ds(acc[e], dm(double(s3[e]), xk));
}
__device__ __forceinline__ void sub_p(float (&acc)[3], const float* s3, float xk) {
#pragma unroll
    for (int e = 0; e < 3; ++e) acc[e] = acc[e] - s3[e] * xk;
}

// acc -= the overflow list's pressure columns times xp, from position q in list order, in chunks as ov_sub
template <class TV, class TA>
__device__ __forceinline__ void ov_sub_p(TV (&acc)[3], const int* __restrict__ oc, const TA* __restrict__ s3v, int q, const TA* xp) {
    for (;; q += OV_CHUNK) {
        int c[OV_CHUNK];
        TA s3[OV_CHUNK][3];
#pragma unroll
        for (int u = 0; u < OV_CHUNK; ++u) {
            c[u] = __ldg(oc + q + u);
#pragma unroll
            for (int e = 0; e < 3; ++e) s3[u][e] = __ldg(s3v + size_t(q + u) * 3 + e);
        }
#pragma unroll
        for (int u = 0; u < OV_CHUNK; ++u) {
            if (c[u] < 0) return;
            sub_p(acc, s3[u], TV(xp[c[u]]));
        }
    }
}

// One CPR application per system. The second-stage input t lives in C.T with the sweep vector's type TV: FP64
// for the FP64 and mixed forms, FP32 for the all-FP32 preconditioner, whose restriction w . r, t = r - S[:,p] xp
// and sweeps then run in FP32 arithmetic (the FP64 unit is a small fraction of the FP32 rate on this part).
template <class TF, class TV, class TA, int MODE, int NT = cta_threads<TF, TV>()>
__global__ void __launch_bounds__(NT) k_cpr_cta(IluArgs<TF> F, CprArgs<TA> C, const double* r, double* pv, const double* v,
                                                        double* z, TV* yglob, size_t smemBytes, const KScal* ks) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int s = blockIdx.x, tid = int(threadIdx.x), nt = int(blockDim.x);
    const int row0 = __ldg(F.sysRow0 + s), ns = __ldg(F.sysRow0 + s + 1) - row0;
    double beta = 0, omega = 0, alpha = 0;
    if (ks) {
        const KScal& K = ks[s];
        if (K.status != ST_RUNNING) return;
        beta = K.beta; omega = K.omega; alpha = K.alpha;
    }
    TV* T = reinterpret_cast<TV*>(C.T);
    // V-cycle vectors of this system: as many of x, b, r on chip as fit
    int R = 0;
    for (int l = 0; l < C.maxL; ++l) R += C.lv[s * C.maxL + l].n;
    const size_t vb = size_t(R) * sizeof(TA);
    VVecs<TA> V;
    TA* sm = reinterpret_cast<TA*>(smraw);
    V.xs = vb <= smemBytes ? sm : nullptr;
    V.bs = 2 * vb <= smemBytes ? sm + R : nullptr;
    V.rs = 3 * vb <= smemBytes ? sm + 2 * R : nullptr;
    V.bGlobal = V.bs == nullptr;
    const AmgSysLv A0 = C.lv[s * C.maxL];
    TA* b0 = V.b(A0, C);
    // input (fused Krylov update) and pressure restriction rp = w . r (bsr.cpp:1064-1067), rows in batches of 4
    // (all loads of a batch issued before any use)
    constexpr int IB = sizeof(TV) == 4 ? 4 : 1;                   // FP64 forms: registers
    for (int base = row0 + tid; base < row0 + ns; base += IB * nt) {
        double ri[IB][3], pi[IB][3], vi[IB][3], wi[IB][3];
#pragma unroll
        for (int u = 0; u < IB; ++u) {
            const int k = min(base + u * nt, row0 + ns - 1);    // past the end: re-read the last row, not stored
#pragma unroll
            for (int e = 0; e < 3; ++e) {
                const size_t q = size_t(k) * 3 + e;
                ri[u][e] = r[q];
                pi[u][e] = MODE == IN_PUPDATE ? pv[q] : 0.0;
                vi[u][e] = MODE != IN_PLAIN ? v[q] : 0.0;
                wi[u][e] = __ldg(C.w + q);
            }
        }
#pragma unroll
        for (int u = 0; u < IB; ++u) {
            const int k = base + u * nt;
            if (k >= row0 + ns) break;
            double in[3];
#pragma unroll
            for (int e = 0; e < 3; ++e) {
                const size_t q = size_t(k) * 3 + e;
                if (MODE == IN_PUPDATE) { in[e] = da(ri[u][e], dm(beta, ds(pi[u][e], dm(omega, vi[u][e])))); pv[q] = in[e]; }
                else if (MODE == IN_SUPDATE) { in[e] = ds(ri[u][e], dm(alpha, vi[u][e])); pv[q] = in[e]; }
                else in[e] = ri[u][e];
                T[q] = TV(in[e]);
            }
            if (sizeof(TV) == 4) {
                const float i0 = float(in[0]), i1 = float(in[1]), i2 = float(in[2]);
                b0[k - row0] = TA(float(wi[u][0]) * i0 + float(wi[u][1]) * i1 + float(wi[u][2]) * i2);
            } else {
                b0[k - row0] = TA(da(da(dm(wi[u][0], in[0]), dm(wi[u][1], in[1])), dm(wi[u][2], in[2])));
            }
        }
    }
    __syncthreads();
    vcycle<TA, NT>(s, C, V);
    // second stage on t = r - S[:,p] xp (pressure columns in S's row order, bsr.cpp:1071-1081); xp to global
    // memory for the final correction when it lived on chip
    const TA* xp = V.x(A0, C);
    TA* xpg = C.x + A0.rowOff;
    // rows in batches of TB (all record loads of a batch issued before any use)
    constexpr int TB = 2;
    for (int base = row0 + tid; base < row0 + ns; base += TB * nt) {
        int4 lc[TB], uc[TB];
        TA sp[TB][SPREC];
        TV acc[TB][3];
#pragma unroll
        for (int u = 0; u < TB; ++u) {
            const int k = min(base + u * nt, row0 + ns - 1);    // past the end: re-read the last row, not stored
            lc[u] = __ldg(F.Lslot + k);
            uc[u] = __ldg(F.Uslot + k);
            ldrec(sp[u], C.sp + size_t(k) * SPREC);
#pragma unroll
            for (int e = 0; e < 3; ++e) acc[u][e] = T[size_t(k) * 3 + e];
        }
#pragma unroll
        for (int u = 0; u < TB; ++u) {
            const int k = base + u * nt;
            if (k >= row0 + ns) break;
#pragma unroll
            for (int j = 0; j < SLOTS; ++j)
                if (slot_col(lc[u], j) >= 0) sub_p(acc[u], sp[u] + 3 * j, TV(xp[slot_col(lc[u], j)]));
            if (lc[u].w >= 0) ov_sub_p(acc[u], F.LovCol, C.spLov, lc[u].w, xp);
            sub_p(acc[u], sp[u] + 3 * SLOTS, TV(xp[k - row0]));
#pragma unroll
            for (int j = 0; j < SLOTS; ++j)
                if (slot_col(uc[u], j) >= 0) sub_p(acc[u], sp[u] + 3 * (SLOTS + 1 + j), TV(xp[slot_col(uc[u], j)]));
            if (uc[u].w >= 0) ov_sub_p(acc[u], F.UovCol, C.spUov, uc[u].w, xp);
            T[size_t(k) * 3] = acc[u][0]; T[size_t(k) * 3 + 1] = acc[u][1]; T[size_t(k) * 3 + 2] = acc[u][2];
            if (V.xs) xpg[k - row0] = xp[k - row0];
        }
    }
    __syncthreads();
    const bool onchip = size_t(ns) * 3 * sizeof(TV) <= smemBytes;
    TV* y = onchip ? reinterpret_cast<TV*>(smraw) : yglob + size_t(row0) * 3;
    const int l0 = __ldg(F.sysLvl0 + s), nl = __ldg(F.sysLvl0 + s + 1) - l0 - 1;
    __shared__ int lvc[kLvCache];
    const int* lv = level_starts(F.lvlStart + l0, nl, lvc);
    const bool writeZ = onchip || sizeof(TV) != sizeof(double);
    if (writeZ) {   // y is not z: z_p += xp (bsr.cpp:1083) as z is written
        ilu_body<TF, TV, TV, IN_PLAIN, true, TA, NT>(F, row0, lv, nl, T, nullptr, nullptr, z, y, true, 0, 0, 0, xpg);
    } else {        // y is z itself: the correction after the sweeps
        ilu_body<TF, TV, TV, IN_PLAIN, false, TA, NT>(F, row0, lv, nl, T, nullptr, nullptr, z, y, false, 0, 0, 0, nullptr);
        for (int k = row0 + tid; k < row0 + ns; k += nt) z[size_t(k) * 3] = da(z[size_t(k) * 3], double(xpg[k - row0]));
    }
}

// ------------------------------------------------------------------ all-FP32 BILU0 factorisation
// The precision form's factorisation: FP32 elimination and storage, the pivot block inverted in FP64
// (invert_pivot3: the reference's pivoting and singular-block shift, engine/src/bsr.cpp:67-87, 204-212) and rounded.
// One thread block per system walks the forward levels; a thread eliminates whole rows (row algorithm of
// engine/src/bsr.cpp:183-215 with the plan's elimination lists, every float operation rounded on its own).
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ void gemm3f(const float* a, const float* b, float* c) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float r0 = 0.f, r1 = 0.f, r2 = 0.f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float f = a[i * 3 + k];
            r0 = fa(r0, fm(f, b[k * 3 + 0]));
            r1 = fa(r1, fm(f, b[k * 3 + 1]));
            r2 = fa(r2, fm(f, b[k * 3 + 2]));
        }
        c[i * 3 + 0] = r0; c[i * 3 + 1] = r1; c[i * 3 + 2] = r2;
    }
}
constexpr int kFacChunk = 4;       // elimination targets of one entry loaded at once
__device__ __forceinline__ void gemm3f_sub(const float* a, const float* b, float* c) {
    float t[9];
    gemm3f(a, b, t);
#pragma unroll
    for (int e = 0; e < 9; ++e) c[e] = fs(c[e], t[e]);
}

__global__ void __launch_bounds__(kCtaThreads) k_factor_cta_f32(const int* __restrict__ sysRow0, const int* __restrict__ sysLvl0,
                                                               const int* __restrict__ lvlStart, const int* __restrict__ rowPtr,
                                                               const int* __restrict__ col, const int* __restrict__ diag,
                                                               const int* __restrict__ elimPtr, const int* __restrict__ elimT,
                                                               const int* __restrict__ elimQ, const double* __restrict__ val, float* F,
                                                               int* nreg) {
    const int s = blockIdx.x, tid = int(threadIdx.x), nt = int(blockDim.x);
    const int r0 = __ldg(sysRow0 + s), r1 = __ldg(sysRow0 + s + 1);
    const size_t e0 = size_t(__ldg(rowPtr + r0)) * 9, e1 = size_t(__ldg(rowPtr + r1)) * 9;
    for (size_t e = e0 + size_t(tid); e < e1; e += size_t(nt)) F[e] = float(__ldg(val + e));
    __syncthreads();
    const int l0 = __ldg(sysLvl0 + s), nl = __ldg(sysLvl0 + s + 1) - l0 - 1;
    __shared__ int lvc[kLvCache];
    const int* lv = level_starts(lvlStart + l0, nl, lvc);
    int reg = 0;
    float Lb[9];
    for (int L = 0; L < nl; ++L) {
        const int k1 = lv[L + 1];
        for (int i = lv[L] + tid; i < k1; i += nt) {
            const int p0 = __ldg(rowPtr + i), d = __ldg(diag + i);
            // the indices of entry p (column k, elimination list [q0, q1)) are loaded one entry ahead, so an entry
            // costs two dependent loads (diag[k] with its first elimination targets, then every block it touches)
            int k = 0, q0 = 0, q1 = 0;
            if (p0 < d) { k = __ldg(col + p0); q0 = __ldg(elimPtr + p0); q1 = __ldg(elimPtr + p0 + 1); }
            for (int p = p0; p < d; ++p) {
                const int kn = p + 1 < d ? __ldg(col + p + 1) : 0;
                const int q2 = p + 1 < d ? __ldg(elimPtr + p + 2) : 0;
                const int dk = __ldg(diag + k);
                for (int qc = q0; qc == q0 || qc < q1; qc += kFacChunk) {
                    int t[kFacChunk], uq[kFacChunk];
#pragma unroll
                    for (int v = 0; v < kFacChunk; ++v) {
                        const bool ok = qc + v < q1;
                        t[v] = ok ? __ldg(elimT + qc + v) : -1;
                        uq[v] = ok ? __ldg(elimQ + qc + v) : 0;
                    }
                    float U[kFacChunk][9], Cb[kFacChunk][9];
#pragma unroll
                    for (int v = 0; v < kFacChunk; ++v)
                        if (t[v] >= 0) {
#pragma unroll
                            for (int e = 0; e < 9; ++e) { U[v][e] = F[size_t(uq[v]) * 9 + e]; Cb[v][e] = F[size_t(t[v]) * 9 + e]; }
                        }
                    if (qc == q0) {                                   // L_ik = A_ik U_kk^-1, once per entry
                        float a[9], u[9];
#pragma unroll
                        for (int e = 0; e < 9; ++e) { a[e] = F[size_t(p) * 9 + e]; u[e] = F[size_t(dk) * 9 + e]; }
                        gemm3f(a, u, Lb);
#pragma unroll
                        for (int e = 0; e < 9; ++e) F[size_t(p) * 9 + e] = Lb[e];
                    }
#pragma unroll
                    for (int v = 0; v < kFacChunk; ++v)
                        if (t[v] >= 0) {
                            gemm3f_sub(Lb, U[v], Cb[v]);                 // A_it -= L_ik U_kq (targets of one entry differ)
#pragma unroll
                            for (int e = 0; e < 9; ++e) F[size_t(t[v]) * 9 + e] = Cb[v][e];
                        }
                }
                k = kn; q0 = q1; q1 = q2;
            }
            double D[9];
#pragma unroll
            for (int e = 0; e < 9; ++e) D[e] = double(F[size_t(d) * 9 + e]);
            reg += invert_pivot3(D);
#pragma unroll
            for (int e = 0; e < 9; ++e) F[size_t(d) * 9 + e] = float(D[e]);
        }
        __syncthreads();
    }
    if (reg) atomicAdd(nreg, reg);
}

// factors (level-space CSR block order) -> slot records; overflow blocks
template <class T>
__global__ void k_pack(int n, int nLov, int nUov, const int* __restrict__ LslotSrc, const int* __restrict__ UslotSrc,
                       const int* __restrict__ Dsrc, const int* __restrict__ LovSrc, const int* __restrict__ UovSrc,
                       const int2* __restrict__ rowLevel, const T* __restrict__ lu, T* L, T* UD, T* Lov, T* Uov) {
    const size_t nL = size_t(n) * LREC, nUD = size_t(n) * UREC, nO = (size_t(nLov) + size_t(nUov)) * 9;
    const size_t total = nL + nUD + nO;
    for (size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x; q < total; q += size_t(gridDim.x) * blockDim.x) {
        if (q < nL) {                                  // value e of row k, component-major within k's level
            const size_t k = q / LREC, e = q % LREC, j = e / 9;
            const int2 lw = __ldg(rowLevel + k);
            const int src = j < size_t(SLOTS) ? __ldg(LslotSrc + k * SLOTS + j) : -1;
            L[size_t(lw.x) * LREC + e * size_t(lw.y) + (k - size_t(lw.x))] = src >= 0 ? lu[size_t(src) * 9 + e % 9] : T(0);
        } else if (q < nL + nUD) {
            const size_t q2 = q - nL, k = q2 / UREC, e = q2 % UREC, j = e / 9;
            const int2 lw = __ldg(rowLevel + k);
            const int src = j < size_t(SLOTS) ? __ldg(UslotSrc + k * SLOTS + j) : __ldg(Dsrc + k);
            UD[size_t(lw.x) * UREC + e * size_t(lw.y) + (k - size_t(lw.x))] = src >= 0 ? lu[size_t(src) * 9 + e % 9] : T(0);
        } else {
            const size_t q3 = q - nL - nUD, b = q3 / 9, e = q3 % 9;
            if (b < size_t(nLov)) {
                const int src = __ldg(LovSrc + b);
                Lov[q3] = src >= 0 ? lu[size_t(src) * 9 + e] : T(0);
            } else {
                const int src = __ldg(UovSrc + (b - nLov));
                Uov[q3 - size_t(nLov) * 9] = src >= 0 ? lu[size_t(src) * 9 + e] : T(0);
            }
        }
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

template <class TF>
IluArgs<TF> ilu_args(const DevPlan& P, const SplitFactors<TF>& S) {
    return IluArgs<TF>{P.sysRow0, P.sysLvl0, P.lvlStart, P.Lslot, P.Uslot, P.LovCol, P.UovCol, S.L, S.UD, S.Lov, S.Uov};
}

template <class TF, class TV, int MODE>
void launch_cta(const DevPlan& P, const SplitFactors<TF>& S, size_t smem, const double* r, double* pv, const double* v, double* z,
                TV* yglob, const KScal* ks, cudaStream_t st) {
    raise_smem_limit(reinterpret_cast<const void*>(k_ilu_cta<TF, TV, MODE>), int(smem));
    k_ilu_cta<TF, TV, MODE><<<P.nsys, cta_threads<TF, TV>(), smem, st>>>(ilu_args(P, S), r, pv, v, z, yglob, smem, ks);
}

template <int MODE>
void dispatch(const DevPlan& P, const PrecDev& M, const double* r, double* pv, const double* v, double* z, const KScal* ks,
              cudaStream_t st) {
    if (M.kind == 0) launch_cta<double, double, MODE>(P, M.s64, M.smem, r, pv, v, z, z, ks, st);
    else if (M.kind == 1) launch_cta<float, double, MODE>(P, M.s32, M.smem, r, pv, v, z, z, ks, st);
    else launch_cta<float, float, MODE>(P, M.s32, M.smem, r, pv, v, z, M.y32, ks, st);
}

}  // namespace

size_t cta_sweep_smem(const DevPlan& P, bool vec32) {
    // the largest system's vector if it fits, else all the opt-in shared memory (systems that fit use it)
    const size_t need = size_t(P.maxSysRows) * 3 * (vec32 ? sizeof(float) : sizeof(double));
    const size_t cap = size_t(max_smem_optin()) - kCtaStaticSmem;
    return need <= cap ? need : cap;
}

bool cta_sweep_supported(const DevPlan& P, const HostPlan& H) {
    // structurally symmetric (reversed forward levels are backward levels) and small enough for one SM
    return H.symmetric && P.maxSysRows > 0 && P.maxSysRows <= 65536;
}

void launch_pack_f64(const DevPlan& P, const double* lu, SplitFactors<double>& F, cudaStream_t st) {
    const size_t total = size_t(P.n) * (LREC + UREC) + (size_t(P.nLov) + size_t(P.nUov)) * 9;
    const int grid = int(std::min<size_t>((total + 255) / 256, size_t(device_sm_count()) * 16));
    k_pack<double><<<grid, 256, 0, st>>>(P.n, P.nLov, P.nUov, P.LslotSrc, P.UslotSrc, P.Dsrc, P.LovSrc, P.UovSrc, P.rowLevel, lu, F.L,
                                         F.UD, F.Lov, F.Uov);
}
void launch_pack_f32(const DevPlan& P, const float* luf, SplitFactors<float>& F, cudaStream_t st) {
    const size_t total = size_t(P.n) * (LREC + UREC) + (size_t(P.nLov) + size_t(P.nUov)) * 9;
    const int grid = int(std::min<size_t>((total + 255) / 256, size_t(device_sm_count()) * 16));
    k_pack<float><<<grid, 256, 0, st>>>(P.n, P.nLov, P.nUov, P.LslotSrc, P.UslotSrc, P.Dsrc, P.LovSrc, P.UovSrc, P.rowLevel, luf, F.L,
                                        F.UD, F.Lov, F.Uov);
}

void launch_factor_cta_f32(const DevPlan& P, const double* val, float* luf, int* nreg, cudaStream_t st) {
    k_factor_cta_f32<<<P.nsys, kCtaThreads, 0, st>>>(P.sysRow0, P.sysLvl0, P.lvlStart, P.rowPtr, P.col, P.diag, P.elimPtr, P.elimT,
                                                     P.elimQ, val, luf, nreg);
}

void launch_ilu_cta_apply(const DevPlan& P, const PrecDev& M, const double* r, double* z, cudaStream_t st) {
    dispatch<IN_PLAIN>(P, M, r, nullptr, nullptr, z, nullptr, st);
}
void launch_ilu_cta_apply_ks(const DevPlan& P, const PrecDev& M, const double* r, double* z, const KScal* ks, cudaStream_t st) {
    dispatch<IN_PLAIN>(P, M, r, nullptr, nullptr, z, ks, st);
}

void launch_ilu_cta_fused(const DevPlan& P, const PrecDev& M, bool pupdate, const double* r, double* pv, const double* v, double* z,
                          const KScal* ks, cudaStream_t st) {
    if (pupdate) dispatch<IN_PUPDATE>(P, M, r, pv, v, z, ks, st);
    else dispatch<IN_SUPDATE>(P, M, r, pv, v, z, ks, st);
}

namespace {
template <class TA>
CprArgs<TA> cpr_args(const DevAmg& G, const TA* val, const TA* slotVal, const TA* diagVal, const TA* lu, TA* x, TA* b, TA* r, const TA* sp,
                     const TA* spLov, const TA* spUov) {
    return CprArgs<TA>{G.lv, G.maxL, G.lvl, G.gsRows, G.ci, val, G.slotCol, slotVal, diagVal, G.rowMeta, G.agg, G.memPtr, G.mem, lu, G.invf,
                       G.luPerm, G.cin, x, b, r, G.w, G.T, sp, spLov, spUov, G.coarse64, G.lu, G.x, G.b, G.r};
}

template <class TF, class TV, class TA, int MODE>
void launch_cpr_t(const DevPlan& P, const SplitFactors<TF>& S, size_t smem, const CprArgs<TA>& C, const DevAmg& G, const double* r,
                  double* pv, const double* v, double* z, TV* yglob, const KScal* ks, cudaStream_t st) {
    // shared memory: the larger of the sweep vector and the V-cycle vectors of the largest system, within the cap
    const size_t cap = size_t(max_smem_optin()) - kCtaStaticSmem;
    smem = std::max(smem, std::min(cap, size_t(G.maxSysAmgRows) * 3 * sizeof(TA)));
    raise_smem_limit(reinterpret_cast<const void*>(k_cpr_cta<TF, TV, TA, MODE>), int(smem));
    k_cpr_cta<TF, TV, TA, MODE><<<P.nsys, cta_threads<TF, TV>(), smem, st>>>(ilu_args(P, S), C, r, pv, v, z, yglob, smem, ks);
}
}  // namespace

void launch_cpr_cta(const DevPlan& P, const PrecDev& M, const DevAmg& G, int mode, bool amgFp32, const double* r, double* pv,
                    const double* v, double* z, const KScal* ks, cudaStream_t st) {
    (void)amgFp32;
    auto go = [&](auto tag_mode) {
        constexpr int MODE = decltype(tag_mode)::value;
        if (M.kind == 0) {
            const CprArgs<double> C = cpr_args<double>(G, G.val, G.slotVal, G.diagVal, G.lu, G.x, G.b, G.r, G.sp, G.spLov, G.spUov);
            launch_cpr_t<double, double, double, MODE>(P, M.s64, M.smem, C, G, r, pv, v, z, z, ks, st);
        } else {
            const CprArgs<float> C = cpr_args<float>(G, G.valf, G.slotValf, G.diagValf, G.luf, G.xf, G.bf, G.rf, G.spf, G.spLovf, G.spUovf);
            if (M.kind == 1) launch_cpr_t<float, double, float, MODE>(P, M.s32, M.smem, C, G, r, pv, v, z, z, ks, st);
            else launch_cpr_t<float, float, float, MODE>(P, M.s32, M.smem, C, G, r, pv, v, z, M.y32, ks, st);
        }
    };
    if (mode == IN_PUPDATE) go(std::integral_constant<int, IN_PUPDATE>());
    else if (mode == IN_SUPDATE) go(std::integral_constant<int, IN_SUPDATE>());
    else go(std::integral_constant<int, IN_PLAIN>());
}

// ------------------------------------------------------------------ CPR application grid-wide (systems of any size)
// The thread-block application above keeps a system on one SM; a system of a million cells needs the whole GPU.
// Here every step of BlockCPR::apply runs over the whole batch, one AMG level at a time, with the arithmetic of
// the thread-block V-cycle:
// * Gauss-Seidel sweeps are sync-free: a persistent grid claims the level's rows in schedule order (forward levels
//   of the reference order, or colours) and a row waits, through per-row flags, only for its neighbours of an
//   earlier wave (the rows a forward sweep updates before it: its lower-numbered neighbours in the reference order,
//   whose forward level is lower, or those of an earlier colour). Its other neighbours wait for it in turn
//   (structurally symmetric levels), so their old values are still in place when it reads them. Claiming in
//   schedule order keeps every awaited row on a running warp; the waits are bounded (rsg_sync.cuh).
// * The residual and the restriction are one pass per coarse row (every fine row belongs to one aggregate), the
//   prolongation one pass per fine row, the coarsest level one thread block per system (dense LU in FP64, the
//   explicit inverse in the FP32 forms).
// * t = r - S[:,p] xp reads the pressure column of every block of S in row order; the BILU0 stage is the grid
//   sync-free sweep of the handle's factors.
namespace {

constexpr int kGridThreads = 128;

int grid_for(long long n, int threads) {
    const long long b = (n + threads - 1) / threads, cap = 16LL * device_sm_count();
    return int(b < 1 ? 1 : (b < cap ? b : cap));
}

// input (the fused Krylov update of the mode), T = input (TS: FP64, or the split form's second-stage type),
// level-0 right-hand side b0 = w . input (bsr.cpp:1064-1067; TT: the arithmetic of the restriction, FP32 in the
// all-FP32 form)
template <int MODE, class TA, class TT, class TS>
__device__ __forceinline__ void gcpr_in_body(int n, const int* __restrict__ rowSys, const double* r, double* pv, const double* v,
                                                 const double* __restrict__ w, TS* T, TA* b0, const KScal* ks) {
    for (int k = int(blockIdx.x * blockDim.x + threadIdx.x); k < n; k += int(gridDim.x * blockDim.x)) {
        double beta = 0, omega = 0, alpha = 0;
        if (ks) {
            const KScal& K = ks[__ldg(rowSys + k)];
            if (K.status != ST_RUNNING) continue;
            beta = K.beta; omega = K.omega; alpha = K.alpha;
        }
        double in[3];
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            const size_t q = size_t(k) * 3 + e;
            if (MODE == IN_PUPDATE) { in[e] = da(r[q], dm(beta, ds(pv[q], dm(omega, v[q])))); pv[q] = in[e]; }
            else if (MODE == IN_SUPDATE) { in[e] = ds(r[q], dm(alpha, v[q])); pv[q] = in[e]; }
            else in[e] = r[q];
            T[q] = TS(in[e]);
        }
        const double w0 = __ldg(w + size_t(k) * 3), w1 = __ldg(w + size_t(k) * 3 + 1), w2 = __ldg(w + size_t(k) * 3 + 2);
        if (sizeof(TT) == 4) b0[k] = TA(float(w0) * float(in[0]) + float(w1) * float(in[1]) + float(w2) * float(in[2]));
        else b0[k] = TA(da(da(dm(w0, in[0]), dm(w1, in[1])), dm(w2, in[2])));
    }
}
template <int MODE, class TA, class TT, class TS>
__global__ void __launch_bounds__(256) k_gcpr_in(int n, const int* __restrict__ rowSys, const double* r, double* pv, const double* v,
                                                 const double* __restrict__ w, TS* T, TA* b0, const KScal* ks) {
    gcpr_in_body<MODE, TA, TT, TS>(n, rowSys, r, pv, v, w, T, b0, ks);
}

// one Gauss-Seidel sweep of level l over every system (engine/src/amg.cpp:98-113). Positions [q0, q1) of the
// level's schedule, claimed forward or backward. phase 0: the smoothing sweeps (systems whose level l is the
// coarsest skip); phase 1: the symmetric GS solve of a coarsest level without dense LU. ZERO: pre-smoothing from
// x = 0 (the terms of the neighbours not yet updated vanish and are not read). Flags of skipped rows are set all
// the same: after every forward sweep of a (level, phase) all its flags are 1, after every backward sweep 0.
template <class TA, bool FWD, bool ZERO, bool POS>
__device__ __forceinline__ void gs_grid_body(int q0, int q1, int maxL, int phase, const int* __restrict__ rowLv,
                                                          const AmgSysLv* __restrict__ lv, const int* __restrict__ gsRows,
                                                          const int* __restrict__ wave, const int* __restrict__ rp,
                                                          const int* __restrict__ ci, const TA* __restrict__ val,
                                                          const int* __restrict__ diag, const TA* b, TA* x, int* flag, unsigned* ctr,
                                                          const KScal* ks, int* err) {
    if (blockIdx.x == 0 && threadIdx.x == 0) ctr[FWD ? 1 : 0] = 0u;   // the opposite direction's counter, for its next sweep
    const int n = q1 - q0, lane = int(threadIdx.x & 31);
    for (;;) {
        __syncwarp();
        const int base = warp_claim(ctr + (FWD ? 0 : 1));
        if (base >= n) break;
        const int idx = base + lane;
        if (idx < n) {
            const int g = FWD ? q0 + idx : q1 - 1 - idx;
            const int sl = __ldg(rowLv + g);
            const AmgSysLv* A = lv + sl;
            const int rowOff = __ldg(&A->rowOff), coarse = __ldg(&A->coarse);
            const int row = rowOff + __ldg(gsRows + g);
            bool act = phase == 0 ? !coarse : (coarse && !__ldg(&A->dense));
            if (act && ks) act = ks[sl / maxL].status == ST_RUNNING;
            if (act) {
                const int k = row - rowOff, rpOff = __ldg(&A->rpOff), entOff = __ldg(&A->entOff);
                const int p0 = __ldg(rp + rpOff + k), p1 = __ldg(rp + rpOff + k + 1), pd = __ldg(diag + row);
                const int* cl = ci + entOff;
                const TA* vl = val + entOff;
                const int wi = POS ? 0 : __ldg(wave + row);
                // the neighbours updated before this row in the sweep: of an earlier wave (forward), a later one
                // (backward); POS: the entries before (after) the diagonal, which the plan checked to be the same
                auto dep = [&](int p) {
                    if (p == pd) return false;
                    if (POS) return FWD ? p < pd : p > pd;
                    const int w = __ldg(wave + rowOff + __ldg(cl + p));
                    return FWD ? w < wi : w > wi;
                };
                const int w0 = POS ? (FWD ? p0 : pd + 1) : p0, w1 = POS ? (FWD ? pd : p1) : p1;
                const int e1 = (FWD && ZERO && POS) ? pd : p1;         // from zero: only the updated neighbours count
                TA vp[8];                                              // the row's first values and columns, loaded
                int jp[8];                                             // before the wait (read-only)
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    vp[u] = p0 + u < e1 ? __ldg(vl + p0 + u) : TA(0);
                    jp[u] = p0 + u < e1 ? rowOff + __ldg(cl + p0 + u) : 0;
                }
                const TA dv = __ldg(vl + pd);
                wait_deps(flag, w0, w1, FWD ? 1 : 0, err, [&](int p) { return rowOff + __ldg(cl + p); }, dep);
                TA s = b[row];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int p = p0 + u;
                    if (p >= e1) break;
                    if (p == pd) continue;
                    if (FWD && ZERO && !POS && __ldg(wave + jp[u]) > wi) continue;   // x_j is still zero: the term vanishes
                    s = asub(s, amul(vp[u], x[jp[u]]));
                }
                for (int p = p0 + 8; p < e1; ++p) {
                    if (p == pd) continue;
                    const int j = rowOff + __ldg(cl + p);
                    if (FWD && ZERO && !POS && __ldg(wave + j) > wi) continue;
                    s = asub(s, amul(__ldg(vl + p), x[j]));
                }
                x[row] = adiv(s, dv);
            }
            st_release(flag + row, FWD ? 1 : 0);
        }
    }
}
template <class TA, bool FWD, bool ZERO, bool POS>
__global__ void __launch_bounds__(kGridThreads) k_gs_grid(int q0, int q1, int maxL, int phase, const int* __restrict__ rowLv,
                                                          const AmgSysLv* __restrict__ lv, const int* __restrict__ gsRows,
                                                          const int* __restrict__ wave, const int* __restrict__ rp,
                                                          const int* __restrict__ ci, const TA* __restrict__ val,
                                                          const int* __restrict__ diag, const TA* b, TA* x, int* flag, unsigned* ctr,
                                                          const KScal* ks, int* err) {
    gs_grid_body<TA, FWD, ZERO, POS>(q0, q1, maxL, phase, rowLv, lv, gsRows, wave, rp, ci, val, diag, b, x, flag, ctr, ks, err);
}

// Multicolour Gauss-Seidel (FP32 forms) on the colour-major row descriptors {row, first entry, end, diagonal}:
// the rows of a colour are independent. ZERO: pre-smoothing from x = 0 (the terms of later colours vanish and are
// not read).
template <class TA, bool ZERO>
__device__ __forceinline__ void gs_colour_row(const int4 d, const int* __restrict__ gci, const TA* __restrict__ val,
                                              const int* __restrict__ wave, const TA* b, TA* x) {
    const int wi = ZERO ? __ldg(wave + d.x) : 0;
    TA s = b[d.x];
    // entries in chunks whose loads are all issued before the terms are taken (in entry order): a row costs two
    // dependent loads per chunk, not per entry
    constexpr int CH = 8;
    for (int p0 = d.y; p0 < d.z; p0 += CH) {
        int j[CH];
        TA a[CH], xv[CH];
        bool use[CH];
#pragma unroll
        for (int u = 0; u < CH; ++u) {
            const int p = p0 + u;
            use[u] = p < d.z && p != d.w;
            j[u] = use[u] ? __ldg(gci + p) : 0;
            a[u] = use[u] ? __ldg(val + p) : TA(0);
        }
#pragma unroll
        for (int u = 0; u < CH; ++u) {
            if (ZERO && use[u] && __ldg(wave + j[u]) > wi) use[u] = false;   // x_j still zero: the term is not taken
            xv[u] = use[u] ? x[j[u]] : TA(0);
        }
#pragma unroll
        for (int u = 0; u < CH; ++u)
            if (use[u]) s = asub(s, amul(a[u], xv[u]));
    }
    x[d.x] = adiv(s, __ldg(val + d.w));
}
// one large colour: a parallel pass over the descriptors [i0, i1)
template <class TA, bool ZERO>
__device__ __forceinline__ void gs_colour_body(int i0, int i1, int maxL, const int4* __restrict__ cdesc, const int* __restrict__ gci,
                                                   const TA* __restrict__ val, const int* __restrict__ wave, const int* __restrict__ rowLv,
                                                   const TA* b, TA* x, const KScal* ks) {
    for (int i = i0 + int(blockIdx.x * blockDim.x + threadIdx.x); i < i1; i += int(gridDim.x * blockDim.x)) {
        const int4 d = __ldg(cdesc + i);
        if (ks && ks[__ldg(rowLv + d.x) / maxL].status != ST_RUNNING) continue;
        gs_colour_row<TA, ZERO>(d, gci, val, wave, b, x);
    }
}
template <class TA, bool ZERO>
__global__ void __launch_bounds__(256) k_gs_colour(int i0, int i1, int maxL, const int4* __restrict__ cdesc, const int* __restrict__ gci,
                                                   const TA* __restrict__ val, const int* __restrict__ wave, const int* __restrict__ rowLv,
                                                   const TA* b, TA* x, const KScal* ks) {
    gs_colour_body<TA, ZERO>(i0, i1, maxL, cdesc, gci, val, wave, rowLv, b, x, ks);
}
// The small colours (from colour `tail` on) of a level in one sync-free pass. Their rows are the long rows of the
// well cliques, so a warp takes one row: rows are claimed in colour order (forward ascending, backward
// descending), the lanes split the row's entries, poll together the flags of its neighbours of an earlier colour
// inside the tail (forward; a later one backward) until the whole warp sees them set, then take the terms in entry
// order. The large colours are done before (forward) or after (backward) by their own passes, so
// their values are final or old as the multicolour order wants. Flags: 1 after the forward pass, 0 after the
// backward one; bounded waits (ERR_TIMEOUT).
template <class TA, bool FWD, bool ZERO>
__device__ __forceinline__ void gs_tail_body(int i0, int i1, int tail, int maxL, const int4* __restrict__ cdesc,
                                                          const int* __restrict__ gci, const TA* __restrict__ val,
                                                          const int* __restrict__ wave, const int* __restrict__ rowLv, const TA* b, TA* x,
                                                          int* flag, unsigned* ctr, const KScal* ks, int* err) {
    if (blockIdx.x == 0 && threadIdx.x == 0) ctr[FWD ? 1 : 0] = 0u;   // the opposite direction's counter, for its next pass
    const int n = i1 - i0, lane = int(threadIdx.x & 31);
    const int want = FWD ? 1 : 0;
    for (;;) {
        unsigned got = 0;
        if (lane == 0) got = atomicAdd(ctr + (FWD ? 0 : 1), 1u);
        const int idx = int(__shfl_sync(0xffffffffu, got, 0));
        if (idx >= n) break;
        const int4 d = __ldg(cdesc + (FWD ? i0 + idx : i1 - 1 - idx));
        const bool run = !ks || ks[__ldg(rowLv + d.x) / maxL].status == ST_RUNNING;
        if (run) {
            const int wi = __ldg(wave + d.x);
            // this lane's entries: up to four polled at once per round (longer rows: the rest in later passes)
            for (int p0 = d.y; p0 < d.z; p0 += 128) {
                int k[4];
                unsigned pending = 0;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int p = p0 + lane + 32 * u;
                    k[u] = -1;
                    if (p < d.z && p != d.w) {
                        const int j = __ldg(gci + p);
                        const int w = __ldg(wave + j);
                        if (FWD ? (w < wi && w >= tail) : w > wi) { k[u] = j; pending |= 1u << u; }
                    }
                }
                unsigned ns = 0;
                for (unsigned it = 0;; ++it) {
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (((pending >> u) & 1u) && ld_relaxed(flag + k[u]) == want) pending &= ~(1u << u);
                    if (!__any_sync(0xffffffffu, pending != 0)) break;
                    if (it >= 64) {
                        __nanosleep(ns);
                        ns = ns < 32 ? 32 : (ns < 256 ? 2 * ns : 256);
                        if (it >= 64 + kSpinLimit) { if (pending) atomicOr(err, ERR_TIMEOUT); break; }
                        if ((it & 255u) == 255u && *(volatile int*)err != 0) break;
                    }
                }
            }
            fence_acquire();
            // s = b - sum a_p x_p in entry order, one rounding after another as the thread-per-row passes and the
            // thread-block sweeps do (the lanes load a chunk's terms, every lane runs the chain on the broadcasts),
            // so a row's value does not depend on which pass took its colour
            TA s = b[d.x];
            for (int p0 = d.y; p0 < d.z; p0 += 32) {
                const int p = p0 + lane;
                TA a = TA(0), xv = TA(0);
                bool use = false;
                if (p < d.z && p != d.w) {
                    const int j = __ldg(gci + p);
                    use = !(ZERO && __ldg(wave + j) > wi);              // x_j still zero: the term is not taken
                    if (use) { a = __ldg(val + p); xv = x[j]; }
                }
                const unsigned m = __ballot_sync(0xffffffffu, use);
                const int cnt = min(32, d.z - p0);
                for (int u = 0; u < cnt; ++u) {
                    const TA au = __shfl_sync(0xffffffffu, a, u), xu = __shfl_sync(0xffffffffu, xv, u);
                    if ((m >> u) & 1u) s = asub(s, amul(au, xu));
                }
            }
            if (lane == 0) x[d.x] = adiv(s, __ldg(val + d.w));
        }
        __syncwarp();
        if (lane == 0) st_release(flag + d.x, want);
    }
}
template <class TA, bool FWD, bool ZERO>
__global__ void __launch_bounds__(kGridThreads) k_gs_tail(int i0, int i1, int tail, int maxL, const int4* __restrict__ cdesc,
                                                          const int* __restrict__ gci, const TA* __restrict__ val,
                                                          const int* __restrict__ wave, const int* __restrict__ rowLv, const TA* b, TA* x,
                                                          int* flag, unsigned* ctr, const KScal* ks, int* err) {
    gs_tail_body<TA, FWD, ZERO>(i0, i1, tail, maxL, cdesc, gci, val, wave, rowLv, b, x, flag, ctr, ks, err);
}

// r = b - A x on the rows [q0, q1) of one level of every system (engine/src/amg.cpp:321-322: the row sum from
// zero in entry order, the diagonal at its place); rows of a system's coarsest level are skipped
template <class TA>
__device__ __forceinline__ void gcpr_resid_body(int q0, int q1, int maxL, const int* __restrict__ rowLv,
                                                    const AmgSysLv* __restrict__ lv, const int* __restrict__ rp,
                                                    const int* __restrict__ ci, const TA* __restrict__ val, const TA* b, const TA* x, TA* r,
                                                    const KScal* ks) {
    for (int g = q0 + int(blockIdx.x * blockDim.x + threadIdx.x); g < q1; g += int(gridDim.x * blockDim.x)) {
        const int sl = __ldg(rowLv + g);
        if (ks && ks[sl / maxL].status != ST_RUNNING) continue;
        const AmgSysLv* F = lv + sl;
        if (__ldg(&F->coarse)) continue;
        const int fOff = __ldg(&F->rowOff), k = g - fOff;
        const int* frp = rp + __ldg(&F->rpOff);
        const int* fci = ci + __ldg(&F->entOff);
        const TA* fv = val + __ldg(&F->entOff);
        const int p0 = __ldg(frp + k), p1 = __ldg(frp + k + 1);
        TA acc = TA(0);
        constexpr int CH = 8;                     // loads of a chunk issued before its terms are summed in order
        for (int q = p0; q < p1; q += CH) {
            int c[CH];
            TA a[CH], xv[CH];
#pragma unroll
            for (int u = 0; u < CH; ++u) {
                c[u] = q + u < p1 ? __ldg(fci + q + u) : 0;
                a[u] = q + u < p1 ? __ldg(fv + q + u) : TA(0);
            }
#pragma unroll
            for (int u = 0; u < CH; ++u) xv[u] = q + u < p1 ? x[fOff + c[u]] : TA(0);
#pragma unroll
            for (int u = 0; u < CH; ++u)
                if (q + u < p1) acc = aadd(acc, amul(a[u], xv[u]));
        }
        r[g] = asub(b[g], acc);
    }
}
template <class TA>
__global__ void __launch_bounds__(256) k_gcpr_resid(int q0, int q1, int maxL, const int* __restrict__ rowLv,
                                                    const AmgSysLv* __restrict__ lv, const int* __restrict__ rp,
                                                    const int* __restrict__ ci, const TA* __restrict__ val, const TA* b, const TA* x, TA* r,
                                                    const KScal* ks) {
    gcpr_resid_body<TA>(q0, q1, maxL, rowLv, lv, rp, ci, val, b, x, r, ks);
}

// restriction b_{l+1} = R r for the coarse rows [c0, c1) of every system: members in ascending natural order
// (engine/src/amg.cpp:324)
template <class TA>
__device__ __forceinline__ void gcpr_restrict_body(int c0, int c1, int maxL, const int* __restrict__ rowLv,
                                                       const AmgSysLv* __restrict__ lv, const int* __restrict__ memPtr,
                                                       const int* __restrict__ mem, TA* b, const TA* r, const KScal* ks) {
    for (int c = c0 + int(blockIdx.x * blockDim.x + threadIdx.x); c < c1; c += int(gridDim.x * blockDim.x)) {
        const int sl = __ldg(rowLv + c);
        if (ks && ks[sl / maxL].status != ST_RUNNING) continue;
        const AmgSysLv* Cl = lv + sl;
        const int I = c - __ldg(&Cl->rowOff);
        const int* mp = memPtr + __ldg(&Cl->rpOff);
        const int* mm = mem + __ldg(&Cl->memOff);
        const TA* rf = r + __ldg(&lv[sl - 1].rowOff);
        const int q0 = __ldg(mp + I), q1 = __ldg(mp + I + 1);
        TA t = TA(0);
        constexpr int CH = 8;
        for (int q = q0; q < q1; q += CH) {
            TA v[CH];
#pragma unroll
            for (int u = 0; u < CH; ++u) v[u] = q + u < q1 ? rf[__ldg(mm + q + u)] : TA(0);
#pragma unroll
            for (int u = 0; u < CH; ++u)
                if (q + u < q1) t = aadd(t, v[u]);
        }
        b[c] = t;
    }
}
template <class TA>
__global__ void __launch_bounds__(256) k_gcpr_restrict(int c0, int c1, int maxL, const int* __restrict__ rowLv,
                                                       const AmgSysLv* __restrict__ lv, const int* __restrict__ memPtr,
                                                       const int* __restrict__ mem, TA* b, const TA* r, const KScal* ks) {
    gcpr_restrict_body<TA>(c0, c1, maxL, rowLv, lv, memPtr, mem, b, r, ks);
}

// x_l += P x_{l+1} (injection of the aggregate's value, engine/src/amg.cpp:326) on the rows [q0, q1) of level l
template <class TA>
__device__ __forceinline__ void gcpr_prolong_body(int q0, int q1, int maxL, const int* __restrict__ rowLv,
                                                      const AmgSysLv* __restrict__ lv, const int* __restrict__ agg, TA* x,
                                                      const KScal* ks) {
    for (int g = q0 + int(blockIdx.x * blockDim.x + threadIdx.x); g < q1; g += int(gridDim.x * blockDim.x)) {
        const int sl = __ldg(rowLv + g);
        if (__ldg(&lv[sl].coarse) || (ks && ks[sl / maxL].status != ST_RUNNING)) continue;
        x[g] = aadd(x[g], x[__ldg(&lv[sl + 1].rowOff) + __ldg(agg + g)]);
    }
}
template <class TA>
__global__ void __launch_bounds__(256) k_gcpr_prolong(int q0, int q1, int maxL, const int* __restrict__ rowLv,
                                                      const AmgSysLv* __restrict__ lv, const int* __restrict__ agg, TA* x,
                                                      const KScal* ks) {
    gcpr_prolong_body<TA>(q0, q1, maxL, rowLv, lv, agg, x, ks);
}

// coarsest level of every system: dense LU (FP64) or explicit inverse (FP32 forms); without a dense LU, x = 0
// before the symmetric GS sweeps of phase 1
template <class TA>
__device__ __forceinline__ void gcpr_coarse_body(CprArgs<TA> C, const KScal* ks, int nsys, int chunks) {
    // work items (system, chunk): with chunks > 1 the rows of an explicit FP32 inverse product are split over several
    // blocks in chunks of blockDim rows (each row's sum is the same whichever block takes it); the LU solves and the
    // FP64 fallback stay with the chunk-0 block of their system
    for (int item = blockIdx.x; item < nsys * chunks; item += gridDim.x) {
        const int s = item / chunks, c = item - s * chunks;
        if (ks && ks[s].status != ST_RUNNING) continue;                  // uniform over the block
        int nlev = 0;
        while (nlev < C.maxL && C.lv[s * C.maxL + nlev].n > 0) ++nlev;
        if (nlev == 0) continue;
        const AmgSysLv A = C.lv[s * C.maxL + nlev - 1];
        TA* x = C.x + A.rowOff;
        if (A.dense) {
            if constexpr (sizeof(TA) == 4) {
                if (C.coarse64[s]) {
                    if (c == 0) coarse_fp64(A, C, x, C.b + A.rowOff);
                } else {
                    coarse_inverse_rows(A, C, x, C.b + A.rowOff, c * int(blockDim.x), chunks > 1 ? (c + 1) * int(blockDim.x) : A.n);
                }
            } else if (c == 0) {
                coarse_dense<TA, 256>(A, C, x, C.b + A.rowOff, C.r + A.rowOff);
            }
        } else if (c == 0) {
            for (int k = threadIdx.x; k < A.n; k += blockDim.x) x[k] = TA(0);
        }
    }
}
template <class TA>
__global__ void __launch_bounds__(256) k_gcpr_coarse(CprArgs<TA> C, const KScal* ks) {
    gcpr_coarse_body<TA>(C, ks, int(gridDim.x), 1);
}

// the coarse part of the V-cycle (levels 1 .. coarsest: smoothing, residual, restriction, coarsest solve,
// prolongation) of one system per thread block, with the thread-block V-cycle's arithmetic (so the values are those of
// the grid passes it replaces); levels this small cost a block barrier per pass instead of a launch
template <class TA, int NT>
__global__ void __launch_bounds__(NT) k_vcycle_lo(CprArgs<TA> C, const KScal* ks, size_t smemBytes) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int s = blockIdx.x;
    if (ks && ks[s].status != ST_RUNNING) return;
    // x, b and r of the levels below the finest on chip when they fit (the Gauss-Seidel colours gather x from shared
    // memory): level 1's right-hand side comes in from the grid restriction, its solution goes out to the grid
    // prolongation; the coarser levels live on chip only
    int R1 = 0;
    for (int l = 1; l < C.maxL; ++l) R1 += C.lv[s * C.maxL + l].n;
    // (a hierarchy of one level has no level 1: the descriptor array holds maxL entries per system)
    const AmgSysLv A1 = C.maxL > 1 ? C.lv[s * C.maxL + 1] : AmgSysLv{};
    if (A1.n > 0 && size_t(3) * size_t(R1) * sizeof(TA) <= smemBytes) {
        TA* sm = reinterpret_cast<TA*>(smraw);
        VVecs<TA> V{sm, sm + R1, sm + 2 * R1, false};
        V.loc0 = A1.locOff;
        const TA* bg = C.b + A1.rowOff;
        for (int k = threadIdx.x; k < A1.n; k += blockDim.x) V.bs[k] = bg[k];
        __syncthreads();
        vcycle<TA, NT>(s, C, V, 1);
        TA* xg = C.x + A1.rowOff;
        for (int k = threadIdx.x; k < A1.n; k += blockDim.x) xg[k] = V.xs[k];
        return;
    }
    const VVecs<TA> V{nullptr, nullptr, nullptr, true};
    vcycle<TA, NT>(s, C, V, 1);
}

// t = input - S[:,p] xp (pressure column of every block in row order, bsr.cpp:1071-1081), in place in T
template <class TA, class TT>
__global__ void __launch_bounds__(256) k_gcpr_t(int n, const int* __restrict__ rowSys, const int* __restrict__ rowPtr,
                                                const int* __restrict__ col, const double* __restrict__ val, const TA* xp, double* T,
                                                const KScal* ks) {
    for (int k = int(blockIdx.x * blockDim.x + threadIdx.x); k < n; k += int(gridDim.x * blockDim.x)) {
        if (ks && ks[__ldg(rowSys + k)].status != ST_RUNNING) continue;
        TT acc[3] = {TT(T[size_t(k) * 3]), TT(T[size_t(k) * 3 + 1]), TT(T[size_t(k) * 3 + 2])};
        for (int p = __ldg(rowPtr + k); p < __ldg(rowPtr + k + 1); ++p) {
            const double* B = val + size_t(p) * 9;
            const TT xk = TT(xp[__ldg(col + p)]);
#pragma unroll
            for (int e = 0; e < 3; ++e) {
                if constexpr (sizeof(TT) == 8) acc[e] = ds(acc[e], dm(__ldg(B + 3 * e), xk));
                else acc[e] = acc[e] - float(__ldg(B + 3 * e)) * xk;
            }
        }
        T[size_t(k) * 3] = double(acc[0]); T[size_t(k) * 3 + 1] = double(acc[1]); T[size_t(k) * 3 + 2] = double(acc[2]);
    }
}

// z_p += xp (bsr.cpp:1083)
template <class TA>
__global__ void __launch_bounds__(256) k_gcpr_zp(int n, const int* __restrict__ rowSys, const TA* xp, double* z, const KScal* ks) {
    for (int k = int(blockIdx.x * blockDim.x + threadIdx.x); k < n; k += int(gridDim.x * blockDim.x)) {
        if (ks && ks[__ldg(rowSys + k)].status != ST_RUNNING) continue;
        z[size_t(k) * 3] = da(z[size_t(k) * 3], double(xp[k]));
    }
}

// split form, second-stage input: t = T - S[:,p] xp in the thread-block kernel's slot order and arithmetic
// (bsr.cpp:1071-1081), one row per thread over every system; xp = the level-0 V-cycle solution of the row's system
template <class TA, class TV>
__device__ __forceinline__ void gcpr_tsp_body(int n, const int* __restrict__ rowSys, const int* __restrict__ sysRow0, int maxL,
                                                  const AmgSysLv* __restrict__ lv, const int4* __restrict__ Lslot,
                                                  const int4* __restrict__ Uslot, const int* __restrict__ LovCol,
                                                  const int* __restrict__ UovCol, const TA* __restrict__ sp, const TA* __restrict__ spLov,
                                                  const TA* __restrict__ spUov, const TA* x, TV* T, const KScal* ks) {
    for (int k = int(blockIdx.x * blockDim.x + threadIdx.x); k < n; k += int(gridDim.x * blockDim.x)) {
        const int s = __ldg(rowSys + k);
        if (ks && ks[s].status != ST_RUNNING) continue;
        const int li = k - __ldg(sysRow0 + s);
        const TA* xp = x + __ldg(&lv[s * maxL].rowOff);
        const int4 lc = __ldg(Lslot + k), uc = __ldg(Uslot + k);
        TA spr[SPREC];
        ldrec(spr, sp + size_t(k) * SPREC);
        TV acc[3] = {T[size_t(k) * 3], T[size_t(k) * 3 + 1], T[size_t(k) * 3 + 2]};
#pragma unroll
        for (int j = 0; j < SLOTS; ++j)
            if (slot_col(lc, j) >= 0) sub_p(acc, spr + 3 * j, TV(xp[slot_col(lc, j)]));
        if (lc.w >= 0) ov_sub_p(acc, LovCol, spLov, lc.w, xp);
        sub_p(acc, spr + 3 * SLOTS, TV(xp[li]));
#pragma unroll
        for (int j = 0; j < SLOTS; ++j)
            if (slot_col(uc, j) >= 0) sub_p(acc, spr + 3 * (SLOTS + 1 + j), TV(xp[slot_col(uc, j)]));
        if (uc.w >= 0) ov_sub_p(acc, UovCol, spUov, uc.w, xp);
        T[size_t(k) * 3] = acc[0]; T[size_t(k) * 3 + 1] = acc[1]; T[size_t(k) * 3 + 2] = acc[2];
    }
}
template <class TA, class TV>
__global__ void __launch_bounds__(256) k_gcpr_tsp(int n, const int* __restrict__ rowSys, const int* __restrict__ sysRow0, int maxL,
                                                  const AmgSysLv* __restrict__ lv, const int4* __restrict__ Lslot,
                                                  const int4* __restrict__ Uslot, const int* __restrict__ LovCol,
                                                  const int* __restrict__ UovCol, const TA* __restrict__ sp, const TA* __restrict__ spLov,
                                                  const TA* __restrict__ spUov, const TA* x, TV* T, const KScal* ks) {
    gcpr_tsp_body<TA, TV>(n, rowSys, sysRow0, maxL, lv, Lslot, Uslot, LovCol, UovCol, sp, spLov, spUov, x, T, ks);
}

// ------------------------------------------------------------------ fused V-cycle: the split form's grid passes in one launch
// The passes above are short and latency-bound (a few dependent loads per row), so as separate launches each costs
// its launch and ramp-up as much as its work. Here one cooperative launch runs them as phases of a persistent kernel:
// every block executes phase after phase over the same row ranges with the same bodies (so every value is the one
// the separate launches compute, bit for bit), separated by grid barriers. The barrier is a counter: each block
// arrives once per barrier and waits until all blocks of the launch have arrived -- the cooperative launch
// guarantees that they are all resident -- with a bounded wait (ERR_TIMEOUT, then the kernel runs on and the host
// reports the error).
template <class TA, class TT>
struct VcArgs {
    CprArgs<TA> C;
    int n, nsys, maxL, totRows;
    const int *rowSys, *sysRow0;
    const double *r, *v;
    double* pv;
    TT* T;
    const int *rowLv, *gsRows, *wave, *rp, *ci, *diag, *gci, *agg;
    const AmgSysLv* lv;
    const int4* cdesc;
    const TA* val;
    int* gsFlag;
    unsigned* gsCtr;
    const int4 *Lslot, *Uslot;
    const int *LovCol, *UovCol;
    int coarseChunks;
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void grid_barrier(unsigned* bar, unsigned& target, int* err) {
    __syncthreads();
    if (threadIdx.x == 0) {
        target += gridDim.x;
        __threadfence();
        atomicAdd(bar, 1u);
        unsigned ns = 0;
        for (unsigned it = 0; ld_acquire_u32(bar) < target; ++it) {
            if (it >= 64) {
                __nanosleep(ns);
                ns = ns < 32 ? 32 : (ns < 256 ? 2 * ns : 256);
                if (it >= 64 + kSpinLimit) { atomicOr(err, ERR_TIMEOUT); break; }
                if ((it & 255u) == 255u && *(volatile int*)err != 0) break;
            }
        }
        __threadfence();
    }
    __syncthreads();
}

template <class TA, class TT, bool POS>
__global__ void __launch_bounds__(256, 4) k_vcycle(const VPhase* __restrict__ ph, int nph, int mode, VcArgs<TA, TT> A, const KScal* ks,
                                                unsigned* bar, int* err) {
    unsigned target = 0;
    for (int i = 0; i < nph; ++i) {
        const VPhase f = ph[i];
        switch (f.kind) {
        case VP_IN:
            if (mode == IN_PUPDATE) gcpr_in_body<IN_PUPDATE, TA, TT, TT>(A.n, A.rowSys, A.r, A.pv, A.v, A.C.w, A.T, A.C.b, ks);
            else if (mode == IN_SUPDATE) gcpr_in_body<IN_SUPDATE, TA, TT, TT>(A.n, A.rowSys, A.r, A.pv, A.v, A.C.w, A.T, A.C.b, ks);
            else gcpr_in_body<IN_PLAIN, TA, TT, TT>(A.n, A.rowSys, A.r, A.pv, A.v, A.C.w, A.T, A.C.b, ks);
            break;
        case VP_COLOUR:
            if (f.c) gs_colour_body<TA, true>(f.a, f.b, A.maxL, A.cdesc, A.gci, A.val, A.wave, A.rowLv, A.C.b, A.C.x, ks);
            else gs_colour_body<TA, false>(f.a, f.b, A.maxL, A.cdesc, A.gci, A.val, A.wave, A.rowLv, A.C.b, A.C.x, ks);
            break;
        case VP_TAIL: {
            unsigned* ctr = A.gsCtr + 4 * f.d;
            if (f.e && f.f)
                gs_tail_body<TA, true, true>(f.a, f.b, f.c, A.maxL, A.cdesc, A.gci, A.val, A.wave, A.rowLv, A.C.b, A.C.x, A.gsFlag, ctr, ks, err);
            else if (f.e)
                gs_tail_body<TA, true, false>(f.a, f.b, f.c, A.maxL, A.cdesc, A.gci, A.val, A.wave, A.rowLv, A.C.b, A.C.x, A.gsFlag, ctr, ks, err);
            else
                gs_tail_body<TA, false, false>(f.a, f.b, f.c, A.maxL, A.cdesc, A.gci, A.val, A.wave, A.rowLv, A.C.b, A.C.x, A.gsFlag, ctr, ks,
                                               err);
            break;
        }
        case VP_GSGRID: {
            int* flag = A.gsFlag + size_t(f.d) * size_t(A.totRows);
            unsigned* ctr = A.gsCtr + 4 * f.c + 2 * f.d;
            if (f.e && f.f)
                gs_grid_body<TA, true, true, POS>(f.a, f.b, A.maxL, f.d, A.rowLv, A.lv, A.gsRows, A.wave, A.rp, A.ci, A.val, A.diag, A.C.b, A.C.x,
                                                  flag, ctr, ks, err);
            else if (f.e)
                gs_grid_body<TA, true, false, POS>(f.a, f.b, A.maxL, f.d, A.rowLv, A.lv, A.gsRows, A.wave, A.rp, A.ci, A.val, A.diag, A.C.b,
                                                   A.C.x, flag, ctr, ks, err);
            else
                gs_grid_body<TA, false, false, POS>(f.a, f.b, A.maxL, f.d, A.rowLv, A.lv, A.gsRows, A.wave, A.rp, A.ci, A.val, A.diag, A.C.b,
                                                    A.C.x, flag, ctr, ks, err);
            break;
        }
        case VP_RESID:
            gcpr_resid_body<TA>(f.a, f.b, A.maxL, A.rowLv, A.lv, A.rp, A.ci, A.val, A.C.b, A.C.x, A.C.r, ks);
            break;
        case VP_RESTRICT:
            gcpr_restrict_body<TA>(f.a, f.b, A.maxL, A.rowLv, A.lv, A.C.memPtr, A.C.mem, A.C.b, A.C.r, ks);
            break;
        case VP_COARSE:
            gcpr_coarse_body<TA>(A.C, ks, A.nsys, A.coarseChunks);
            break;
        case VP_PROLONG:
            gcpr_prolong_body<TA>(f.a, f.b, A.maxL, A.rowLv, A.lv, A.agg, A.C.x, ks);
            break;
        case VP_TSP:
            gcpr_tsp_body<TA, TT>(A.n, A.rowSys, A.sysRow0, A.maxL, A.lv, A.Lslot, A.Uslot, A.LovCol, A.UovCol, A.C.sp, A.C.spLov, A.C.spUov,
                                  A.C.x, A.T, ks);
            break;
        default:
            break;
        }
        if (i + 1 < nph) grid_barrier(bar, target, err);
    }
}

// split form, second stage: the BILU0 sweeps of one system per thread block on t, z_p += xp as z is written (the
// tail of k_cpr_cta)
template <class TF, class TV, class TA, int NT = cta_threads<TF, TV>()>
__global__ void __launch_bounds__(NT) k_cpr2_cta(IluArgs<TF> F, int maxL, const AmgSysLv* __restrict__ lv, const TA* x, const TV* T,
                                                 double* z, TV* yglob, size_t smemBytes, const KScal* ks) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int s = blockIdx.x, tid = int(threadIdx.x), nt = int(blockDim.x);
    if (ks && ks[s].status != ST_RUNNING) return;
    const int row0 = __ldg(F.sysRow0 + s), ns = __ldg(F.sysRow0 + s + 1) - row0;
    const TA* xpg = x + __ldg(&lv[s * maxL].rowOff);
    const bool onchip = size_t(ns) * 3 * sizeof(TV) <= smemBytes;
    TV* y = onchip ? reinterpret_cast<TV*>(smraw) : yglob + size_t(row0) * 3;
    const int l0 = __ldg(F.sysLvl0 + s), nl = __ldg(F.sysLvl0 + s + 1) - l0 - 1;
    __shared__ int lvc[kLvCache];
    const int* ls = level_starts(F.lvlStart + l0, nl, lvc);
    // FP32 factors at 256 threads: three register buffers (rows loaded two levels ahead); at 512 threads (every row of a
    // wide level has its own thread) the two-buffer sweep, whose registers fit the smaller per-thread budget. With FP32
    // factors, vector and correction and room beside the vector, the records staged by cp.async instead.
    constexpr bool three = sizeof(TF) == 4 && NT <= 256;
    if constexpr (sizeof(TF) == 4 && sizeof(TV) == 4 && sizeof(TA) == 4) {
        const size_t vec = (size_t(ns) * 3 * sizeof(TV) + 15) & ~size_t(15);
        if (onchip && vec + size_t(kStageWords) * size_t(NT < kStageSlots ? NT : kStageSlots) * 4 <= smemBytes) {
            ilu_body_async<TA>(F, row0, ls, nl, T, z, y, xpg, reinterpret_cast<unsigned*>(smraw + vec));
            return;
        }
    }
    if (onchip || sizeof(TV) != sizeof(double)) {
        if constexpr (three) ilu_body3<TF, TV, TV, true, TA>(F, row0, ls, nl, T, z, y, true, xpg);
        else ilu_body<TF, TV, TV, IN_PLAIN, true, TA, NT>(F, row0, ls, nl, T, nullptr, nullptr, z, y, true, 0, 0, 0, xpg);
    } else {
        if constexpr (three) ilu_body3<TF, TV, TV, false, TA>(F, row0, ls, nl, T, z, y, false, (const TA*)nullptr);
        else ilu_body<TF, TV, TV, IN_PLAIN, false, TA, NT>(F, row0, ls, nl, T, nullptr, nullptr, z, y, false, 0, 0, 0, nullptr);
        for (int k = row0 + tid; k < row0 + ns; k += nt) z[size_t(k) * 3] = da(z[size_t(k) * 3], double(xpg[k - row0]));
    }
}

// second stage of the split form: TF = TA (FP64 factors in the FP64 form, FP32 otherwise), TV = TT; 128, 256 or 512
// threads per system (every row is swept by one thread in the same arithmetic either way)
template <class TF, class TV, class TA, int NT>
void launch_cpr2_nt(const DevPlan& P, const PrecDev& M, const DevAmg& G, const CprArgs<TA>& C, const TV* T, double* z, TV* yglob,
                    const KScal* ks, cudaStream_t st) {
    IluArgs<TF> F;
    if constexpr (sizeof(TF) == 8) F = ilu_args(P, M.s64);
    else F = ilu_args(P, M.s32);
    // FP32 records, vector and correction: room for the cp.async stage beside the largest system's vector when it fits
    size_t sm = M.smem;
    if constexpr (sizeof(TF) == 4 && sizeof(TV) == 4 && sizeof(TA) == 4) {
        const size_t vec = (size_t(P.maxSysRows) * 3 * sizeof(TV) + 15) & ~size_t(15);
        const size_t want = vec + size_t(kStageWords) * size_t(NT < kStageSlots ? NT : kStageSlots) * 4;
        if (want <= size_t(max_smem_optin()) - kCtaStaticSmem) sm = std::max(sm, want);
    }
    raise_smem_limit(reinterpret_cast<const void*>(k_cpr2_cta<TF, TV, TA, NT>), int(sm));
    k_cpr2_cta<TF, TV, TA, NT><<<P.nsys, NT, sm, st>>>(F, G.maxL, G.lv, C.x, T, z, yglob, sm, ks);
}
template <class TA, class TT>
void launch_cpr2(const DevPlan& P, const PrecDev& M, const DevAmg& G, const CprArgs<TA>& C, TT* Tsplit, double* z, const KScal* ks,
                 cudaStream_t st) {
    const int nt = M.cpr2Threads;
    if constexpr (sizeof(TA) == 8) {
        if (nt >= 512) launch_cpr2_nt<double, double, TA, 512>(P, M, G, C, Tsplit, z, z, ks, st);
        else if (nt <= 128) launch_cpr2_nt<double, double, TA, 128>(P, M, G, C, Tsplit, z, z, ks, st);
        else launch_cpr2_nt<double, double, TA, 256>(P, M, G, C, Tsplit, z, z, ks, st);
    } else if constexpr (sizeof(TT) == 8) {
        if (nt >= 512) launch_cpr2_nt<float, double, TA, 512>(P, M, G, C, Tsplit, z, z, ks, st);
        else if (nt <= 128) launch_cpr2_nt<float, double, TA, 128>(P, M, G, C, Tsplit, z, z, ks, st);
        else launch_cpr2_nt<float, double, TA, 256>(P, M, G, C, Tsplit, z, z, ks, st);
    } else {
        if (nt >= 512) launch_cpr2_nt<float, float, TA, 512>(P, M, G, C, Tsplit, z, M.y32, ks, st);
        else if (nt <= 128) launch_cpr2_nt<float, float, TA, 128>(P, M, G, C, Tsplit, z, M.y32, ks, st);
        else launch_cpr2_nt<float, float, TA, 256>(P, M, G, C, Tsplit, z, M.y32, ks, st);
    }
}

// the fused V-cycle as one cooperative launch: as many blocks as can be resident at once (queried once per kernel)
template <class TA, class TT, bool POS>
void launch_vcycle(const DevAmg& G, const VcArgs<TA, TT>& A, int mode, const KScal* ks, int* err, cudaStream_t st) {
    static int perSm[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    int& nb = perSm[dev & 63];
    if (nb == 0) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_vcycle<TA, TT, POS>, 256, 0);
        nb = b > 0 ? b : 1;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(nb * device_sm_count()));
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_vcycle<TA, TT, POS>, (const VPhase*)G.phases, G.nPhases, mode, A, ks, G.vbar, err);
}

template <class TA, class TT>
int cpr_grid(const DevPlan& P, const PrecDev& M, const DevAmg& G, const CprArgs<TA>& C, const TA* val, int mode, const double* r,
             double* pv, const double* v, double* z, const KScal* ks, SweepState& S, int* err, cudaStream_t st) {
    const int n = P.n, gn = grid_for(n, 256);
    int launches = 0;
    // the split form keeps t in the second stage's sweep type (TT: FP32 in the all-FP32 form), as the thread-block
    // kernel does
    TT* Tsplit = reinterpret_cast<TT*>(G.T);
    if (M.split && M.vform == 1 && G.nPhases > 0) {
        // the whole pass sequence (input .. t) as the phases of one cooperative launch, then the BILU0 stage
        VcArgs<TA, TT> A{C, n, P.nsys, G.maxL, G.totRows, P.rowSys, P.sysRow0, r, v, pv, Tsplit, G.rowLv, G.gsRows, G.wave, G.rp, G.ci,
                         G.diag, G.gci, G.agg, G.lv, G.cdesc, val, G.gsFlag, G.gsCtr, P.Lslot, P.Uslot, P.LovCol, P.UovCol,
                         G.coarseChunks};
        cudaMemsetAsync(G.vbar, 0, sizeof(unsigned), st);
        if (G.posOrder) launch_vcycle<TA, TT, true>(G, A, mode, ks, err, st);
        else launch_vcycle<TA, TT, false>(G, A, mode, ks, err, st);
        launches += 1;
        launch_cpr2<TA, TT>(P, M, G, C, Tsplit, z, ks, st);
        return launches + 1;
    }
    if (M.split) {
        if (mode == IN_PUPDATE) k_gcpr_in<IN_PUPDATE, TA, TT, TT><<<gn, 256, 0, st>>>(n, P.rowSys, r, pv, v, G.w, Tsplit, C.b, ks);
        else if (mode == IN_SUPDATE) k_gcpr_in<IN_SUPDATE, TA, TT, TT><<<gn, 256, 0, st>>>(n, P.rowSys, r, pv, v, G.w, Tsplit, C.b, ks);
        else k_gcpr_in<IN_PLAIN, TA, TT, TT><<<gn, 256, 0, st>>>(n, P.rowSys, r, pv, v, G.w, Tsplit, C.b, ks);
    } else {
        if (mode == IN_PUPDATE) k_gcpr_in<IN_PUPDATE, TA, TT, double><<<gn, 256, 0, st>>>(n, P.rowSys, r, pv, v, G.w, G.T, C.b, ks);
        else if (mode == IN_SUPDATE) k_gcpr_in<IN_SUPDATE, TA, TT, double><<<gn, 256, 0, st>>>(n, P.rowSys, r, pv, v, G.w, G.T, C.b, ks);
        else k_gcpr_in<IN_PLAIN, TA, TT, double><<<gn, 256, 0, st>>>(n, P.rowSys, r, pv, v, G.w, G.T, C.b, ks);
    }
    ++launches;
    const auto& LB = G.levelRowBeg;
    auto sweep = [&](int l, int phase, bool fwd, bool zero) {
        const std::vector<int>& cb = G.colBeg[size_t(l)];
        if (phase == 0 && cb.size() > 1) {                 // multicolour: a parallel pass per large colour, the small ones in one block
            const int nc = int(cb.size()) - 1, tail = G.colTail[size_t(l)];
            auto big = [&](int c) {
                const int i0 = cb[size_t(c)], i1 = cb[size_t(c) + 1];
                if (zero)
                    k_gs_colour<TA, true><<<grid_for(i1 - i0, 256), 256, 0, st>>>(i0, i1, G.maxL, G.cdesc, G.gci, val, G.wave, G.rowLv, C.b,
                                                                                 C.x, ks);
                else
                    k_gs_colour<TA, false><<<grid_for(i1 - i0, 256), 256, 0, st>>>(i0, i1, G.maxL, G.cdesc, G.gci, val, G.wave, G.rowLv,
                                                                                  C.b, C.x, ks);
                ++launches;
            };
            auto small = [&]() {
                if (tail >= nc) return;
                const int i0 = cb[size_t(tail)], i1 = cb[size_t(nc)];
                const int g = std::max(1, std::min(G.gsBlocks[size_t(l)], (i1 - i0 + kGridThreads / 32 - 1) / (kGridThreads / 32)));
                int* flag = G.gsFlag;                               // phase-0 flags: unused otherwise on multicolour levels
                unsigned* ctr = G.gsCtr + 4 * l;
                if (fwd && zero)
                    k_gs_tail<TA, true, true><<<g, kGridThreads, 0, st>>>(i0, i1, tail, G.maxL, G.cdesc, G.gci, val, G.wave, G.rowLv, C.b,
                                                                          C.x, flag, ctr, ks, err);
                else if (fwd)
                    k_gs_tail<TA, true, false><<<g, kGridThreads, 0, st>>>(i0, i1, tail, G.maxL, G.cdesc, G.gci, val, G.wave, G.rowLv, C.b,
                                                                           C.x, flag, ctr, ks, err);
                else
                    k_gs_tail<TA, false, false><<<g, kGridThreads, 0, st>>>(i0, i1, tail, G.maxL, G.cdesc, G.gci, val, G.wave, G.rowLv,
                                                                            C.b, C.x, flag, ctr, ks, err);
                ++launches;
            };
            if (fwd) {
                for (int c = 0; c < tail; ++c) big(c);
                small();
            } else {
                small();
                for (int c = tail - 1; c >= 0; --c) big(c);
            }
            return;
        }
        const int q0 = LB[size_t(l)], q1 = LB[size_t(l) + 1];
        int* flag = G.gsFlag + size_t(phase) * size_t(G.totRows);
        unsigned* ctr = G.gsCtr + 4 * l + 2 * phase;
        const int g = G.gsBlocks[size_t(l)];
        auto go = [&](auto pos) {
            constexpr bool POS = decltype(pos)::value;
            if (fwd && zero)
                k_gs_grid<TA, true, true, POS><<<g, kGridThreads, 0, st>>>(q0, q1, G.maxL, phase, G.rowLv, G.lv, G.gsRows, G.wave, G.rp,
                                                                            G.ci, val, G.diag, C.b, C.x, flag, ctr, ks, err);
            else if (fwd)
                k_gs_grid<TA, true, false, POS><<<g, kGridThreads, 0, st>>>(q0, q1, G.maxL, phase, G.rowLv, G.lv, G.gsRows, G.wave, G.rp,
                                                                             G.ci, val, G.diag, C.b, C.x, flag, ctr, ks, err);
            else
                k_gs_grid<TA, false, false, POS><<<g, kGridThreads, 0, st>>>(q0, q1, G.maxL, phase, G.rowLv, G.lv, G.gsRows, G.wave, G.rp,
                                                                              G.ci, val, G.diag, C.b, C.x, flag, ctr, ks, err);
        };
        if (G.posOrder) go(std::true_type());
        else go(std::false_type());
        ++launches;
    };
    // form 3 (split only): the levels below the finest in one launch, a thread block per system
    const bool lo = M.split && M.vform == 3;
    const int lTop = lo ? std::min(1, G.maxL - 1) : G.maxL - 1;   // levels smoothed by grid passes: [0, lTop)
    for (int l = 0; l < lTop; ++l) {                       // pre-smoothing and restriction, finest to coarsest
        sweep(l, 0, true, true);
        const int f0 = LB[size_t(l)], f1 = LB[size_t(l) + 1], c0 = LB[size_t(l) + 1], c1 = LB[size_t(l) + 2];
        k_gcpr_resid<TA><<<grid_for(f1 - f0, 256), 256, 0, st>>>(f0, f1, G.maxL, G.rowLv, G.lv, G.rp, G.ci, val, C.b, C.x, C.r, ks);
        k_gcpr_restrict<TA><<<grid_for(c1 - c0, 256), 256, 0, st>>>(c0, c1, G.maxL, G.rowLv, G.lv, G.memPtr, G.mem, C.b, C.r, ks);
        launches += 2;
    }
    if (lo) {
        // the on-chip vectors of the largest system's coarse levels, if they fit (no more: the rest is L1)
        const size_t want = size_t(G.maxSysLoRows) * 3 * sizeof(TA);
        const size_t sm = want <= size_t(max_smem_optin()) - kCtaStaticSmem ? want : 0;
        raise_smem_limit(reinterpret_cast<const void*>(k_vcycle_lo<TA, 256>), int(sm));
        k_vcycle_lo<TA, 256><<<G.nsys, 256, sm, st>>>(C, ks, sm);
        ++launches;
    } else {
        k_gcpr_coarse<TA><<<G.nsys, 256, 0, st>>>(C, ks);
        ++launches;
        for (int l : G.coarseGsLevels)                     // coarsest levels without dense LU (amg.cpp:313-315)
            for (int it = 0; it < 20; ++it) {
                sweep(l, 1, true, false);
                sweep(l, 1, false, false);
            }
    }
    for (int l = lTop - 1; l >= 0; --l) {                  // prolongation and post-smoothing, coarsest to finest
        const int q0 = LB[size_t(l)], q1 = LB[size_t(l) + 1];
        k_gcpr_prolong<TA><<<grid_for(q1 - q0, 256), 256, 0, st>>>(q0, q1, G.maxL, G.rowLv, G.lv, G.agg, C.x, ks);
        ++launches;
        sweep(l, 0, false, false);
    }
    if (M.split) {
        k_gcpr_tsp<TA, TT><<<gn, 256, 0, st>>>(n, P.rowSys, P.sysRow0, G.maxL, G.lv, P.Lslot, P.Uslot, P.LovCol, P.UovCol, C.sp, C.spLov,
                                              C.spUov, C.x, Tsplit, ks);
        launch_cpr2<TA, TT>(P, M, G, C, Tsplit, z, ks, st);
        return launches + 2;
    }
    k_gcpr_t<TA, TT><<<gn, 256, 0, st>>>(n, P.rowSys, P.rowPtr, P.col, M.val, C.x, G.T, ks);
    launch_ilu_grid_ks(P, M, G.T, z, ks, S, err, st);
    k_gcpr_zp<TA><<<gn, 256, 0, st>>>(n, P.rowSys, C.x, z, ks);
    return launches + 4;
}

}  // namespace

void vcycle_phases(const DevAmg& G, std::vector<VPhase>& out) {
    out.clear();
    if (!G.coarseGsLevels.empty() || G.maxL < 1) return;        // coarsest levels smoothed 20 times: separate launches
    const auto& LB = G.levelRowBeg;
    out.push_back(VPhase{VP_IN, 0, 0, 0, 0, 0, 0, 0});
    auto sweep = [&](int l, bool fwd, bool zero) {
        const std::vector<int>& cb = G.colBeg[size_t(l)];
        if (cb.size() > 1) {                                  // multicolour: large colours one phase each, the tail in one
            const int nc = int(cb.size()) - 1, tail = G.colTail[size_t(l)];
            auto big = [&](int c) { out.push_back(VPhase{VP_COLOUR, cb[size_t(c)], cb[size_t(c) + 1], zero ? 1 : 0, 0, 0, 0, 0}); };
            auto small = [&]() {
                if (tail < nc) out.push_back(VPhase{VP_TAIL, cb[size_t(tail)], cb[size_t(nc)], tail, l, fwd ? 1 : 0, zero ? 1 : 0, 0});
            };
            if (fwd) {
                for (int c = 0; c < tail; ++c) big(c);
                small();
            } else {
                small();
                for (int c = tail - 1; c >= 0; --c) big(c);
            }
        } else {
            out.push_back(VPhase{VP_GSGRID, LB[size_t(l)], LB[size_t(l) + 1], l, 0, fwd ? 1 : 0, zero ? 1 : 0, 0});
        }
    };
    for (int l = 0; l + 1 < G.maxL; ++l) {
        sweep(l, true, true);
        out.push_back(VPhase{VP_RESID, LB[size_t(l)], LB[size_t(l) + 1], 0, 0, 0, 0, 0});
        out.push_back(VPhase{VP_RESTRICT, LB[size_t(l) + 1], LB[size_t(l) + 2], 0, 0, 0, 0, 0});
    }
    out.push_back(VPhase{VP_COARSE, 0, 0, 0, 0, 0, 0, 0});
    for (int l = G.maxL - 2; l >= 0; --l) {
        out.push_back(VPhase{VP_PROLONG, LB[size_t(l)], LB[size_t(l) + 1], 0, 0, 0, 0, 0});
        sweep(l, false, false);
    }
    out.push_back(VPhase{VP_TSP, 0, 0, 0, 0, 0, 0, 0});
}

int launch_cpr_grid(const DevPlan& P, const PrecDev& M, const DevAmg& G, int mode, const double* r, double* pv, const double* v,
                    double* z, const KScal* ks, SweepState& S, int* err, cudaStream_t st) {
    if (M.kind == 0) {
        const CprArgs<double> C = cpr_args<double>(G, G.val, G.slotVal, G.diagVal, G.lu, G.x, G.b, G.r, G.sp, G.spLov, G.spUov);
        return cpr_grid<double, double>(P, M, G, C, G.val, mode, r, pv, v, z, ks, S, err, st);
    }
    const CprArgs<float> C = cpr_args<float>(G, G.valf, G.slotValf, G.diagValf, G.luf, G.xf, G.bf, G.rf, G.spf, G.spLovf, G.spUovf);
    if (M.kind == 1) return cpr_grid<float, double>(P, M, G, C, G.valf, mode, r, pv, v, z, ks, S, err, st);
    return cpr_grid<float, float>(P, M, G, C, G.valf, mode, r, pv, v, z, ks, S, err, st);
}

}  // namespace rsg
