// Allocation-free variant of the fused block SpMV + inner product: y = A x and <w, y>.
//
// It is the kernel of the solver's <r0, v> step (k_spmv_tile with its per-tile partial sums) with the scratch
// moved out of the caller's reach: the per-tile partials and the arrival counter of the last-tile reduction live
// in one file-scope device array, so a call needs no device allocation at all. The caller still owns the matrix,
// the vectors and the scalar result.
//
// The array is shared by every call on a device and keeps the previous call's contents; the entry point clears the
// arrival counter before each launch. Two calls whose work overlaps on the GPU (different streams, no ordering)
// race on the array and give wrong results: order them, or use the handle-based entry points.
#include "rsg.h"
#include "rsg_impl.h"

#include <cuda_runtime.h>

#include <mutex>
#include <string>

// The caller-visible bound: tiles of 256 block rows, at most RSG_NOALLOC_MAX_TILES of them.
#define RSG_NOALLOC_TILE_ROWS 256
#define RSG_NOALLOC_MAX_TILES 16384

// partial sums [0, MAX_TILES) followed by one 256-byte slot holding the arrival counter: 129 KiB per device
static __device__ __align__(256) double rsg_noalloc_scratch[RSG_NOALLOC_MAX_TILES + 32];

namespace rsg {
void set_last_error(const std::string& msg);
}

namespace {

constexpr int kThreads = 192;   // 64 block rows per pass, 3 threads per block row

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }

__global__ void __launch_bounds__(kThreads) k_spmv_dot_noalloc(int n, const int* __restrict__ rowPtr, const int* __restrict__ col,
                                                              const double* __restrict__ val, const double* __restrict__ x,
                                                              double* y, const double* __restrict__ w, double* dot, double* part,
                                                              unsigned* done, int ntiles) {
    __shared__ double sh[32];
    __shared__ int amLast;
    const int tile = blockIdx.x;
    const int r0 = tile * RSG_NOALLOC_TILE_ROWS;
    const int r1 = min(n, r0 + RSG_NOALLOC_TILE_ROWS);
    const int e = threadIdx.x % 3;
    double acc = 0;
    for (int row = r0 + int(threadIdx.x) / 3; row < r1; row += kThreads / 3) {
        double yv = 0;
        const int p1 = __ldg(rowPtr + row + 1);
        for (int p = __ldg(rowPtr + row); p < p1; ++p) {            // engine/src/bsr.cpp:109-117, reference order
            const double* a = val + size_t(p) * 9 + e * 3;
            const double* xc = x + size_t(__ldg(col + p)) * 3;
            yv = da(yv, da(da(dm(__ldg(a), __ldg(xc)), dm(__ldg(a + 1), __ldg(xc + 1))), dm(__ldg(a + 2), __ldg(xc + 2))));
        }
        const size_t q = size_t(row) * 3 + e;
        y[q] = yv;
        acc += __ldg(w + q) * yv;
    }
    // tile partial, then the last tile to arrive reduces all partials in a fixed order
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int k = 0; k < kThreads / 32; ++k) s += sh[k];
        part[tile] = s;
        __threadfence();
        amLast = atomicAdd(done, 1u) == unsigned(ntiles) - 1u;
    }
    __syncthreads();
    if (!amLast) return;
    __threadfence();
    double s = 0;
    for (int t = threadIdx.x; t < ntiles; t += kThreads) s += ((volatile double*)part)[t];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int k = 0; k < kThreads / 32; ++k) t += sh[k];
        *dot = t;
        *done = 0u;
    }
}

// device address of the scratch array, looked up once per device (host code cannot use the symbol itself). The
// address belongs to the device's context of the first call: after cudaDeviceReset the library's module is loaded
// again in a new context, and this cache would hand the kernel the old address, so a process that resets a device
// must not call this entry point on that device again.
std::mutex g_mu;
double* g_addr[64] = {nullptr};

int scratch_address(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { rsg::set_last_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e)); return RSG_ECUDA; }
    if (dev < 0 || dev >= 64) { rsg::set_last_error("device ordinal out of range for the no-alloc entry point"); return RSG_EINVAL; }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, rsg_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            rsg::set_last_error(std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(e));
            return RSG_ECUDA;
        }
        g_addr[dev] = static_cast<double*>(p);
    }
    *out = g_addr[dev];
    return RSG_OK;
}

}  // namespace

extern "C" int rsg_spmv_dot_noalloc(int n, int nb, const int* d_rowPtr, const int* d_col, const double* d_val, const double* d_x,
                                    double* d_y, const double* d_w, double* d_dot, void* stream) {
    if (nb != 3) { rsg::set_last_error("rsg_spmv_dot_noalloc: only nb = 3 is supported"); return RSG_EINVAL; }
    if (n < 1) { rsg::set_last_error("rsg_spmv_dot_noalloc: n must be >= 1"); return RSG_EINVAL; }
    const long long ntiles = (static_cast<long long>(n) + RSG_NOALLOC_TILE_ROWS - 1) / RSG_NOALLOC_TILE_ROWS;
    if (ntiles > RSG_NOALLOC_MAX_TILES) {
        rsg::set_last_error("rsg_spmv_dot_noalloc: n = " + std::to_string(n) + " block rows exceeds the maximum of " +
                            std::to_string(RSG_NOALLOC_MAX_TILES * RSG_NOALLOC_TILE_ROWS) + " of this entry point");
        return RSG_EINVAL;
    }
    if (!d_rowPtr || !d_col || !d_val || !d_x || !d_y || !d_w || !d_dot) {
        rsg::set_last_error("rsg_spmv_dot_noalloc: null pointer");
        return RSG_EINVAL;
    }
    if (d_x == d_y || d_w == d_y) {   // x and w are read through the read-only path while y is written
        rsg::set_last_error("rsg_spmv_dot_noalloc: d_y must not alias d_x or d_w");
        return RSG_EINVAL;
    }
    double* scratch = nullptr;
    const int rc = scratch_address(&scratch);
    if (rc != RSG_OK) return rc;
    unsigned* done = reinterpret_cast<unsigned*>(scratch + RSG_NOALLOC_MAX_TILES);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemsetAsync(done, 0, sizeof(unsigned), st);   // the counter must start at zero
    if (e != cudaSuccess) { rsg::set_last_error(std::string("cudaMemsetAsync: ") + cudaGetErrorString(e)); return RSG_ECUDA; }
    k_spmv_dot_noalloc<<<int(ntiles), kThreads, 0, st>>>(n, d_rowPtr, d_col, d_val, d_x, d_y, d_w, d_dot, scratch, done, int(ntiles));
    e = cudaGetLastError();
    if (e != cudaSuccess) { rsg::set_last_error(std::string("rsg_spmv_dot_noalloc launch: ") + cudaGetErrorString(e)); return RSG_ECUDA; }
    return RSG_OK;
}
