// Synchronisation helpers of the sync-free (flag-driven) kernels, shared by the device translation units
// (internal linkage in each): release stores and relaxed polls of per-row flags at GPU scope with one acquire
// fence per row, the bounded waits, and the warp's claim of 32 consecutive positions from an atomic counter.
#pragma once
#include <cuda_runtime.h>

#include "rsg_impl.h"

namespace rsg {
namespace {

constexpr unsigned kSpinLimit = 1u << 22;   // x up to 256 ns back-off: about one second per wait

__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void fence_acquire() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// Wait until flag[idx(q)] == want for every q in [q0, q1) with need(q), then one acquire fence. A row's
// dependencies are polled four at a time, and every poll round re-issues the loads of all those still pending
// together (relaxed loads, in flight at once): a round costs one memory round trip however many are pending.
// Bounded: a short busy phase, then back-off up to 256 ns; on time-out ERR_TIMEOUT is set and the wait ends.
template <class Idx, class Need>
__device__ __forceinline__ void wait_deps(const int* flag, int q0, int q1, int want, int* err, Idx idx, Need need) {
    for (int q = q0; q < q1; q += 4) {
        int k[4];
        unsigned pending = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            k[u] = (q + u < q1 && need(q + u)) ? idx(q + u) : -1;
            if (k[u] >= 0) pending |= 1u << u;
        }
        unsigned ns = 0;
        for (unsigned it = 0; pending; ++it) {
            int v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) v[u] = (pending >> u) & 1u ? ld_relaxed(flag + k[u]) : want;
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (v[u] == want) pending &= ~(1u << u);
            if (!pending) break;
            if (it >= 64) {
                __nanosleep(ns);
                ns = ns < 32 ? 32 : (ns < 256 ? 2 * ns : 256);
                if (it >= 64 + kSpinLimit) { atomicOr(err, ERR_TIMEOUT); break; }
                if ((it & 255u) == 255u && *(volatile int*)err != 0) break;   // another wait already gave up
            }
        }
    }
    fence_acquire();
}
// the common case: the dependencies are the columns col[p0 .. p1)
__device__ __forceinline__ void wait_cols(const int* flag, const int* __restrict__ col, int p0, int p1, int want, int* err) {
    wait_deps(flag, p0, p1, want, err, [&](int p) { return __ldg(col + p); }, [](int) { return true; });
}
__device__ __forceinline__ int warp_claim(unsigned* ctr) {
    unsigned base = 0;
    if ((threadIdx.x & 31) == 0) base = atomicAdd(ctr, 32u);
    return int(__shfl_sync(0xffffffffu, base, 0));
}

}  // namespace
}  // namespace rsg
