// Device helpers shared by the kernels: exact-rounding arithmetic used on the parity path,
// acquire/release accessors for the decoupled look-back, and bounded spin-waits.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "qses_internal.h"

namespace qses {

// Spin-waits give up after this many polls and raise QSES_ERR_TIMEOUT in the error word.
constexpr unsigned kSpinLimit = 1u << 24;

// Voxel coordinate along one axis: origin + i * dx with one rounding (fma).  The CPU
// oracle computes fmaf((float)i, dx, o), so the two agree bit for bit.
__device__ __forceinline__ float vox(int i, float dx, float o) { return __fmaf_rn((float)i, dx, o); }

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void raise_error(int *err, int code) {
    if (err) atomicCAS(err, 0, code);
}

// Look-back status word: flag in the top two bits (0 = not ready, 1 = tile aggregate,
// 2 = inclusive prefix), payload below.
constexpr unsigned long long kFlagAgg = 1ull << 62;
constexpr unsigned long long kFlagPre = 2ull << 62;

// Polls a status word until its flag is non-zero.  Returns 0 (and raises the error) if
// the limit is reached; callers then treat the predecessor as contributing nothing and
// every scatter stays bounds-checked.
__device__ __forceinline__ unsigned long long wait_status(const unsigned long long *p, int *err) {
    for (unsigned it = 0; it < kSpinLimit; ++it) {
        unsigned long long s = ld_acquire(p);
        if (s >> 62) return s;
        if (it > 64) __nanosleep(32);
    }
    raise_error(err, QSES_ERR_TIMEOUT);
    return 0;
}

__device__ __forceinline__ uint2 add2(uint2 a, uint2 b) { return make_uint2(a.x + b.x, a.y + b.y); }

// Warp-inclusive scan of uint2 (both components).
__device__ __forceinline__ uint2 warp_incl_scan2(uint2 v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned a = __shfl_up_sync(0xffffffffu, v.x, o);
        unsigned b = __shfl_up_sync(0xffffffffu, v.y, o);
        if (lane >= o) { v.x += a; v.y += b; }
    }
    return v;
}

__device__ __forceinline__ unsigned warp_incl_scan(unsigned v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned a = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += a;
    }
    return v;
}

// Block-exclusive scan of uint2 for NT threads; smem holds NT/32 entries.
template <int NT>
__device__ __forceinline__ uint2 block_excl_scan2(uint2 v, uint2 &total, uint2 *smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint2 inc = warp_incl_scan2(v);
    if (lane == 31) smem[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint2 w = lane < NT / 32 ? smem[lane] : make_uint2(0, 0);
        w = warp_incl_scan2(w);
        if (lane < NT / 32) smem[lane] = w;
    }
    __syncthreads();
    uint2 pre = warp ? smem[warp - 1] : make_uint2(0, 0);
    total = smem[NT / 32 - 1];
    __syncthreads();
    return make_uint2(pre.x + inc.x - v.x, pre.y + inc.y - v.y);
}

template <int NT>
__device__ __forceinline__ unsigned block_excl_scan(unsigned v, unsigned &total, unsigned *smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned inc = warp_incl_scan(v);
    if (lane == 31) smem[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        unsigned w = lane < NT / 32 ? smem[lane] : 0u;
        w = warp_incl_scan(w);
        if (lane < NT / 32) smem[lane] = w;
    }
    __syncthreads();
    unsigned pre = warp ? smem[warp - 1] : 0u;
    total = smem[NT / 32 - 1];
    __syncthreads();
    return pre + inc - v;
}

}  // namespace qses
