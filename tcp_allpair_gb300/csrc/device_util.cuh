// device_util.cuh -- PTX helpers shared by the kernels of libtcpgpu.so:
// mbarrier + cp.async.bulk (bulk-copy engine) staging with bounded waits,
// SFU approximations, compensated FP32 sums and block reductions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace tcp {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make mbarrier initialisation visible to the async (bulk-copy) proxy
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Bulk global->shared copy completing on `bar`.  dst, src 16-byte aligned,
// bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for phase `parity` of `bar`, giving up after `limit` clock cycles
// (returns false then).  A legitimate wait here is a few microseconds.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, long long limit) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > limit) return false;
    }
    return true;
}

constexpr long long kWaitLimitCycles = 4000000000LL;  // ~2 s at 2 GHz

// ---- SFU approximations (one MUFU op each) ---------------------------------
__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// ---- fixed-point coordinates ------------------------------------------------
// 2^32 units per box length (iL = 1/L, computed once on the host); the int32
// difference of two coordinates is the minimum-image separation.  Every
// entry point quantises positions through this function, so that they all
// see the same grid.
// x - L DNINT(x/L) (vverlet.f90:153); x/L from the reciprocal with one FMA
// correction (the quotient to within rounding of the divided value): GB300's
// FP64 division costs dozens of FP64 operations
__device__ __forceinline__ double wrap_box(double x, double L, double iL) {
    double q = x * iL;
    q = fma(fma(-q, L, x), iL, q);
    return x - L * round(q);
}

__device__ __forceinline__ int fixed_coord(double x, double iL) {
    double t = fma(x, iL, 0.5);
    t -= floor(t);
    const unsigned long long u = (unsigned long long)llrint(t * 4294967296.0);
    return (int)(unsigned)(u & 0xffffffffull);
}

// 2^64 units per box length (the FP64 Newton-3 kernel): the wrapped int64
// difference is the minimum image, exact before its conversion to FP64.
__device__ __forceinline__ long long fixed_coord64(double x, double iL) {
    double t = fma(x, iL, 0.5);
    t -= floor(t);                                  // [0, 1)
    const double s = t * 18446744073709551616.0;    // [0, 2^64]
    const unsigned long long u = s >= 18446744073709551615.0 ? 0ull : (unsigned long long)s;
    return (long long)u;
}

// ---- compensated FP32 sums -------------------------------------------------
// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    float bp = s - a;
    float ap = s - bp;
    e = (a - ap) + (b - bp);
}

// (hi, lo) += v
__device__ __forceinline__ void acc2(float &hi, float &lo, float v) {
    float s, e;
    two_sum(hi, v, s, e);
    hi = s;
    lo += e;
}

// ---- reductions ------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the block (blockDim.x a multiple of 32, <= 1024); result valid in
// thread 0.  `sh` needs 32 doubles.
__device__ __forceinline__ double block_sum(double v, double *sh) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

}  // namespace tcp
