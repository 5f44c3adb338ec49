// Common device/host helpers of libkoregpu: complex arithmetic on float2/double2,
// the bounded grid barrier used by the persistent kernels, status plumbing and
// launch accounting.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <atomic>

#include "kore_gpu.h"

// ----------------------------------------------------------------------------- complex
template <typename C> struct real_of;
template <> struct real_of<double2> { using type = double; };
template <> struct real_of<float2>  { using type = float;  };

__host__ __device__ __forceinline__ double2 mk(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ float2  mkf(float r, float i)  { return make_float2(r, i); }

template <typename C> __host__ __device__ __forceinline__ C czero();
template <> __host__ __device__ __forceinline__ double2 czero<double2>() { return make_double2(0.0, 0.0); }
template <> __host__ __device__ __forceinline__ float2  czero<float2>()  { return make_float2(0.f, 0.f); }

template <typename C> __host__ __device__ __forceinline__ C cone();
template <> __host__ __device__ __forceinline__ double2 cone<double2>() { return make_double2(1.0, 0.0); }
template <> __host__ __device__ __forceinline__ float2  cone<float2>()  { return make_float2(1.f, 0.f); }

#define KORE_CPLX_OPS(C, R)                                                                 \
    __host__ __device__ __forceinline__ C operator+(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; } \
    __host__ __device__ __forceinline__ C operator-(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; } \
    __host__ __device__ __forceinline__ C operator-(C a) { C r; r.x = -a.x; r.y = -a.y; return r; }                 \
    __host__ __device__ __forceinline__ C operator*(C a, C b) {                             \
        C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r; }          \
    __host__ __device__ __forceinline__ C operator*(R s, C a) { C r; r.x = s * a.x; r.y = s * a.y; return r; }      \
    __host__ __device__ __forceinline__ C conjg(C a) { C r; r.x = a.x; r.y = -a.y; return r; }                      \
    __host__ __device__ __forceinline__ R abs2(C a) { return a.x * a.x + a.y * a.y; }       \
    /* a + b*c */                                                                           \
    __host__ __device__ __forceinline__ C cfma(C a, C b, C c) {                             \
        C r; r.x = fma(b.x, c.x, fma(-b.y, c.y, a.x)); r.y = fma(b.x, c.y, fma(b.y, c.x, a.y)); return r; } \
    /* a - b*c */                                                                           \
    __host__ __device__ __forceinline__ C cfms(C a, C b, C c) {                             \
        C r; r.x = fma(-b.x, c.x, fma(b.y, c.y, a.x)); r.y = fma(-b.x, c.y, fma(-b.y, c.x, a.y)); return r; } \
    /* a + conj(b)*c */                                                                     \
    __host__ __device__ __forceinline__ C cfmaconj(C a, C b, C c) {                         \
        C r; r.x = fma(b.x, c.x, fma(b.y, c.y, a.x)); r.y = fma(b.x, c.y, fma(-b.y, c.x, a.y)); return r; } \
    __host__ __device__ __forceinline__ C cdiv(C a, C b) {                                  \
        /* Smith's algorithm (scaled division, avoids overflow of |b|^2) */                 \
        C r; R s;                                                                           \
        if (fabs(b.x) >= fabs(b.y)) { R t = b.y / b.x; s = b.x + b.y * t;                   \
            r.x = (a.x + a.y * t) / s; r.y = (a.y - a.x * t) / s; }                         \
        else { R t = b.x / b.y; s = b.y + b.x * t;                                          \
            r.x = (a.x * t + a.y) / s; r.y = (a.y * t - a.x) / s; }                         \
        return r; }

KORE_CPLX_OPS(double2, double)
KORE_CPLX_OPS(float2, float)

__host__ __device__ __forceinline__ double2 to_c128(double2 a) { return a; }
__host__ __device__ __forceinline__ double2 to_c128(float2 a) { return make_double2(a.x, a.y); }
template <typename C> __host__ __device__ __forceinline__ C from_c128(double2 a);
template <> __host__ __device__ __forceinline__ double2 from_c128<double2>(double2 a) { return a; }
template <> __host__ __device__ __forceinline__ float2 from_c128<float2>(double2 a) {
    return make_float2((float)a.x, (float)a.y);
}

__device__ __forceinline__ double2 shfl_down(double2 v, int o) {
    v.x = __shfl_down_sync(0xffffffffu, v.x, o);
    v.y = __shfl_down_sync(0xffffffffu, v.y, o);
    return v;
}
__device__ __forceinline__ float2 shfl_down(float2 v, int o) {
    v.x = __shfl_down_sync(0xffffffffu, v.x, o);
    v.y = __shfl_down_sync(0xffffffffu, v.y, o);
    return v;
}
template <typename C> __device__ __forceinline__ C warp_sum(C v) {
    for (int o = 16; o > 0; o >>= 1) v = v + shfl_down(v, o);
    return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// ----------------------------------------------------------------------------- errors
// Device error flag values (plan->d_err); the first writer wins.
#define KORE_DEVERR_BARRIER 1   // a grid barrier wait ran out
#define KORE_DEVERR_PIVOT   2   // zero pivot in Gauss-Jordan
#define KORE_DEVERR_FLAG    3   // a dataflow flag wait ran out

// Iteration limit of every device spin-wait: ~2^26 polls with 64 ns sleeps is a few
// seconds, far above any legitimate wait, far below a watchdog.
#define KORE_SPIN_LIMIT (1u << 26)

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_relaxed_i32(const int *p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid-wide barrier for a cooperative (co-resident) launch.  `counter` is a
// monotonically increasing arrival count zeroed before the launch; episode e
// completes when counter reaches (e+1)*gridDim.x.  Every wait is bounded: on
// timeout the error flag is set and the barrier returns, and once the flag is set
// all later barriers return immediately so the kernel drains instead of hanging.
struct GridBarrier {
    unsigned *counter;
    int *err;
    unsigned target;
    __device__ __forceinline__ void init(unsigned *c, int *e) { counter = c; err = e; target = 0; }
    __device__ __forceinline__ void sync() {
        __syncthreads();
        target += gridDim.x;
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(counter, 1u);
            unsigned spins = 0;
            while (ld_acquire_u32(counter) < target) {
                if (ld_relaxed_i32(err) != 0) break;
                if (++spins > KORE_SPIN_LIMIT) { atomicCAS(err, 0, KORE_DEVERR_BARRIER); break; }
                __nanosleep(64);
            }
            __threadfence();
        }
        __syncthreads();
    }
};

// ----------------------------------------------------------------------------- host side
extern std::atomic<long long> g_kore_launches;

#define KORE_LAUNCHED(n) g_kore_launches.fetch_add((n), std::memory_order_relaxed)

#define KORE_CUDA_TRY(expr)                                                                 \
    do {                                                                                    \
        cudaError_t _e = (expr);                                                            \
        if (_e != cudaSuccess) {                                                            \
            std::fprintf(stderr, "kore: CUDA error %s at %s:%d: %s\n", cudaGetErrorName(_e), \
                         __FILE__, __LINE__, cudaGetErrorString(_e));                       \
            return (_e == cudaErrorMemoryAllocation) ? KORE_ENOMEM : KORE_ECUDA;            \
        }                                                                                   \
    } while (0)

#define KORE_TRY(expr)                                                                      \
    do { int _s = (expr); if (_s != KORE_OK) return _s; } while (0)

static inline unsigned kore_div_up(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// Let a kernel use the device's largest dynamic shared memory.  The attribute is
// process-wide, so every caller sets the same value: a plan of another size on another
// host thread cannot lower it between this thread's setting and its launch.
template <typename K>
int kore_allow_max_dyn_smem(K kern, int device) {
    cudaFuncAttributes fa;
    KORE_CUDA_TRY(cudaFuncGetAttributes(&fa, (const void *)kern));
    int optin = 0;
    KORE_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    KORE_CUDA_TRY(cudaFuncSetAttribute((const void *)kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       optin - (int)fa.sharedSizeBytes));
    return 0;
}
