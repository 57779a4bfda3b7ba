// Shared helpers for the sm_103a MPS kernels: complex64 arithmetic, error
// reporting and launch checks.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>
#include <string>

#include "../../include/mpsim_gb300.h"

namespace mps {

typedef float2 cf;

__host__ __device__ __forceinline__ cf cmake(float r, float i) { return make_float2(r, i); }
__host__ __device__ __forceinline__ cf cadd(cf a, cf b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ cf csub(cf a, cf b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ cf cmul(cf a, cf b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ cf cconj(cf a) { return make_float2(a.x, -a.y); }
__host__ __device__ __forceinline__ cf cscale(cf a, float s) { return make_float2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ float cabs2(cf a) { return a.x * a.x + a.y * a.y; }
// acc += a * b
__host__ __device__ __forceinline__ void cfma(cf& acc, cf a, cf b) {
    acc.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x));
    acc.y = fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y));
}
// acc += conj(a) * b
__host__ __device__ __forceinline__ void cfma_conj(cf& acc, cf a, cf b) {
    acc.x = fmaf(a.x, b.x, fmaf(a.y, b.y, acc.x));
    acc.y = fmaf(a.x, b.y, fmaf(-a.y, b.x, acc.y));
}

// Shared-memory mbarrier (CTA scope): init with an arrival count, arrive
// (release), and a bounded try_wait on a phase parity (acquire) that suspends
// the calling thread for up to about suspend_ns while the phase is open.
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(a)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity, unsigned suspend_ns) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity), "r"(suspend_ns)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Circle-method round-robin: nplayers (even) players, round r in
// [0, nplayers-1), pair p in [0, nplayers/2).  Every unordered pair meets
// exactly once per nplayers-1 rounds and the pairs of one round are disjoint.
__host__ __device__ __forceinline__ void tournament_pair(int nplayers, int r, int p,
                                                         int& i, int& j) {
    const int m = nplayers - 1;
    if (p == 0) {
        i = r % m;
        j = m;
    } else {
        i = (r + p) % m;
        j = (r - p + m) % m;
    }
    if (i > j) { int t = i; i = j; j = t; }
}

void set_error(const std::string& msg);
void count_launch();
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define MPS_CUDA_CHECK(call)                                        \
    do {                                                            \
        cudaError_t _e = (call);                                    \
        if (_e != cudaSuccess) return ::mps::cuda_fail(_e, #call);  \
    } while (0)

#define MPS_LAUNCH_CHECK(name)                                      \
    do {                                                            \
        ::mps::count_launch();                                      \
        cudaError_t _e = cudaGetLastError();                        \
        if (_e != cudaSuccess) return ::mps::cuda_fail(_e, name);   \
    } while (0)

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Devices a process may use with this library (per-device one-time setup).
constexpr int kMaxDevices = 64;

// One-time setup of a kernel on each device: the dynamic shared-memory
// opt-in (cudaFuncAttributeMaxDynamicSharedMemorySize) is a per-device
// attribute, and resident-CTA counts depend on the device.
struct KernelSetup {
    std::once_flag once[kMaxDevices];
    int rc[kMaxDevices];
    int limit[kMaxDevices];   // largest dynamic shared memory the kernel may request
    int ctas[kMaxDevices];    // resident CTAs on the whole device (where computed)
};

}  // namespace mps
