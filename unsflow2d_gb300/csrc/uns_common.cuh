// uns_common.cuh -- shared plumbing of the UNSFlow2D GB300 library: status
// handling, the device error word, warp reductions and the bounded
// acquire/release flag waits of the dataflow LU-SGS sweeps.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "unsflow_types.h"

namespace uns {

// Last error message of the calling host thread (uns_last_error()).
void set_last_error(const std::string& s);

#define UNS_CUDA(call)                                                                         \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) {                                                               \
            ::uns::set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_));         \
            return UNS_ERR_CUDA;                                                               \
        }                                                                                      \
    } while (0)

// Device error word: [0] first error code, [1] index of the offending
// face/cell/node, [2] iteration (set by the iterate driver), [3] spare.
struct DevErr {
    int code, index, iter, spare;
};

__device__ __forceinline__ void set_err(DevErr* e, int code, int index) {
    if (atomicCAS(&e->code, 0, code) == 0) e->index = index;
}

constexpr int kBlock = 256;

inline int nblocks(long long n, int bs = kBlock) { return (int)((n + bs - 1) / bs); }

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Bound on every spin-wait in the library's kernels (~2 s at 2 GHz).
constexpr long long kWaitCycles = 4000000000LL;

// L2-coherent (L1-bypassing) 32-byte load / store for data that other SMs
// publish within the same kernel.
__device__ __forceinline__ double4 ldcg4(const double4* p) {
    const double2* q = reinterpret_cast<const double2*>(p);
    double2 a = __ldcg(q), b = __ldcg(q + 1);
    return make_double4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ void stcg4(double4* p, const double4& v) {
    double2* q = reinterpret_cast<double2*>(p);
    __stcg(q, make_double2(v.x, v.y));
    __stcg(q + 1, make_double2(v.z, v.w));
}

// Acquire / release accesses to per-node completion flags (dataflow sweeps).
__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" : : "l"(p), "r"(v) : "memory");
}

// Three-stage RK weights q = a*qold + b*(qc - dt/area*res), stage irk = 1..3
// (CCFVM/main.F90:39-44 airk/birk, the same weights in NCFVM/main.f90).
// Selected by branch, not by indexing a local table (which lands on the stack).
__device__ __forceinline__ double rk3_a(int irk) { return irk == 2 ? 3.0 / 4.0 : (irk == 3 ? 1.0 / 3.0 : 0.0); }
__device__ __forceinline__ double rk3_b(int irk) { return irk == 2 ? 1.0 / 4.0 : (irk == 3 ? 2.0 / 3.0 : 1.0); }

// Waits until *flag >= want.  Bounded: gives up after kWaitCycles (or as
// soon as another thread has recorded UNS_ERR_TIMEOUT) and records
// UNS_ERR_TIMEOUT, so no dataflow wait can hang the device.
__device__ __forceinline__ bool wait_flag(const int* flag, int want, DevErr* err) {
    if (ld_acquire(flag) >= want) return true;
    long long t0 = clock64();
    int spins = 0;
    while (ld_acquire(flag) < want) {
        if (*((volatile int*)&err->code) == UNS_ERR_TIMEOUT || clock64() - t0 > kWaitCycles) {
            set_err(err, UNS_ERR_TIMEOUT, -1);
            return false;
        }
        // Dependencies usually land within a microsecond: poll tightly first,
        // then back off so long waits leave issue slots to the producers.
        if (++spins > 64) __nanosleep(32);
    }
    return true;
}

}  // namespace uns
