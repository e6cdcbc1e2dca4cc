// uns_common.cuh -- shared plumbing of the UNSFlow2D GB300 library: status
// handling, the device error word, warp reductions and the bounded record
// polls of the LU-SGS sweeps.
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

// 0.0 + x exactly as the FP64 addition rounds it (x itself; -0.0 becomes
// +0.0), on the integer pipe: the first term of a sum that starts from zero,
// one FP64 instruction less on a sweep item's dependent chain.
__device__ __forceinline__ double zero_plus(double x) {
    const long long b = __double_as_longlong(x);
    return __longlong_as_double(b == (long long)0x8000000000000000ULL ? 0LL : b);
}

// Default bound on every spin-wait in the library's kernels (~2 s at
// 2 GHz); a handle may set a shorter one (uns_*_set_wait_limit).
constexpr long long kWaitCycles = 4000000000LL;

// ---------------------------------------------------------------------------
// Sweep records.  Each LU-SGS sweep item publishes its values once, into
// slots pre-filled with kUnset: a signalling-NaN bit pattern, which no
// floating-point operation produces (IEEE 754 results are never signalling
// NaNs).  A consumer polls the slots themselves until none holds kUnset, so
// a value and its "ready" state travel together: the producer needs no
// release fence and the consumer no separate flag load.  Every slot is an
// aligned 64-bit word written exactly once per sweep, so a value that is not
// kUnset is final.
constexpr unsigned long long kUnset = 0x7FF40000DEAD0001ULL;

__device__ __forceinline__ bool is_unset(double x) {
    return (unsigned long long)__double_as_longlong(x) == kUnset;
}
__device__ __forceinline__ double2 ld_relaxed2(const double2* p) {
    double2 v;
    asm volatile("ld.relaxed.gpu.global.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed2(double2* p, double a, double b) {
    asm volatile("st.relaxed.gpu.global.v2.f64 [%0], {%1, %2};" : : "l"(p), "d"(a), "d"(b) : "memory");
}

// Bounded wait shared by the record polls: false (and UNS_ERR_TIMEOUT
// recorded) once `limit` cycles have passed or another thread has timed out.
// The shared error word is read every 64 spins only: every waiting warp of
// the GPU reading that one line on every spin slowed the NCFVM sweeps by
// about 1.6 % (measured); a thread still stops within 64 spins of another's
// timeout, and at its own limit in any case.
__device__ __forceinline__ bool poll_continue(int spins, long long& t0, DevErr* err, long long limit = kWaitCycles) {
    if (spins == 0) t0 = clock64();
    if (((spins & 63) == 63 && *((volatile int*)&err->code) == UNS_ERR_TIMEOUT) || clock64() - t0 > limit) {
        set_err(err, UNS_ERR_TIMEOUT, -1);
        return false;
    }
    if (spins > 64) __nanosleep(32);
    return true;
}

// Reads the 2 x 32-byte record (a, b) of a sweep item into out[0..8), all
// four loads in flight together, waiting (bounded) until none is kUnset.
__device__ __forceinline__ bool poll_record2(const double4* a, const double4* b, double out[8], DevErr* err,
                                             long long limit = kWaitCycles) {
    const double2* pa = reinterpret_cast<const double2*>(a);
    const double2* pb = reinterpret_cast<const double2*>(b);
    long long t0 = 0;
    for (int spins = 0;; ++spins) {
        double2 x0 = ld_relaxed2(pa), x1 = ld_relaxed2(pa + 1), x2 = ld_relaxed2(pb), x3 = ld_relaxed2(pb + 1);
        out[0] = x0.x; out[1] = x0.y; out[2] = x1.x; out[3] = x1.y;
        out[4] = x2.x; out[5] = x2.y; out[6] = x3.x; out[7] = x3.y;
        bool ready = true;
#pragma unroll
        for (int j = 0; j < 8; ++j) ready = ready && !is_unset(out[j]);
        if (ready) return true;
        if (!poll_continue(spins, t0, err, limit)) return false;
    }
}

// One published value, waiting (bounded) until it is not kUnset.
__device__ __forceinline__ bool poll_value(const double* p, double& out, DevErr* err, long long limit = kWaitCycles) {
    long long t0 = 0;
    for (int spins = 0;; ++spins) {
        asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(out) : "l"(p) : "memory");
        if (!is_unset(out)) return true;
        if (!poll_continue(spins, t0, err, limit)) return false;
    }
}

// FP32 records (mixed precision) use a signalling-NaN float pattern the same way.
constexpr unsigned kUnsetF = 0x7FA0DEADu;
__device__ __forceinline__ bool is_unset(float x) { return (unsigned)__float_as_int(x) == kUnsetF; }

// Reads a float4 record without waiting (an early look or one poll try).
__device__ __forceinline__ void peek_f4(const float4* a, float w[4]) {
    asm volatile("ld.relaxed.gpu.global.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(w[0]), "=f"(w[1]), "=f"(w[2]), "=f"(w[3]) : "l"(a) : "memory");
}

__device__ __forceinline__ bool set_f4(const float w[4]) {
    return !is_unset(w[0]) && !is_unset(w[1]) && !is_unset(w[2]) && !is_unset(w[3]);
}

// A float4 record, waiting (bounded) until none of its values is kUnsetF.
__device__ __forceinline__ bool poll_f4(const float4* a, float w[4], DevErr* err, long long limit = kWaitCycles) {
    long long t0 = 0;
    for (int spins = 0;; ++spins) {
        peek_f4(a, w);
        if (set_f4(w)) return true;
        if (!poll_continue(spins, t0, err, limit)) return false;
    }
}

// LU-SGS normal flux change F(q + dq) - F(q) along (nx, ny), component k, in
// FP32 and in delta form: from dq and q's state and primitives (fields rho,
// ru, rv, E, u, v, p, un = u.n, nx, ny of `e`), never as the difference of
// two O(1) fluxes, so its rounding error is relative to the change itself.
// F = ((E + p) u.n, rho u.n, rho u.n u + p nx, rho u.n v + p ny).
template <class Rec>
__device__ __forceinline__ float dflux_k(const Rec& e, float gm1, const float dq[4], int k) {
    const float dE = dq[0], dr = dq[1], dru = dq[2], drv = dq[3];
    const float rn = e.rho + dr;
    const float du = (dru - e.u * dr) / rn, dv = (drv - e.v * dr) / rn;
    const float u2 = e.u + du, v2 = e.v + dv;
    const float dp = gm1 * (dE - 0.5f * (dru * u2 + e.ru * du + drv * v2 + e.rv * dv));
    const float dun = du * e.nx + dv * e.ny;
    const float un2 = e.un + dun;
    const float df1 = dr * un2 + e.rho * dun;  // change of rho u.n
    const float run = e.rho * e.un;
    if (k == 0) return (dE + dp) * un2 + (e.E + e.p) * dun;
    if (k == 1) return df1;
    if (k == 2) return df1 * u2 + run * du + dp * e.nx;
    return df1 * v2 + run * dv + dp * e.ny;
}

// Publishes a mixed-form sweep record: lane 0 the FP32 dq (one float4
// slot), lane 1 the FP64 dq (two double2), as predicated stores of one
// instruction sequence; lane-divergent branches around the stores cost a
// sweep's critical path more than the stores themselves (measured).
__device__ __forceinline__ void publish_mixed(int lane, float4* a, double2* b, const float f[4], double d0, double d1,
                                              double d2, double d3) {
    const int p0 = lane == 0, p1 = lane == 1;
    asm volatile(
        "{\n\t.reg .pred q0, q1;\n\t"
        "setp.ne.s32 q0, %0, 0;\n\t"
        "setp.ne.s32 q1, %1, 0;\n\t"
        "@q0 st.relaxed.gpu.global.v4.f32 [%2], {%3, %4, %5, %6};\n\t"
        "@q1 st.relaxed.gpu.global.v2.f64 [%7], {%8, %9};\n\t"
        "@q1 st.relaxed.gpu.global.v2.f64 [%10], {%11, %12};\n\t}"
        :
        : "r"(p0), "r"(p1), "l"(a), "f"(f[0]), "f"(f[1]), "f"(f[2]), "f"(f[3]), "l"(b), "d"(d0), "d"(d1), "l"(b + 1),
          "d"(d2), "d"(d3)
        : "memory");
}

static __global__ void __launch_bounds__(kBlock) k_fill_unset_f(float4* p, long long n4) {
    const float u = __int_as_float((int)kUnsetF);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += (long long)gridDim.x * blockDim.x)
        p[i] = make_float4(u, u, u, u);
}

// Fills n doubles with kUnset (re-arms the records before a sweep).
static __global__ void __launch_bounds__(kBlock) k_fill_unset(double2* p, long long n2) {
    const double u = __longlong_as_double((long long)kUnset);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n2; i += (long long)gridDim.x * blockDim.x)
        p[i] = make_double2(u, u);
}

// Three-stage RK weights q = a*qold + b*(qc - dt/area*res), stage irk = 1..3
// (CCFVM/main.F90:39-44 airk/birk, the same weights in NCFVM/main.f90).
// Selected by branch, not by indexing a local table (which lands on the stack).
__device__ __forceinline__ double rk3_a(int irk) { return irk == 2 ? 3.0 / 4.0 : (irk == 3 ? 1.0 / 3.0 : 0.0); }
__device__ __forceinline__ double rk3_b(int irk) { return irk == 2 ? 1.0 / 4.0 : (irk == 3 ? 2.0 / 3.0 : 1.0); }

}  // namespace uns
