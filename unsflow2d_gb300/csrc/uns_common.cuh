// uns_common.cuh -- shared plumbing of the UNSFlow2D GB300 library: status
// handling, the device error word, warp/block reductions and the bounded grid
// barrier used by the level-scheduled LU-SGS sweeps.
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

// Grid-wide barrier for cooperative launches.  Every wait is bounded: after
// ~kBarrierCycles without progress the block records UNS_ERR_TIMEOUT and the
// caller returns, so a stuck peer can never hang the device.
constexpr long long kBarrierCycles = 4000000000LL;  // ~2 s at 2 GHz

struct GridSync {
    unsigned int count;
    unsigned int gen;
};

__device__ __forceinline__ bool grid_barrier(GridSync* gs, DevErr* err) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        volatile unsigned int* vgen = &gs->gen;
        unsigned int g = *vgen;
        __threadfence();
        unsigned int arrived = atomicAdd(&gs->count, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(&gs->count, 0u);
            __threadfence();
            atomicAdd(&gs->gen, 1u);
        } else {
            long long t0 = clock64();
            while (*vgen == g) {
                if (*((volatile int*)&err->code) == UNS_ERR_TIMEOUT || clock64() - t0 > kBarrierCycles) {
                    set_err(err, UNS_ERR_TIMEOUT, (int)blockIdx.x);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

}  // namespace uns
