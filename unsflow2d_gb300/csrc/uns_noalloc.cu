// uns_noalloc.cu -- a residual-norm entry point that allocates no memory.
//
// uns_cc_residue reduces a handle's residual through per-block partial sums
// kept in memory that uns_cc_create allocated.  uns_residue_rms_noalloc does
// the same reduction over a residual array the caller owns, with its partial
// sums in a fixed static device array, so the call itself never allocates or
// frees device memory.  The two kernels below repeat the block size and the
// summation tree of k_res_partial / k_res_final in uns_cc.cu, so both entry
// points return the same bits for the same residual.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "uns_common.cuh"
#include "unsflow_gpu.h"

using namespace uns;

namespace {

// Capacity of the static scratch: one partial sum per kBlock cells.
constexpr int kMaxParts = UNS_RMS_NOALLOC_MAX_CELLS / kBlock;
static_assert(kMaxParts * kBlock == UNS_RMS_NOALLOC_MAX_CELLS, "limit must be a multiple of the block size");

// Partial sums [0, kMaxParts) and the result slot [kMaxParts].  Every launch
// writes each slot it later reads, so nothing here has to start at zero.
static __device__ __align__(256) double g_rms_scratch[kMaxParts + 1];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
// Device address of g_rms_scratch per device ordinal, with the id of the
// context it was looked up in.  A module's globals live in one context: after
// cudaDeviceReset (or any reset of the device's primary context) the library
// is loaded again in a new context and the old address means nothing, so the
// address is looked up again whenever the current context's id differs.
double* g_addr[kMaxDevices] = {};
unsigned long long g_ctx_id[kMaxDevices] = {};

// Driver entry points for the current context's id, resolved through the
// runtime so the library does not link libcuda itself.
typedef int (*ctx_get_current_fn)(void**);
typedef int (*ctx_get_id_fn)(void*, unsigned long long*);

// Id of the current context, 0 when the driver cannot say (then the address
// is looked up on every call).
unsigned long long current_ctx_id() {
    static ctx_get_current_fn get_current = nullptr;
    static ctx_get_id_fn get_id = nullptr;
    static bool resolved = false;
    if (!resolved) {
        void* f0 = nullptr;
        void* f1 = nullptr;
        cudaDriverEntryPointQueryResult q0 = cudaDriverEntryPointSymbolNotFound;
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            q0 == cudaDriverEntryPointSuccess && q1 == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<ctx_get_current_fn>(f0);
            get_id = reinterpret_cast<ctx_get_id_fn>(f1);
        }
        cudaGetLastError();
        resolved = true;
    }
    if (!get_current || !get_id) return 0;
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

__global__ void __launch_bounds__(kBlock) k_rms_partial(const double4* __restrict__ res, int n, double* part) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double rr = 0.0;
    if (i < n) {
        double4 r = res[i];
        rr = r.x * r.x + r.y * r.y + r.z * r.z + r.w * r.w;
    }
    __shared__ double s[kBlock / 32];
    rr = warp_sum(rr);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = rr;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < kBlock / 32; ++k) t = t + s[k];
        part[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kBlock) k_rms_final(const double* part, int nparts, int n, double* out) {
    __shared__ double s[kBlock];
    double t = 0.0;
    for (int k = threadIdx.x; k < nparts; k += blockDim.x) t = t + part[k];
    s[threadIdx.x] = t;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) s[threadIdx.x] = s[threadIdx.x] + s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sqrt(s[0] / (double)n / 4.0);
}

// Address of the scratch on the current device: looked up on the first call
// for that device, and again on the first call in each new context of it.
int scratch_address(double** out) {
    int dev = -1;
    UNS_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_last_error("uns_residue_rms_noalloc: device ordinal out of range");
        return UNS_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    const unsigned long long ctx = current_ctx_id();
    if (!g_addr[dev] || ctx == 0 || ctx != g_ctx_id[dev]) {
        void* p = nullptr;
        UNS_CUDA(cudaGetSymbolAddress(&p, g_rms_scratch));
        g_addr[dev] = static_cast<double*>(p);
        g_ctx_id[dev] = ctx;
    }
    *out = g_addr[dev];
    return UNS_OK;
}

}  // namespace

extern "C" int uns_residue_rms_noalloc(const double* res, int ncells, double* fres_raw, void* stream) {
    if (!res || !fres_raw || ncells <= 0) {
        set_last_error("uns_residue_rms_noalloc: null pointer or empty residual");
        return UNS_ERR_ARG;
    }
    if (ncells > UNS_RMS_NOALLOC_MAX_CELLS) {
        set_last_error("uns_residue_rms_noalloc: more cells than the static scratch holds");
        return UNS_ERR_ARG;
    }
    if (reinterpret_cast<std::uintptr_t>(res) % 32 != 0) {
        set_last_error("uns_residue_rms_noalloc: residual array is not 32-byte aligned");
        return UNS_ERR_ARG;
    }
    double* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nparts = nblocks(ncells);
    k_rms_partial<<<nparts, kBlock, 0, s>>>(reinterpret_cast<const double4*>(res), ncells, scratch);
    UNS_CUDA(cudaGetLastError());
    k_rms_final<<<1, kBlock, 0, s>>>(scratch, nparts, ncells, scratch + kMaxParts);
    UNS_CUDA(cudaGetLastError());
    UNS_CUDA(cudaMemcpyAsync(fres_raw, scratch + kMaxParts, sizeof(double), cudaMemcpyDeviceToHost, s));
    UNS_CUDA(cudaStreamSynchronize(s));
    return UNS_OK;
}
