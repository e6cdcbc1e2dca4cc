// uns_api.cu -- library-wide entry points of libunsflow_gpu.so.
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "uns_common.cuh"
#include "uns_phys.cuh"
#include "unsflow_gpu.h"

namespace {
__global__ void k_selftest_div(const double* a, const double* b, double* out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = uns::div_rn_recip(a[i], b[i], 1.0 / b[i]);
}
__global__ void k_selftest_ratio(const double* a, const double* b, const double* c, const double* d, int* lt, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    lt[i] = (uns::ratio_ok(a[i], b[i]) && uns::ratio_ok(c[i], d[i])) ? (uns::ratio_less(a[i], b[i], c[i], d[i]) ? 1 : 0) : -1;
}

// Copies n values of each host array in, runs launch, copies out.
template <class T, class L>
int run_selftest(const char* name, int n, std::initializer_list<const double*> in, T* out, L launch) {
    if (n < 0) return UNS_ERR_ARG;
    if (n == 0) return UNS_OK;
    std::vector<double*> d;
    T* dout = nullptr;
    int rc = UNS_OK;
    for (const double* h : in) {
        double* p = nullptr;
        if (!h || cudaMalloc(&p, sizeof(double) * n) != cudaSuccess) { rc = h ? UNS_ERR_CUDA : UNS_ERR_ARG; break; }
        d.push_back(p);
        if (cudaMemcpy(p, h, sizeof(double) * n, cudaMemcpyHostToDevice) != cudaSuccess) { rc = UNS_ERR_CUDA; break; }
    }
    if (!rc && (!out || cudaMalloc(&dout, sizeof(T) * n) != cudaSuccess)) rc = out ? UNS_ERR_CUDA : UNS_ERR_ARG;
    if (!rc) {
        launch(d, dout, (n + 255) / 256);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(out, dout, sizeof(T) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = UNS_ERR_CUDA;
    }
    if (rc) uns::set_last_error(std::string(name) + ": bad argument or CUDA call failed");
    for (double* p : d) cudaFree(p);
    cudaFree(dout);
    return rc;
}
}  // namespace

namespace uns {
thread_local std::string g_last_error;
void set_last_error(const std::string& s) { g_last_error = s; }
}  // namespace uns

extern "C" {
const char* uns_last_error(void) { return uns::g_last_error.c_str(); }
const char* uns_version(void) { return "unsflow_gpu 0.1 (sm_103a)"; }

int uns_selftest_div(const double* a, const double* b, double* out, int n) {
    return run_selftest("uns_selftest_div", n, {a, b}, out, [&](std::vector<double*>& d, double* o, int nb) {
        k_selftest_div<<<nb, 256>>>(d[0], d[1], o, n);
    });
}

int uns_selftest_ratio(const double* a, const double* b, const double* c, const double* d, int* lt, int n) {
    return run_selftest("uns_selftest_ratio", n, {a, b, c, d}, lt, [&](std::vector<double*>& p, int* o, int nb) {
        k_selftest_ratio<<<nb, 256>>>(p[0], p[1], p[2], p[3], o, n);
    });
}
}
