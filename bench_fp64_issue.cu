// bench_fp64_issue.cu -- GB300 arithmetic and memory latencies that bound the
// LU-SGS sweeps and the FP64 face kernels (not part of the library).
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 --fmad=false \
//        -o fp64_issue bench_fp64_issue.cu && ./fp64_issue
//
// Prints, for FP64 add / mul / fma / divide, FP32 add / divide and an
// FP64 -> FP32 conversion, the
// cycles per dependent operation of one thread and the whole-GPU rate at
// 1, 4 and 8 warps per SM sub-partition, with 1 and 32 active lanes (does an
// FP64 warp-instruction cost less with fewer active lanes?), and the latency
// of a dependent L2-coherent load chain over 16 MB, 64 MB and 2 GB.
#include <cuda_runtime.h>

#include <cstdio>

constexpr int kN = 1024;

template <int OP>
__global__ void k_chain(double* out, double a, int active, long long* cyc) {
    double x = a;
    long long t0 = clock64();
    if ((threadIdx.x & 31) < active) {
        if (OP == 0) {
#pragma unroll 16
            for (int i = 0; i < kN; ++i) x = x + a;
        } else if (OP == 1) {
#pragma unroll 16
            for (int i = 0; i < kN; ++i) x = x * a;
        } else if (OP == 2) {
#pragma unroll 16
            for (int i = 0; i < kN; ++i) x = fma(x, a, a);
        } else if (OP == 3) {
#pragma unroll 4
            for (int i = 0; i < kN / 8; ++i) x = a / x;
        } else if (OP == 4) {
            float y = (float)x, b = (float)a;
#pragma unroll 16
            for (int i = 0; i < kN; ++i) y = y + b;
            x = y;
        } else if (OP == 5) {
            float y = (float)x, b = (float)a;
#pragma unroll 4
            for (int i = 0; i < kN / 8; ++i) y = b / y;
            x = y;
        } else {  // independent FP64 -> FP32 conversions feeding one FP32 sum
            const long long bits = __double_as_longlong(a) + threadIdx.x;
            float acc = 0.f;
#pragma unroll 16
            for (int i = 0; i < kN; ++i) acc += (float)__longlong_as_double(bits + ((long long)i << 20));
            x = acc;
        }
    }
    long long t1 = clock64();
    if (threadIdx.x == 0 && blockIdx.x == 0) *cyc = t1 - t0;
    out[blockIdx.x * blockDim.x + threadIdx.x] = x;
}

__global__ void k_chase(const unsigned* next, int steps, long long* cyc, unsigned* sink) {
    unsigned j = 0;
    long long t0 = clock64();
    for (int i = 0; i < steps; ++i) j = __ldcg(next + j);
    long long t1 = clock64();
    *cyc = t1 - t0;
    *sink = j;
}

int main() {
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0);
    double* out;
    long long* cyc;
    cudaMalloc(&out, (size_t)nsm * 1024 * sizeof(double));
    cudaMalloc(&cyc, sizeof(long long));
    struct Op { const char* name; void (*f)(double*, double, int, long long*); int ops; };
    Op ops[] = {{"f64 add", k_chain<0>, kN}, {"f64 mul", k_chain<1>, kN}, {"f64 fma", k_chain<2>, kN},
                {"f64 div", k_chain<3>, kN / 8}, {"f32 add", k_chain<4>, kN}, {"f32 div", k_chain<5>, kN / 8},
                {"cvt f64>f32 (independent) + f32 add", k_chain<6>, kN}};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (auto& op : ops)
        for (int threads : {128, 512, 1024})
            for (int active : {1, 32}) {
                op.f<<<nsm, threads>>>(out, 1.0000001, active, cyc);
                cudaEventRecord(e0);
                op.f<<<nsm, threads>>>(out, 1.0000001, active, cyc);
                cudaEventRecord(e1);
                cudaEventSynchronize(e1);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                long long c = 0;
                cudaMemcpy(&c, cyc, sizeof(c), cudaMemcpyDeviceToHost);
                double winstr = (double)op.ops * nsm * (threads / 32);
                printf("%s  warps/sub-partition %d  active lanes %2d: %7.1f cycles/op (one thread), "
                       "%6.2f G warp-instr/s\n", op.name, threads / 128, active, (double)c / op.ops,
                       winstr / ms / 1e6);
            }
    for (size_t mb : {16, 64, 2048}) {
        size_t n = mb * 1024 * 1024 / 4, lines = n / 32;
        unsigned* h = new unsigned[n]();
        unsigned* perm = new unsigned[lines];
        for (size_t i = 0; i < lines; ++i) perm[i] = (unsigned)i;
        unsigned long long s = 88172645463325252ull;
        for (size_t i = lines - 1; i > 0; --i) {
            s ^= s << 13; s ^= s >> 7; s ^= s << 17;
            size_t j = s % (i + 1);
            unsigned t = perm[i]; perm[i] = perm[j]; perm[j] = t;
        }
        for (size_t i = 0; i < lines; ++i) h[(size_t)perm[i] * 32] = perm[(i + 1) % lines] * 32;
        unsigned *d, *sink;
        cudaMalloc(&d, n * 4);
        cudaMalloc(&sink, 4);
        cudaMemcpy(d, h, n * 4, cudaMemcpyHostToDevice);
        const int steps = 20000;
        k_chase<<<1, 1>>>(d, steps, cyc, sink);
        k_chase<<<1, 1>>>(d, steps, cyc, sink);
        long long c = 0;
        cudaMemcpy(&c, cyc, sizeof(c), cudaMemcpyDeviceToHost);
        printf("dependent ld.global.cg chain over %zu MB: %.0f cycles per load\n", mb, (double)c / steps);
        cudaFree(d);
        cudaFree(sink);
        delete[] h;
        delete[] perm;
    }
    cudaError_t e = cudaDeviceSynchronize();
    printf("status: %s\n", cudaGetErrorString(e));
    return e == cudaSuccess ? 0 : 1;
}
