// fma_probe.cu -- FP64 / FP32 FMA rate probes for the benchmark
// (libpbt_probe.so, loaded by pascal_btdma_gb300/peaks.py).
//
// Measurement tooling, not part of the solver library or its C ABI: the
// solve's ceilings on GB300 are the FP64 and FP32 FMA rates as well as HBM
// bandwidth, so bench.py measures them on the device it runs on and reports
// the kernels against them.
#include <cuda_runtime.h>

extern "C" {
/* Sustained fused multiply-add rates of the current device in FMA/s, from
 * kernels with 8 independent FMA chains per thread on 4 CTAs x 256 threads
 * per SM (best of 3 timed launches each, CUDA events).  Either pointer may be
 * NULL.  Returns 0, or 2 when a CUDA call failed. */
int pbt_probe_fma_rates(double* fp64_fma_per_s, double* fp32_fma_per_s);
/* The same for the packed two-lane FP32 FMA (PTX fma.rn.f32x2, two FMAs per
 * instruction), counted in FMAs. */
int pbt_probe_fma2_rate(double* fp32x2_fma_per_s);
}

namespace {

template <typename T, int CH>
__global__ void fma_chains(T* out, int iters, T a, T b) {
    T x[CH];
#pragma unroll
    for (int k = 0; k < CH; ++k) x[k] = (T)(threadIdx.x * 1e-7) + (T)k;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int k = 0; k < CH; ++k) x[k] = fma(x[k], a, b);
    T s = 0;
#pragma unroll
    for (int k = 0; k < CH; ++k) s += x[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__device__ __forceinline__ unsigned long long fma2(unsigned long long x, unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(x), "l"(a), "l"(b));
    return d;
}

// Packed FP32 pairs: the chains carry two lanes each.
__global__ void fma2_chains(float* out, int iters, float a, float b) {
    unsigned long long x[8], av, bv;
    asm("mov.b64 %0, {%1, %1};" : "=l"(av) : "f"(a));
    asm("mov.b64 %0, {%1, %1};" : "=l"(bv) : "f"(b));
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const float v = threadIdx.x * 1e-7f + (float)k;
        asm("mov.b64 %0, {%1, %2};" : "=l"(x[k]) : "f"(v), "f"(v + 0.5f));
    }
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma2(x[k], av, bv);
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        float lo, hi;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(x[k]));
        s += lo + hi;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
double rate(int sms, int iters, cudaError_t& err) {
    const int blocks = sms * 4, threads = 256, ch = 8;
    T* out = nullptr;
    err = cudaMalloc(&out, sizeof(T) * blocks * threads);
    if (err != cudaSuccess) return 0.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_chains<T, 8><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
    float best = 1e30f;
    for (int r = 0; r < 3; ++r) {
        cudaEventRecord(e0);
        fma_chains<T, 8><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return (double)blocks * threads * ch * iters / (best * 1e-3);
}

}  // namespace

extern "C" int pbt_probe_fma_rates(double* fp64, double* fp32) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 2;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 2;
    cudaError_t e = cudaSuccess;
    if (fp64) {
        *fp64 = rate<double>(sms, 2048, e);
        if (e != cudaSuccess) return 2;
    }
    if (fp32) {
        *fp32 = rate<float>(sms, 65536, e);
        if (e != cudaSuccess) return 2;
    }
    return 0;
}

extern "C" int pbt_probe_fma2_rate(double* fp32x2) {
    int dev = 0, sms = 0;
    if (!fp32x2) return 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 2;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 2;
    const int blocks = sms * 4, threads = 256, iters = 65536;
    float* out = nullptr;
    cudaError_t e = cudaMalloc(&out, sizeof(float) * blocks * threads);
    if (e != cudaSuccess) return 2;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma2_chains<<<blocks, threads>>>(out, iters, 0.999999f, 1e-7f);
    float best = 1e30f;
    for (int r = 0; r < 3; ++r) {
        cudaEventRecord(e0);
        fma2_chains<<<blocks, threads>>>(out, iters, 0.999999f, 1e-7f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return 2;
    *fp32x2 = (double)blocks * threads * 8 * 2 * iters / (best * 1e-3);
    return 0;
}
