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
