/*
 * pbt_probe.h -- arithmetic-rate probes of the current GPU (part of libpbt.so).
 *
 * No counterpart in the reference.  The solve's ceilings on GB300 are the
 * FP64 and FP32 FMA rates, not only HBM bandwidth, so the benchmark measures
 * them on the device it runs on and reports its kernels against them.
 */
#ifndef PBT_PROBE_H
#define PBT_PROBE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Sustained fused multiply-add rates of the current device in FMA/s, from
 * kernels with 8 independent FMA chains per thread on 4 CTAs x 256 threads
 * per SM (best of 3 timed launches each, CUDA events).  Either pointer may be
 * NULL.  Returns 0 or a pbt_status code. */
int pbt_probe_fma_rates(double* fp64_fma_per_s, double* fp32_fma_per_s);

#ifdef __cplusplus
}
#endif
#endif
