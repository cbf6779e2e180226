/*
 * spacelab_diag.h -- diagnostics of libspacelab_gb300.so (no counterpart in
 * the reference): device-side checks and measurements used by the tests
 * and the benchmark.  Not needed to run a simulation.
 */
#ifndef SPACELAB_DIAG_H
#define SPACELAB_DIAG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* For i < n computes on the current GPU q_recip[i] = the step kernels'
 * reciprocal-based quotient of a[i] / b[i] (b[i] > 0, with RN(1/b[i])) and
 * q_ieee[i] = the IEEE double quotient a[i] / b[i].  Host arrays. */
int sl_diag_division(int n, const double* a, const double* b, double* q_recip, double* q_ieee);

/* For i < n, on the current GPU: out[i] = a[i]/b[i] and out[2n+i] =
 * sqrt(|a[i]|) as the step kernels compute them (an FP64 estimate rounded
 * exactly with integer arithmetic), out[n+i] and out[3n+i] = the hardware
 * IEEE results.  Host arrays; out has 4n entries. */
int sl_diag_exact_ops(int n, const double* a, const double* b, double* out);

/* The integer-pipe arithmetic of the exact step, rounded exactly: out[6n]
 * = a/b with a fixed-point reciprocal of b made at set-up, a/b with a
 * Newton fixed-point reciprocal, sqrt(|a|) from a fixed-point 1/sqrt,
 * a / RN(sqrt(|b|)) from the fixed-point 1/sqrt of |b|, a*b, and -(a/b)
 * with the sign set in the integer result.  Each must equal the IEEE
 * result bit for bit.  No reference counterpart (a self-test). */
int sl_diag_int_ops(int n, const double* a, const double* b, double* out);

/* Latency of a dependent FP64 add chain: one block of warps_per_sm warps per
 * SM, active_lanes lanes of each warp running a chain; *cycles_per_add at
 * the rated SM clock.  No reference counterpart (a self-test). */
int sl_diag_fp64_add_latency(int warps_per_sm, int active_lanes, double* cycles_per_add);

/* Measured FP64 fused-multiply-add throughput of the current GPU in
 * GFLOP/s (2 flops per FMA), from a kernel of independent FMA chains timed
 * with CUDA events. */
int sl_diag_fp64_peak(double* gflops);

/* The same for FP32 fused multiply-adds (the mixed form's pipe). */
int sl_diag_fp32_peak(double* gflops);

/* One surrogate GEMM on host data, for checking the GEMM kernels:
 * C[M][N] = A[M][K] . B[N][K]^T (+ bias[N]) with A, B bf16 bit patterns,
 * row-major; C f32 [M][N]; Cb (may be NULL) gets bf16(act ? GELU(C) : C).
 * kernel 0: the mma.sync kernel (K a multiple of 32); 1: the tcgen05 kernel
 * (K a multiple of 8).  Allocates its own device buffers.  No counterpart in
 * the reference. */
int sl_diag_gemm_bf16(int M, int N, int K, const uint16_t* A, const uint16_t* B, const float* bias, int act,
                      int kernel, float* C, uint16_t* Cb);

#ifdef __cplusplus
}
#endif
#endif /* SPACELAB_DIAG_H */
