// sl_diag.cu -- diagnostics (include/spacelab_diag.h).
#include "../../include/spacelab_diag.h"
#include "../../include/spacelab_gpu.h"
#include "sl_device.cuh"
#include "sl_fp64_exact.cuh"

#include <cuda_runtime.h>

namespace {

__global__ void division_kernel(int n, const double* a, const double* b, double* qr, double* qi)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double y = 1.0 / b[i];
    qr[i] = sl::div_by_recip(a[i], b[i], y);
    qi[i] = a[i] / b[i];
}

// out[0..n): quotient via estimate + integer rounding, [n..2n): hardware
// quotient, [2n..3n): sqrt(|a|) via estimate, [3n..4n): hardware sqrt
__global__ void exact_ops_kernel(int n, const double* a, const double* b, double* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = a[i], y = b[i];
    const double yi = sl::rsqrt_refined(y * y);  // ~1/|y|
    out[i] = sl::div_from_estimate(x, y, x * (y < 0 ? -yi : yi));
    out[n + i] = x / y;
    const double ax = fabs(x);
    const double r = sl::rsqrt_refined(ax);
    out[2 * (size_t)n + i] = sl::sqrt_from_estimate(ax, ax * r);
    out[3 * (size_t)n + i] = sqrt(ax);
}

// out[0..n): a / b with the fixed-point reciprocal made at set-up
// (recip_sig), [n..2n): a / b with the Newton reciprocal, [2n..3n):
// sqrt(|a|) from the fixed-point 1/sqrt, [3n..4n): a / RN(sqrt(|b|)) from
// the same 1/sqrt of |b|, [4n..5n): a * b on the integer pipe, [5n..6n):
// -(a / b) with the sign set in the integer result.
__global__ void int_ops_kernel(int n, const double* a, const double* b, const unsigned long long* rb, double* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = a[i], y = b[i];
    out[i] = sl::div_by_fixed<false>(x, y, rb[i]);
    out[n + i] = sl::div_by_fixed<true>(x, y, sl::recip_newton(y));
    int p;
    unsigned long long F;
    const double ax = fabs(x);
    const unsigned long long Y = sl::rsqrt_fix(ax, p, F);
    out[2 * (size_t)n + i] = sl::sqrt_fix(ax, F, Y, p);
    const double ay = fabs(y);
    int q;
    unsigned long long G;
    const unsigned long long Z = sl::rsqrt_fix(ay, q, G);
    const double d = sl::sqrt_fix(ay, G, Z, q);
    out[3 * (size_t)n + i] = sl::div_by_rsqrt(x, d, Z, q);
    out[4 * (size_t)n + i] = sl::mul_int(x, y);
    out[5 * (size_t)n + i] = sl::div_by_fixed<false, true>(x, y, rb[i]);
}

__global__ void recip_kernel(int n, const double* b, unsigned long long* rb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) rb[i] = sl::recip_of(b[i]);
}

// One dependent FP64 add chain per thread of `active` lanes of each warp.
__global__ void add_chain_kernel(double* out, int iters, int active, double inc)
{
    const int lane = threadIdx.x & 31;
    if (lane >= active) return;
    double a = threadIdx.x * 1e-3;
    for (int i = 0; i < iters; ++i) {
        a = a + inc;
        a = a + inc;
        a = a + inc;
        a = a + inc;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a;
}

constexpr int kChains = 8;
constexpr int kIters = 4096;

__global__ void fma_chain_kernel(double* out, double seed)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double v[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) v[k] = seed + t * 1e-9 + k;
    const double b = 0.999999, c = 1e-7;
    for (int i = 0; i < kIters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) v[k] = fma(v[k], b, c);
    }
    double s = 0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += v[k];
    out[t] = s;
}

constexpr int kIters32 = 16384;

__global__ void fma32_chain_kernel(float* out, float seed)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    float v[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) v[k] = seed + t * 1e-6f + k;
    const float b = 0.9999f, c = 1e-4f;
    for (int i = 0; i < kIters32; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) v[k] = fmaf(v[k], b, c);
    }
    float s = 0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += v[k];
    out[t] = s;
}

// Best-of-3 time (after one untimed launch) of `launch`, in ms; <0 on error.
template <typename F>
float best_time_ms(F launch)
{
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        launch();
        cudaEventRecord(e1);
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
            best = -1.0f;
            break;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return best;
}

}  // namespace

extern "C" int sl_diag_division(int n, const double* a, const double* b, double* q_recip, double* q_ieee)
{
    if (n < 1 || !a || !b || !q_recip || !q_ieee) return SL_ERR_ARG;
    double* d = nullptr;
    const size_t bytes = (size_t)n * sizeof(double);
    if (cudaMalloc(&d, 4 * bytes) != cudaSuccess) return SL_ERR_ALLOC;
    int rc = SL_OK;
    if (cudaMemcpy(d, a, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(d + n, b, bytes, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = SL_ERR_CUDA;
    if (rc == SL_OK) {
        division_kernel<<<(n + 255) / 256, 256>>>(n, d, d + n, d + 2 * (size_t)n, d + 3 * (size_t)n);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = SL_ERR_CUDA;
    }
    if (rc == SL_OK && (cudaMemcpy(q_recip, d + 2 * (size_t)n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess ||
                        cudaMemcpy(q_ieee, d + 3 * (size_t)n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess))
        rc = SL_ERR_CUDA;
    cudaFree(d);
    return rc;
}

extern "C" int sl_diag_exact_ops(int n, const double* a, const double* b, double* out)
{
    if (n < 1 || !a || !b || !out) return SL_ERR_ARG;
    double* d = nullptr;
    const size_t bytes = (size_t)n * sizeof(double);
    if (cudaMalloc(&d, 6 * bytes) != cudaSuccess) return SL_ERR_ALLOC;
    int rc = SL_OK;
    if (cudaMemcpy(d, a, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(d + n, b, bytes, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = SL_ERR_CUDA;
    if (rc == SL_OK) {
        exact_ops_kernel<<<(n + 255) / 256, 256>>>(n, d, d + n, d + 2 * (size_t)n);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = SL_ERR_CUDA;
    }
    if (rc == SL_OK && cudaMemcpy(out, d + 2 * (size_t)n, 4 * bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = SL_ERR_CUDA;
    cudaFree(d);
    return rc;
}

extern "C" int sl_diag_int_ops(int n, const double* a, const double* b, double* out)
{
    if (n < 1 || !a || !b || !out) return SL_ERR_ARG;
    double* d = nullptr;
    const size_t bytes = (size_t)n * sizeof(double);
    if (cudaMalloc(&d, 9 * bytes) != cudaSuccess) return SL_ERR_ALLOC;
    unsigned long long* rb = reinterpret_cast<unsigned long long*>(d + 8 * (size_t)n);
    int rc = SL_OK;
    if (cudaMemcpy(d, a, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(d + n, b, bytes, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = SL_ERR_CUDA;
    if (rc == SL_OK) {
        recip_kernel<<<(n + 255) / 256, 256>>>(n, d + n, rb);
        int_ops_kernel<<<(n + 255) / 256, 256>>>(n, d, d + n, rb, d + 2 * (size_t)n);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = SL_ERR_CUDA;
    }
    if (rc == SL_OK && cudaMemcpy(out, d + 2 * (size_t)n, 6 * bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = SL_ERR_CUDA;
    cudaFree(d);
    return rc;
}

extern "C" int sl_diag_fp64_peak(double* gflops)
{
    if (!gflops) return SL_ERR_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return SL_ERR_CUDA;
    const int blocks = sms * 8, threads = 256;
    double* out = nullptr;
    if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) return SL_ERR_ALLOC;
    const float best = best_time_ms([&] { fma_chain_kernel<<<blocks, threads>>>(out, 1.0); });
    cudaFree(out);
    if (best <= 0) return SL_ERR_CUDA;
    const double flops = 2.0 * blocks * threads * (double)kChains * kIters;
    *gflops = flops / (best * 1e-3) / 1e9;
    return SL_OK;
}

extern "C" int sl_diag_fp32_peak(double* gflops)
{
    if (!gflops) return SL_ERR_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return SL_ERR_CUDA;
    const int blocks = sms * 8, threads = 256;
    float* out = nullptr;
    if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(float)) != cudaSuccess) return SL_ERR_ALLOC;
    const float best = best_time_ms([&] { fma32_chain_kernel<<<blocks, threads>>>(out, 1.0f); });
    cudaFree(out);
    if (best <= 0) return SL_ERR_CUDA;
    const double flops = 2.0 * blocks * threads * (double)kChains * kIters32;
    *gflops = flops / (best * 1e-3) / 1e9;
    return SL_OK;
}

extern "C" int sl_diag_fp64_add_latency(int warps_per_sm, int active_lanes, double* cycles_per_add)
{
    if (warps_per_sm < 1 || warps_per_sm > 32 || active_lanes < 1 || active_lanes > 32 || !cycles_per_add)
        return SL_ERR_ARG;
    int dev = 0, sms = 0, khz = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev) != cudaSuccess)
        return SL_ERR_CUDA;
    const int threads = 32 * warps_per_sm;
    double* out = nullptr;
    if (cudaMalloc(&out, (size_t)sms * threads * sizeof(double)) != cudaSuccess) return SL_ERR_ALLOC;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int iters = 20000;
    add_chain_kernel<<<sms, threads>>>(out, 100, active_lanes, 1e-9);
    cudaEventRecord(e0);
    add_chain_kernel<<<sms, threads>>>(out, iters, active_lanes, 1e-9);
    cudaEventRecord(e1);
    int rc = SL_OK;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess) rc = SL_ERR_CUDA;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (rc != SL_OK) return rc;
    // cycles at the device's rated SM clock
    *cycles_per_add = ms * 1e-3 * (khz * 1e3) / (4.0 * iters);
    return SL_OK;
}
