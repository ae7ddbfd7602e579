// FP64 arithmetic rate of the device: the roof of the FP64 form of the path, whose face-flux and
// sweep kernels are bound by the FP64 pipe rather than by HBM. Each thread runs eight independent
// chains of dependent FMAs (x = x * a + b, |a| < 1, so the values stay bounded); the grid covers
// every SM several times over, so the FP64 pipe, not latency, sets the rate. Two FLOPs per FMA.
// Also here: a device check of the FP64 form's Newton-refined reciprocal, quotient and square root
// against the IEEE operations.
#include "../../include/gbturbo.h"
#include "gbt_common.cuh"
#include "dfloat.cuh"
#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_fp64_fma(int iters, double a, double b, double *out)
{
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = (double)(threadIdx.x + c) * 1e-3;
    for (int n = 0; n < iters; n++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) x[c] = fma(x[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += x[c];
    // a store that never happens for these inputs keeps every thread's chains live; one real store
    if (s < 0.0) out[blockIdx.x] = s;
    if (threadIdx.x == 0) out[blockIdx.x] = s;
}

}  // namespace

extern "C" int gb_fp64_rate(double *flop_per_s)
{
    if (!flop_per_s) return GB_ERR_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return GB_ERR_CUDA;
    const int blocks = sms * 8, iters = 4096;
    double *out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = GB_OK;
    if (cudaMalloc(&out, sizeof(double) * blocks) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
        rc = GB_ERR_CUDA;
    } else {
        float best = 1e30f;
        for (int rep = 0; rep < 6 && rc == GB_OK; rep++) {
            cudaEventRecord(e0);
            k_fp64_fma<<<blocks, kThreads>>>(iters, 0.9999999, 1e-7, out);
            cudaEventRecord(e1);
            if (cudaEventSynchronize(e1) != cudaSuccess) { rc = GB_ERR_CUDA; break; }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0 && ms < best) best = ms;        // the first launch is a warm-up
        }
        if (rc == GB_OK) {
            const double fmas = (double)blocks * kThreads * iters * kChains;
            *flop_per_s = 2.0 * fmas / (best * 1e-3);
        }
    }
    if (cudaGetLastError() != cudaSuccess) rc = GB_ERR_CUDA;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (out) cudaFree(out);
    return rc;
}

// ---- the FP64 form's reciprocal, quotient and square root against the IEEE FP64 operations, and ----
// ---- the integer splits and conversions of dfloat.cuh                                            ----
namespace {

__global__ void k_arith(int op, const double *__restrict__ x, const double *__restrict__ y, long long n, double *out)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double a = x[t], b = y[t];
    double v;
    switch (op) {
    case 0: v = gbt::fdiv<double>(a, b); break;
    case 1: v = gbt::fsqrt<double>(a); break;
    case 2: v = gbt::frcp<double>(a); break;
    case 3: v = a / b; break;
    case 4: v = sqrt(a); break;
    // the split of an FP64 value into an FP32 pair (its value summed back in FP64), and FP32 <->
    // FP64 conversions by integer operations against the conversion instructions
    case 5: { const gbt::dfloat d = gbt::df_from(a); v = (double)d.hi + (double)d.lo; } break;
    case 6: v = gbt::f32_to_f64(gbt::f64_to_f32_rn(a)); break;
    default: v = (double)__double2float_rn(a); break;
    }
    out[t] = v;
}

}  // namespace

extern "C" int gb_fp64_arith_check(int op, const double *x, const double *y, long long n, double *out)
{
    const bool binary = op == 0 || op == 3;
    if (op < 0 || op > 7 || !x || !out || n < 1 || (binary && !y)) return GB_ERR_ARG;
    double *d = nullptr;
    const size_t bytes = sizeof(double) * (size_t)n;
    if (cudaMalloc(&d, 3 * bytes) != cudaSuccess) return GB_ERR_CUDA;
    int rc = GB_OK;
    if (cudaMemcpy(d, x, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(d + n, y ? y : x, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
        rc = GB_ERR_CUDA;
    } else {
        k_arith<<<(unsigned)((n + 255) / 256), 256>>>(op, d, d + n, n, d + 2 * n);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(out, d + 2 * n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = GB_ERR_CUDA;
    }
    cudaFree(d);
    return rc;
}
