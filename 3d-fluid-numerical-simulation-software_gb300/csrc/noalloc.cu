// Residual norm (CMesh::Res_Calculate) that performs no allocation on success: its scratch is a
// fixed, statically sized device array in this file instead of memory owned by the handle or
// taken from an allocator.
//
// Who needs it: a caller that must not allocate between iterations, e.g. a convergence monitor
// of a batch whose device memory is already committed to the solve pools, or a host thread that
// runs under a rule of no heap allocation at steady state. The ordinary gb_res_calculate builds
// a host-side vector of the batch's solve states on every call; this variant writes the norms
// into the static array and copies them straight into the caller's buffer.
//
// Limits and sharing:
//  - at most GB_NOALLOC_MAX_SOLVES blocks (slots) per handle (the array holds 64 partial sums of
//    5 components for each of them); larger batches are rejected with GB_ERR_ARG;
//  - every call, from every handle on a device, shares the one array: calls that overlap in time
//    (two host threads, or two streams in flight at once) race on it and must be serialised by
//    the caller;
//  - the first call on a device looks the array's address up (cudaGetSymbolAddress, with that
//    device current) and zeroes it on the calling handle's stream; make that first call before any
//    stream capture begins;
//  - the address is kept per device for the life of the process: after cudaDeviceReset the kept
//    address belongs to a context that no longer exists, so do not call this entry point again in a
//    process that has reset the device.
#include "../../include/gbturbo.h"
#include "kernels.hpp"
#include "solver.hpp"
#include <mutex>

namespace gbt {
namespace {

constexpr int kBlocks = 64;                                        // partial sums per solve
constexpr int kMaxSolves = GB_NOALLOC_MAX_SOLVES;
constexpr size_t kPartials = (size_t)kMaxSolves * kBlocks * 5;     // doubles
constexpr size_t kOut = (size_t)kMaxSolves * 5;                    // doubles
constexpr size_t kCounterWords = (size_t)kMaxSolves;               // one unsigned per solve, padded to a double
constexpr size_t kScratchDoubles = kPartials + kOut + kCounterWords;

// partials | norms out | arrival counters (must be zero when a call's kernel starts)
static __device__ __align__(256) double g_norm_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
double *g_scratch_addr[kMaxDevices] = {};

// Device address of g_norm_scratch on the current device, looked up (and zeroed on `stream`) once
// per device.
cudaError_t scratch_for_current_device(cudaStream_t stream, double **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_norm_scratch);
        if (e != cudaSuccess) return e;
        e = cudaMemsetAsync(p, 0, sizeof(double) * kScratchDoubles, stream);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = (double *)p;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

// One launch per call: every block folds a strided share of the cells (the same per-cell terms as
// the two-launch norm), the last block of each solve to arrive adds the 64 partials in block
// order. The two-launch norm uses more blocks, so the two agree to rounding, not bit for bit.
template <typename T>
__global__ void __launch_bounds__(256) k_norm_onepass(Batch B, Geo G, Flow<T> W, const double *__restrict__ totalvol,
                                                      double *partials, double *norms, unsigned *arrivals)
{
    const int s = blockIdx.y;
    const Lvl L = B.lv[s];
    const int nI = L.IM - 1, nJ = L.JM - 1, nK = L.KM - 1;
    const long long n = (long long)nI * nJ * nK;
    double acc[5] = {0, 0, 0, 0, 0};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)kBlocks * blockDim.x) {
        const int k = (int)(t % nK) + 1;
        const long long q = t / nK;
        const int j = (int)(q % nJ) + 1, i = (int)(q / nJ) + 1;
        const long long p = ix(L, i, j, k);
        const double vol = G.vol[p];
#pragma unroll
        for (int c = 0; c < 5; c++) {
            const double o = W.cvold[c][p];
            acc[c] += rel_change_t<T>(o, W.cv[c][p]) * vol;
        }
    }
    __shared__ double sh[8][5];
    __shared__ bool last;
#pragma unroll
    for (int c = 0; c < 5; c++) {
        double v = acc[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double v = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += sh[w][threadIdx.x];
        partials[((long long)s * kBlocks + blockIdx.x) * 5 + threadIdx.x] = v;
        __threadfence();
    }
    __syncthreads();
    // the blocks of all slots of a case count on the case's first slot; the last to arrive adds
    // the partials of the case's blocks in block order and gives every slot of the case the norm
    const SolveConst &sc = B.sc[s];
    if (threadIdx.x == 0) last = atomicAdd(&arrivals[sc.lead], 1u) == (unsigned)(kBlocks * sc.nblk - 1);
    __syncthreads();
    if (!last || threadIdx.x >= 5) return;
    __threadfence();
    double v = 0;
    for (int q = sc.lead; q < sc.lead + sc.nblk; q++)
        for (int b = 0; b < kBlocks; b++) v += __ldcg(&partials[((long long)q * kBlocks + b) * 5 + threadIdx.x]);
    v = v / totalvol[s];
    for (int q = sc.lead; q < sc.lead + sc.nblk; q++) B.st[q].res[threadIdx.x] = v;
    norms[sc.cix * 5 + threadIdx.x] = v;
    if (threadIdx.x == 0) {
        if (!isfinite(v)) B.st[sc.lead].status |= GBT_STATUS_NAN;
        arrivals[sc.lead] = 0u;
    }
}

}  // namespace

template <typename T>
void launch_res_norm_static(const LaunchCtx &ctx, const Geo &G, Flow<T> W, const double *totalvol, int ncase, double *host_out)
{
    const Batch &B = ctx.batch;
    if (B.nsolve > kMaxSolves) throw std::invalid_argument("batch larger than the static norm scratch");
    double *base = nullptr;
    check_cuda(scratch_for_current_device(ctx.stream, &base), "cudaGetSymbolAddress(g_norm_scratch)");
    double *partials = base, *norms = base + kPartials;
    unsigned *arrivals = reinterpret_cast<unsigned *>(base + kPartials + kOut);
    ctx.mark("res_norm_static", 1, 1);
    check_cuda(cudaMemsetAsync(arrivals, 0, sizeof(unsigned) * B.nsolve, ctx.stream), "cudaMemsetAsync");
    k_norm_onepass<T><<<dim3(kBlocks, B.nsolve), 256, 0, ctx.stream>>>(B, G, W, totalvol, partials, norms, arrivals);
    check_cuda(cudaGetLastError(), "k_norm_onepass launch");
    ctx.mark("res_norm_static", 0, 1);
    if (host_out) {
        check_cuda(cudaMemcpyAsync(host_out, norms, sizeof(double) * 5 * ncase, cudaMemcpyDeviceToHost, ctx.stream),
                   "cudaMemcpyAsync");
        check_cuda(cudaStreamSynchronize(ctx.stream), "cudaStreamSynchronize");
    }
}

template void launch_res_norm_static<double>(const LaunchCtx &, const Geo &, Flow<double>, const double *, int, double *);
template void launch_res_norm_static<float>(const LaunchCtx &, const Geo &, Flow<float>, const double *, int, double *);

}  // namespace gbt
