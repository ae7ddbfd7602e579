// Learned warm start (see warmstart.hpp): the network's kernels and its host side.
//
// The three products of training and inference run on the tcgen05 tensor cores with the
// accumulator in tensor memory (TMEM):
//   forward        Z[cells x N]   = H[cells x K] . W[N x K]^T        (+ bias, SiLU in the epilogue)
//   backward data  dH[cells x K]  = dZ[cells x N] . W[N x K]          (x SiLU'(Z) in the epilogue)
//   weight grad    dW[N x K]      = dZ^T . H  (the cells are the reduction dimension)
// Operands are staged in shared memory in the canonical K-major layout without swizzle (core
// matrices of 8 rows x 16 bytes, 128 contiguous bytes each), one elected thread issues
// tcgen05.mma (kind::f16, BF16 x BF16 -> FP32, M = 128), tcgen05.commit arrives on an mbarrier
// that every thread waits on (bounded), and the epilogue reads the accumulator rows with
// tcgen05.ld (warp w owns TMEM lanes 32w..32w+31, i.e. rows 32w..32w+31 of the tile).
#include "warmstart.hpp"
#include "gbt_common.cuh"
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <stdexcept>
#include <string>

namespace gbt {

typedef __nv_bfloat16 bf16;

#define WCK(x) check_cuda((x), #x)

// ---------------------------------------------------------------- tcgen05 / mbarrier primitives
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor (tcgen05 form, no swizzle): start address, byte distance between
// core matrices adjacent along K (lbo) and along M/N (sbo), all in 16-byte units; bits 46-47 = 1
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1),
// both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// about a second at most; a wait that runs out is reported through the error flag
constexpr int kMbarWaitLimit = 1 << 22;
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity)
{
    for (int t = 0; t < kMbarWaitLimit; t++) {
        if (mbar_try_wait(bar, parity)) return true;
        if (t > 32) __nanosleep(64);
    }
    return false;
}
// 32 TMEM lanes x 16 columns of 32 bits: thread t of the warp receives lane (base lane + t)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------- operand staging
__device__ __forceinline__ float sigmoidf_(float z) { return __fdividef(1.0f, 1.0f + __expf(-z)); }

// ---------------------------------------------------------------- the row product
// D[128 x N] = A[128 x K] . B[N x K]^T per tile of 128 rows (cells); N, K multiples of 16, N <= 256,
// K <= 256. Warp-specialised and persistent over the row tiles:
//   warp 16: TMA producer. For every K chunk of up to 64 elements it loads, into one stage of a
//     4-deep shared-memory ring, the A chunk (128 rows) and the B chunk (N rows) as boxes of
//     8 elements x rows from 2D tensor maps; a box lands as rows x 16 bytes, i.e. a column of core
//     matrices of the K-major layout (M/N neighbours 128 bytes apart, K neighbours one box apart).
//     Rows past M read as zeros.
//   warp 17: MMA issuer. Waits for a stage, issues its tcgen05.mma (K = 16 each) into one of two TMEM
//     accumulators (256 columns each), and tcgen05.commit frees the stage when they complete;
//     after a tile's last chunk a commit marks the accumulator full.
//   warps 0-15: epilogue. Read the full accumulator (warp w: TMEM lanes 32(w%4)..32(w%4)+31, the
//     (w/4)-th quarter of the columns), apply the epilogue, store, and hand the accumulator back,
//     while the next tile accumulates in the other.
// Epilogues:
//   0: z = D + bias -> Z (BF16), H = SiLU(z) (BF16)
//   1: y = D + bias -> Y (FP32)
//   2: dZ = D * SiLU'(Zp) (BF16)
struct GemmArgs {
    long long M; int N, K;
    const float *bias;
    bf16 *Z, *H; float *Y; long long ldo;
    const bf16 *Zp; bf16 *dZ;
    int *err;
};

constexpr int kTcSmem = 200 * 1024;              // one CTA per SM (and so at most 512 TMEM columns in use)
constexpr int kStages = 4, kChunk = 64;
constexpr int kEpiWarps = 16;                    // four per TMEM lane quadrant
constexpr int kStageA = 128 * kChunk * 2, kStageB = 256 * kChunk * 2;

__host__ __device__ inline int tmem_cols(int n) { int c = 32; while (c < n) c <<= 1; return c; }

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

template <int EPI>
__global__ void __launch_bounds__(32 * (kEpiWarps + 2), 1) k_mlp_gemm(const __grid_constant__ CUtensorMap tmA,
                                                     const __grid_constant__ CUtensorMap tmB, GemmArgs g)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char *ring = sm;                                           // kStages x (A | B)
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + kStages * (kStageA + kStageB));
    // bars: full[kStages], empty[kStages], acc_full[2], acc_empty[2]
    uint32_t *slot = reinterpret_cast<uint32_t *>(bars + 2 * kStages + 4);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t bar0 = smem_u32(bars);
    auto full = [&](int s) { return bar0 + 8u * (uint32_t)s; };
    auto empty = [&](int s) { return bar0 + 8u * (uint32_t)(kStages + s); };
    auto accf = [&](int a) { return bar0 + 8u * (uint32_t)(2 * kStages + a); };
    auto acce = [&](int a) { return bar0 + 8u * (uint32_t)(2 * kStages + 2 + a); };
    if (warp == kEpiWarps) tmem_alloc(smem_u32(slot), 512);
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; s++) { mbar_init(full(s), 1); mbar_init(empty(s), 1); }
        for (int a = 0; a < 2; a++) { mbar_init(accf(a), 1); mbar_init(acce(a), kEpiWarps); }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *slot;
    const int chunk = g.K < kChunk ? g.K : kChunk, nchunk = g.K / chunk, nk8 = chunk / 8;
    const long long tiles = (g.M + 127) / 128;
    bool failed = false;
    if (warp == kEpiWarps) {
        if (lane == 0) {
            const uint32_t bytes = (uint32_t)nk8 * (128u + (uint32_t)g.N) * 16u;
            long long it = 0;
            for (long long t = blockIdx.x; t < tiles && !failed; t += gridDim.x)
                for (int kc = 0; kc < nchunk; kc++, it++) {
                    const int s = (int)(it % kStages);
                    const uint32_t ph = (uint32_t)((it / kStages) & 1);
                    if (!mbar_wait_bounded(empty(s), ph ^ 1u)) { failed = true; break; }
                    mbar_expect_tx(full(s), bytes);
                    const uint32_t a_s = smem_u32(ring + (size_t)s * (kStageA + kStageB));
                    const uint32_t b_s = a_s + kStageA;
                    for (int k8 = 0; k8 < nk8; k8++) {
                        const int x = kc * chunk + k8 * 8;
                        tma_load_2d(a_s + (uint32_t)k8 * 128u * 16u, &tmA, x, (int)(t * 128), full(s));
                        tma_load_2d(b_s + (uint32_t)k8 * (uint32_t)g.N * 16u, &tmB, x, 0, full(s));
                    }
                }
        }
    } else if (warp == kEpiWarps + 1) {
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(128, g.N);
            long long it = 0, ai = 0;
            for (long long t = blockIdx.x; t < tiles && !failed; t += gridDim.x, ai++) {
                const int a = (int)(ai & 1);
                if (!mbar_wait_bounded(acce(a), (uint32_t)(((ai >> 1) & 1) ^ 1))) { failed = true; break; }
                tc_fence_after();
                for (int kc = 0; kc < nchunk; kc++, it++) {
                    const int s = (int)(it % kStages);
                    if (!mbar_wait_bounded(full(s), (uint32_t)((it / kStages) & 1))) { failed = true; break; }
                    tc_fence_after();
                    const uint32_t a_s = smem_u32(ring + (size_t)s * (kStageA + kStageB));
                    const uint32_t b_s = a_s + kStageA;
                    for (int ks = 0; ks < chunk / 16; ks++)
                        mma_bf16(tmem + (uint32_t)(a * 256), smem_desc(a_s + (uint32_t)ks * 2u * 2048u, 2048u, 128u),
                                 smem_desc(b_s + (uint32_t)ks * 2u * (uint32_t)g.N * 16u, (uint32_t)g.N * 16u, 128u), idesc,
                                 (kc > 0 || ks > 0) ? 1u : 0u);
                    mma_commit(empty(s));
                }
                if (failed) break;
                mma_commit(accf(a));
            }
        }
    } else {
        long long ai = 0;
        for (long long t = blockIdx.x; t < tiles; t += gridDim.x, ai++) {
            const int a = (int)(ai & 1);
            const bool ok = mbar_wait_bounded(accf(a), (uint32_t)((ai >> 1) & 1));
            tc_fence_after();
            if (!ok) { failed = true; break; }
            const int quad = warp & 3;
            const int cols = g.N >= 64 ? g.N / 4 : 16;        // a quarter of the columns, at least 16
            const int cbeg = (warp >> 2) * cols, cend = cbeg + cols < g.N ? cbeg + cols : g.N;
            const long long row = t * 128 + quad * 32 + lane;
            const bool live = row < g.M;
            for (int c0 = cbeg; c0 < cend; c0 += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(a * 256 + c0), v);
                if (!live) continue;
                if constexpr (EPI == 0) {
                    alignas(16) bf16 zo[16], ho[16];
#pragma unroll
                    for (int i = 0; i < 16; i++) {
                        const float z = v[i] + g.bias[c0 + i];
                        zo[i] = __float2bfloat16_rn(z);
                        ho[i] = __float2bfloat16_rn(z * sigmoidf_(z));
                    }
                    uint4 *zp = reinterpret_cast<uint4 *>(g.Z + row * g.ldo + c0);
                    uint4 *hp = reinterpret_cast<uint4 *>(g.H + row * g.ldo + c0);
                    zp[0] = reinterpret_cast<uint4 *>(zo)[0]; zp[1] = reinterpret_cast<uint4 *>(zo)[1];
                    hp[0] = reinterpret_cast<uint4 *>(ho)[0]; hp[1] = reinterpret_cast<uint4 *>(ho)[1];
                } else if constexpr (EPI == 1) {
                    float4 *yp = reinterpret_cast<float4 *>(g.Y + row * g.ldo + c0);
#pragma unroll
                    for (int i = 0; i < 4; i++)
                        yp[i] = make_float4(v[4 * i] + g.bias[c0 + 4 * i], v[4 * i + 1] + g.bias[c0 + 4 * i + 1],
                                            v[4 * i + 2] + g.bias[c0 + 4 * i + 2], v[4 * i + 3] + g.bias[c0 + 4 * i + 3]);
                } else {
                    alignas(16) bf16 zi[16], dz[16];
                    const uint4 *zs = reinterpret_cast<const uint4 *>(g.Zp + row * g.ldo + c0);
                    reinterpret_cast<uint4 *>(zi)[0] = zs[0];
                    reinterpret_cast<uint4 *>(zi)[1] = zs[1];
#pragma unroll
                    for (int i = 0; i < 16; i++) {
                        const float z = __bfloat162float(zi[i]);
                        const float sg = sigmoidf_(z);
                        dz[i] = __float2bfloat16_rn(v[i] * (sg * (1.0f + z * (1.0f - sg))));
                    }
                    uint4 *dp = reinterpret_cast<uint4 *>(g.dZ + row * g.ldo + c0);
                    dp[0] = reinterpret_cast<uint4 *>(dz)[0]; dp[1] = reinterpret_cast<uint4 *>(dz)[1];
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(acce(a));
        }
    }
    if (failed) atomicOr(g.err, 1);
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == kEpiWarps) tmem_dealloc(tmem, 512);
}

// ---------------------------------------------------------------- inference, all layers fused
// Y[rows x 16] = the whole network on X[rows x 64], per tile of 128 rows, the activations kept on
// chip: the tile's activations live in one shared-memory buffer in the K-major core-matrix layout
// (8-column groups 2 KB apart, rows 16 B apart), each layer's accumulator in TMEM. Roles as in
// k_mlp_gemm, persistent over the tiles:
//   warp 16: TMA producer. Loads the tile's features into the activation buffer once the previous
//     tile's last layer has read it, and streams the weights, 64-column chunk by chunk, layer by
//     layer, through a 3-stage ring (the same chunks for every tile; they stay in L2).
//   warp 17: MMA issuer. Per layer: waits for the epilogue of the layer before (its outputs are this
//     layer's inputs, and it has read the accumulator out), issues the layer's MMAs with A from the
//     activation buffer, commits the accumulator; after the last layer it frees the buffer.
//   warps 0-15: epilogue. Per layer: bias and SiLU of the accumulator, rounded to BF16 and written
//     over the activation buffer (hidden layers), or bias and FP32 rows of Y (the output layer).
// The arithmetic is the layer-by-layer forward's (same MMA order, same epilogue), so the outputs
// are the same bits; nothing but X and Y crosses HBM.
struct InferArgs {
    long long M;
    const float *bias[kWsLayers];
    float *Y;
    int *err;
};
constexpr int kInfStages = 3;
constexpr int kInfH = 128 * kWsHidden * 2;                  // 64 KB of activations
constexpr int kInfSmem = kInfH + kInfStages * kStageB + 256;
__host__ __device__ constexpr int inf_n(int l) { return l == kWsLayers - 1 ? kWsOut : kWsHidden; }
__host__ __device__ constexpr int inf_chunks(int l) { return l == 0 ? kWsIn / kChunk : kWsHidden / kChunk; }

__global__ void __launch_bounds__(32 * (kEpiWarps + 2), 1) k_mlp_infer(
    const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tw0, const __grid_constant__ CUtensorMap tw1,
    const __grid_constant__ CUtensorMap tw2, const __grid_constant__ CUtensorMap tw3, const __grid_constant__ CUtensorMap tw4,
    const __grid_constant__ CUtensorMap tw5, InferArgs g)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char *hbuf = sm;                                           // activations
    unsigned char *ring = sm + kInfH;                                   // weight chunks
    uint64_t *bars = reinterpret_cast<uint64_t *>(ring + kInfStages * kStageB);
    // bars: full[3], empty[3], x_full, h_free, acc_full, h_ready
    uint32_t *slot = reinterpret_cast<uint32_t *>(bars + 2 * kInfStages + 4);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t bar0 = smem_u32(bars);
    auto full = [&](int s) { return bar0 + 8u * (uint32_t)s; };
    auto empty = [&](int s) { return bar0 + 8u * (uint32_t)(kInfStages + s); };
    const uint32_t x_full = bar0 + 8u * (2 * kInfStages), h_free = x_full + 8u, acc_full = x_full + 16u,
                   h_ready = x_full + 24u;
    const uint32_t hb = smem_u32(hbuf);
    if (warp == kEpiWarps) tmem_alloc(smem_u32(slot), 256);
    if (threadIdx.x == 0) {
        for (int s = 0; s < kInfStages; s++) { mbar_init(full(s), 1); mbar_init(empty(s), 1); }
        mbar_init(x_full, 1);
        mbar_init(h_free, 1);
        mbar_init(acc_full, 1);
        mbar_init(h_ready, kEpiWarps);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *slot;
    const long long tiles = (g.M + 127) / 128;
    bool failed = false;
    if (warp == kEpiWarps) {
        if (lane == 0) {
            long long it = 0, ti = 0;
            for (long long t = blockIdx.x; t < tiles && !failed; t += gridDim.x, ti++) {
                if (!mbar_wait_bounded(h_free, (uint32_t)((ti & 1) ^ 1))) { failed = true; break; }
                mbar_expect_tx(x_full, (uint32_t)(kWsIn / 8) * 128u * 16u);
                for (int k8 = 0; k8 < kWsIn / 8; k8++) tma_load_2d(hb + (uint32_t)k8 * 2048u, &tmX, k8 * 8, (int)(t * 128), x_full);
                for (int l = 0; l < kWsLayers && !failed; l++) {
                    const CUtensorMap *wm = l == 0 ? &tw0 : l == 1 ? &tw1 : l == 2 ? &tw2 : l == 3 ? &tw3 : l == 4 ? &tw4 : &tw5;
                    const int n = inf_n(l);
                    for (int kc = 0; kc < inf_chunks(l); kc++, it++) {
                        const int s = (int)(it % kInfStages);
                        if (!mbar_wait_bounded(empty(s), (uint32_t)(((it / kInfStages) & 1) ^ 1))) { failed = true; break; }
                        mbar_expect_tx(full(s), 8u * (uint32_t)n * 16u);
                        const uint32_t b_s = smem_u32(ring + (size_t)s * kStageB);
                        for (int k8 = 0; k8 < 8; k8++) tma_load_2d(b_s + (uint32_t)k8 * (uint32_t)n * 16u, wm, kc * kChunk + k8 * 8, 0, full(s));
                    }
                }
            }
        }
    } else if (warp == kEpiWarps + 1) {
        if (lane == 0) {
            long long it = 0, ti = 0, hu = 0;
            for (long long t = blockIdx.x; t < tiles && !failed; t += gridDim.x, ti++) {
                if (!mbar_wait_bounded(x_full, (uint32_t)(ti & 1))) { failed = true; break; }
                for (int l = 0; l < kWsLayers && !failed; l++) {
                    // the epilogue of the layer before has written this layer's inputs and read the accumulator
                    if (ti > 0 || l > 0) {
                        if (!mbar_wait_bounded(h_ready, (uint32_t)(hu & 1))) { failed = true; break; }
                        hu++;
                    }
                    tc_fence_after();
                    const int n = inf_n(l);
                    const uint32_t idesc = idesc_bf16(128, n);
                    for (int kc = 0; kc < inf_chunks(l); kc++, it++) {
                        const int s = (int)(it % kInfStages);
                        if (!mbar_wait_bounded(full(s), (uint32_t)((it / kInfStages) & 1))) { failed = true; break; }
                        tc_fence_after();
                        const uint32_t b_s = smem_u32(ring + (size_t)s * kStageB);
                        for (int ks = 0; ks < kChunk / 16; ks++)
                            mma_bf16(tmem, smem_desc(hb + (uint32_t)(kc * (kChunk / 16) + ks) * 2u * 2048u, 2048u, 128u),
                                     smem_desc(b_s + (uint32_t)ks * 2u * (uint32_t)n * 16u, (uint32_t)n * 16u, 128u), idesc,
                                     (kc > 0 || ks > 0) ? 1u : 0u);
                        mma_commit(empty(s));
                    }
                    if (failed) break;
                    mma_commit(acc_full);
                    if (l == kWsLayers - 1) mma_commit(h_free);
                }
            }
        }
    } else {
        long long au = 0;
        const int quad = warp & 3;
        const int r = quad * 32 + lane;                                // the TMEM lane = row of the tile
        for (long long t = blockIdx.x; t < tiles && !failed; t += gridDim.x) {
            const long long row = t * 128 + r;
            for (int l = 0; l < kWsLayers; l++, au++) {
                const bool ok = mbar_wait_bounded(acc_full, (uint32_t)(au & 1));
                tc_fence_after();
                if (!ok) { failed = true; break; }
                const int n = inf_n(l);
                const int cols = n >= 64 ? n / 4 : 16;
                const int cbeg = (warp >> 2) * cols, cend = cbeg + cols < n ? cbeg + cols : n;
                const float *bias = g.bias[l];
                for (int c0 = cbeg; c0 < cend; c0 += 16) {
                    float v[16];
                    tmem_ld16(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)c0, v);
                    if (l < kWsLayers - 1) {
                        alignas(16) bf16 ho[16];
#pragma unroll
                        for (int i = 0; i < 16; i++) {
                            const float z = v[i] + bias[c0 + i];
                            ho[i] = __float2bfloat16_rn(z * sigmoidf_(z));
                        }
                        uint4 *h0 = reinterpret_cast<uint4 *>(hbuf + (size_t)(c0 / 8) * 2048 + (size_t)r * 16);
                        uint4 *h1 = reinterpret_cast<uint4 *>(hbuf + (size_t)(c0 / 8 + 1) * 2048 + (size_t)r * 16);
                        *h0 = reinterpret_cast<uint4 *>(ho)[0];
                        *h1 = reinterpret_cast<uint4 *>(ho)[1];
                    } else if (row < g.M) {
                        float4 *yp = reinterpret_cast<float4 *>(g.Y + row * kWsOut + c0);
#pragma unroll
                        for (int i = 0; i < 4; i++)
                            yp[i] = make_float4(v[4 * i] + bias[c0 + 4 * i], v[4 * i + 1] + bias[c0 + 4 * i + 1],
                                                v[4 * i + 2] + bias[c0 + 4 * i + 2], v[4 * i + 3] + bias[c0 + 4 * i + 3]);
                    }
                }
                fence_proxy_async();                                   // the activations, for the tensor cores
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(h_ready);
            }
        }
    }
    if (failed) atomicOr(g.err, 1);
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == kEpiWarps) tmem_dealloc(tmem, 256);
}

// ---------------------------------------------------------------- the weight gradient
// part[(ay * gridDim.x + bx)][a][b] = sum over the CTA's cells of Xa[cell][128 ay + a] Xb[cell][b]
// (a < 128, b < Nb): the cells are the product's K. Both operands are MN-major: a TMA box of 8
// features x 64 cells lands as 64 rows of 16 bytes, i.e. eight core matrices of the MN-major
// no-swizzle layout stacked along K (128 bytes apart), the next 8 features one box (1024 bytes)
// further. Warp 4 loads (4-stage ring), warp 5 issues the MMAs into one accumulator, warps 0-3
// write it out once the CTA's cells are done.
struct WgradArgs {
    long long M; int Nb; long long chunk;
    float *part;
    int *err;
};

constexpr int kWgCells = 64;
constexpr int kWgStageA = 128 * kWgCells * 2, kWgStageB = 256 * kWgCells * 2;

__global__ void __launch_bounds__(192, 1) k_mlp_wgrad(const __grid_constant__ CUtensorMap tmA,
                                                      const __grid_constant__ CUtensorMap tmB, WgradArgs g)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char *ring = sm;
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + kStages * (kWgStageA + kWgStageB));
    uint32_t *slot = reinterpret_cast<uint32_t *>(bars + 2 * kStages + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t bar0 = smem_u32(bars);
    auto full = [&](int s) { return bar0 + 8u * (uint32_t)s; };
    auto empty = [&](int s) { return bar0 + 8u * (uint32_t)(kStages + s); };
    const uint32_t accf = bar0 + 8u * (uint32_t)(2 * kStages);
    const uint32_t ncols = (uint32_t)tmem_cols(g.Nb);
    if (warp == 4) tmem_alloc(smem_u32(slot), ncols);
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; s++) { mbar_init(full(s), 1); mbar_init(empty(s), 1); }
        mbar_init(accf, 1);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *slot;
    const long long c_begin = (long long)blockIdx.x * g.chunk;
    const long long c_end = c_begin + g.chunk < g.M ? c_begin + g.chunk : g.M;
    const int nch = c_end > c_begin ? (int)((c_end - c_begin + kWgCells - 1) / kWgCells) : 0;
    const int a0 = (int)blockIdx.y * 128;
    bool failed = false;
    if (warp == 4) {
        if (lane == 0) {
            const uint32_t bytes = (uint32_t)(16 + g.Nb / 8) * 1024u;
            for (int it = 0; it < nch; it++) {
                const int s = it % kStages;
                if (!mbar_wait_bounded(empty(s), (uint32_t)(((it / kStages) & 1) ^ 1))) { failed = true; break; }
                mbar_expect_tx(full(s), bytes);
                const uint32_t a_s = smem_u32(ring + (size_t)s * (kWgStageA + kWgStageB));
                const uint32_t b_s = a_s + kWgStageA;
                const int y = (int)(c_begin + (long long)it * kWgCells);
                for (int a8 = 0; a8 < 16; a8++) tma_load_2d(a_s + (uint32_t)a8 * 1024u, &tmA, a0 + a8 * 8, y, full(s));
                for (int b8 = 0; b8 < g.Nb / 8; b8++) tma_load_2d(b_s + (uint32_t)b8 * 1024u, &tmB, b8 * 8, y, full(s));
            }
        }
    } else if (warp == 5) {
        if (lane == 0 && nch > 0) {
            // MN-major A and B (bits 15 and 16); in 16-byte units LBO = K step (128 B), SBO = MN step (1024 B)
            const uint32_t idesc = idesc_bf16(128, g.Nb) | (1u << 15) | (1u << 16);
            for (int it = 0; it < nch && !failed; it++) {
                const int s = it % kStages;
                if (!mbar_wait_bounded(full(s), (uint32_t)((it / kStages) & 1))) { failed = true; break; }
                tc_fence_after();
                const uint32_t a_s = smem_u32(ring + (size_t)s * (kWgStageA + kWgStageB));
                const uint32_t b_s = a_s + kWgStageA;
                for (int ks = 0; ks < kWgCells / 16; ks++)
                    mma_bf16(tmem, smem_desc(a_s + (uint32_t)ks * 256u, 128u, 1024u), smem_desc(b_s + (uint32_t)ks * 256u, 128u, 1024u),
                             idesc, (it > 0 || ks > 0) ? 1u : 0u);
                mma_commit(empty(s));
            }
            if (!failed) mma_commit(accf);
        }
    } else {
        float *out = g.part + ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * 128 * g.Nb;
        const int a = warp * 32 + lane;
        bool ok = true;
        if (nch > 0) {
            ok = mbar_wait_bounded(accf, 0u);
            tc_fence_after();
        }
        if (!ok) failed = true;
        else
            for (int c0 = 0; c0 < g.Nb; c0 += 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
                for (int i = 0; i < 16; i++) out[(size_t)a * g.Nb + c0 + i] = nch > 0 ? v[i] : 0.0f;
            }
    }
    if (failed) atomicOr(g.err, 1);
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 4) tmem_dealloc(tmem, ncols);
}

// dst = scale * sum over the CTAs (fixed order); trans stores element (a, b) at b * Wa + a
__global__ void k_wgrad_reduce(const float *part, int gx, int Wa, int Nb, float scale, int trans, float *dst)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= Wa * Nb) return;
    const int a = t / Nb, b = t - a * Nb, ay = a >> 7, al = a & 127;
    float s = 0.0f;
    for (int bx = 0; bx < gx; bx++) s += part[((size_t)ay * gx + bx) * 128 * Nb + (size_t)al * Nb + b];
    dst[trans ? (size_t)b * Wa + a : (size_t)a * Nb + b] = scale * s;
}

// column sums of X[M x W] (W <= 256): per block partial sums, then a fixed-order reduction
__global__ void __launch_bounds__(256) k_colsum_partial(const bf16 *X, long long M, int W, long long rows_per, float *part)
{
    const int c = threadIdx.x;
    if (c >= W) return;
    const long long r0 = (long long)blockIdx.x * rows_per, r1 = std::min(M, r0 + rows_per);
    float s = 0.0f;
    for (long long r = r0; r < r1; r++) s += __bfloat162float(X[r * W + c]);
    part[(size_t)blockIdx.x * W + c] = s;
}
__global__ void k_colsum_reduce(const float *part, int nb, int W, float scale, float *dst)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= W) return;
    float s = 0.0f;
    for (int b = 0; b < nb; b++) s += part[(size_t)b * W + c];
    dst[c] = scale * s;
}

// ---------------------------------------------------------------- features, loss, optimiser
// normalisation constants: coord min[3], max[3] (axial z, radius, pitch angle); parameter
// mean[3], std[3]; target mean[6], std[6]
__device__ __forceinline__ void ws_features(const float *nrm, float z, float r, float th, const float *pr, bf16 *out)
{
    float c[3] = {z, r, th};
#pragma unroll
    for (int d = 0; d < 3; d++) c[d] = (c[d] - nrm[d]) / (nrm[3 + d] - nrm[d]);
    int o = 0;
#pragma unroll
    for (int d = 0; d < 3; d++)
#pragma unroll
        for (int f = 0; f < 8; f++) {
            float s, co;
            sincospif((float)(1 << f) * c[d], &s, &co);
            out[o++] = __float2bfloat16_rn(s);
            out[o++] = __float2bfloat16_rn(co);
        }
#pragma unroll
    for (int d = 0; d < 3; d++) out[o++] = __float2bfloat16_rn(c[d]);
#pragma unroll
    for (int q = 0; q < 3; q++) out[o++] = __float2bfloat16_rn((pr[q] - nrm[6 + q]) / nrm[9 + q]);
    for (; o < kWsIn; o++) out[o] = __float2bfloat16_rn(0.0f);
}

// training sample layout: z, r, theta, params[3], targets[6]
constexpr int kWsSample = 12;

__device__ __forceinline__ unsigned long long mix64(unsigned long long x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__global__ void k_ws_gather(const float *set, long long n_set, unsigned long long seed, long long M, const float *nrm,
                            bf16 *X0, float *T)
{
    const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const long long s = (long long)(mix64(seed ^ (unsigned long long)m * 0xD1B54A32D192ED03ull) % (unsigned long long)n_set);
    const float *p = set + s * kWsSample;
    alignas(16) bf16 f[kWsIn];
    ws_features(nrm, p[0], p[1], p[2], p + 3, f);
    uint4 *dst = reinterpret_cast<uint4 *>(X0 + m * kWsIn);
#pragma unroll
    for (int q = 0; q < kWsIn / 8; q++) dst[q] = reinterpret_cast<uint4 *>(f)[q];
#pragma unroll
    for (int o = 0; o < kWsOutUsed; o++) T[m * 8 + o] = (p[6 + o] - nrm[12 + o]) / nrm[18 + o];
    T[m * 8 + 6] = 0.0f;
    T[m * 8 + 7] = 0.0f;
}

// dY = 2 (y - t) / 6 on the six used outputs (the 1 / M of the mean is applied to the gradients);
// per block, the sum of squared errors
__global__ void __launch_bounds__(256) k_ws_loss(const float *Y, const float *T, long long M, bf16 *dY, float *part)
{
    const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    float se = 0.0f;
    if (m < M) {
        alignas(16) bf16 d[kWsOut];
#pragma unroll
        for (int o = 0; o < kWsOut; o++) {
            float g = 0.0f;
            if (o < kWsOutUsed) {
                const float e = Y[m * kWsOut + o] - T[m * 8 + o];
                se += e * e;
                g = 2.0f * e / (float)kWsOutUsed;
            }
            d[o] = __float2bfloat16_rn(g);
        }
        reinterpret_cast<uint4 *>(dY + m * kWsOut)[0] = reinterpret_cast<uint4 *>(d)[0];
        reinterpret_cast<uint4 *>(dY + m * kWsOut)[1] = reinterpret_cast<uint4 *>(d)[1];
    }
    __shared__ float sh[256];
    sh[threadIdx.x] = se;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, long long n, float lr, float b1, float b2, float eps,
                       float c1, float c2)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi, vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// BF16 copies of a layer's weights, as stored [N x K] and transposed [K x N]
__global__ void k_ws_weights_bf16(const float *w, int N, int K, bf16 *wb, bf16 *wt)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * K) return;
    const int n = t / K, k = t - n * K;
    const bf16 b = __float2bfloat16_rn(w[t]);
    wb[t] = b;
    wt[(size_t)k * N + n] = b;
}

__global__ void k_f32_to_bf16(const float *x, long long n, bf16 *y)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __float2bfloat16_rn(x[i]);
}

// ---------------------------------------------------------------- cells of a solver's fine level
// cell t of the batch: slot by bisection of the prefix counts, then (i, j, k) with k fastest
__device__ __forceinline__ int ws_cell(const Lvl *lv, const long long *off, int nslot, long long t, long long &p)
{
    int lo = 0, hi = nslot - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const Lvl L = lv[lo];
    const long long q = t - off[lo];
    const int nk = L.KM - 1, nj = L.JM - 1;
    const int k = (int)(q % nk) + 1;
    const long long r = q / nk;
    const int j = (int)(r % nj) + 1, i = (int)(r / nj) + 1;
    p = ix(L, i, j, k);
    return lo;
}

struct CellsArgs {
    const Lvl *lv; const long long *off; int nslot;
    const int *slot_case; const float *params;           // per case
    const double *cc0, *cc1, *cc2;
    double *cv0, *cv1, *cv2, *cv3, *cv4;
    const void *mut; int fp32;
};

// training samples from the current fields of cells t0 .. t0+n
__global__ void k_ws_collect(CellsArgs a, long long t0, long long n, float *out)
{
    const long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= n) return;
    long long p;
    const int s = ws_cell(a.lv, a.off, a.nslot, t0 + u, p);
    const double x = a.cc0[p], y = a.cc1[p], z = a.cc2[p];
    float *o = out + u * kWsSample;
    o[0] = (float)z;
    o[1] = (float)sqrt(x * x + y * y);
    o[2] = (float)atan2(y, x);
    const float *pr = a.params + (size_t)a.slot_case[s] * kWsParams;
    o[3] = pr[0]; o[4] = pr[1]; o[5] = pr[2];
    o[6] = (float)a.cv0[p]; o[7] = (float)a.cv1[p]; o[8] = (float)a.cv2[p]; o[9] = (float)a.cv3[p]; o[10] = (float)a.cv4[p];
    o[11] = a.fp32 ? ((const float *)a.mut)[p] : (float)((const double *)a.mut)[p];
}

__global__ void k_ws_cell_features(CellsArgs a, long long t0, long long n, const float *nrm, bf16 *X0)
{
    const long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= n) return;
    long long p;
    const int s = ws_cell(a.lv, a.off, a.nslot, t0 + u, p);
    const double x = a.cc0[p], y = a.cc1[p], z = a.cc2[p];
    alignas(16) bf16 f[kWsIn];
    ws_features(nrm, (float)z, (float)sqrt(x * x + y * y), (float)atan2(y, x), a.params + (size_t)a.slot_case[s] * kWsParams, f);
    uint4 *dst = reinterpret_cast<uint4 *>(X0 + u * kWsIn);
#pragma unroll
    for (int q = 0; q < kWsIn / 8; q++) dst[q] = reinterpret_cast<uint4 *>(f)[q];
}

__global__ void k_ws_write_cv(CellsArgs a, long long t0, long long n, const float *nrm, const float *Y)
{
    const long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= n) return;
    long long p;
    ws_cell(a.lv, a.off, a.nslot, t0 + u, p);
    const float *y = Y + u * kWsOut;
    double q[5];
#pragma unroll
    for (int c = 0; c < 5; c++) q[c] = (double)(y[c] * nrm[18 + c] + nrm[12 + c]);
    a.cv0[p] = q[0]; a.cv1[p] = q[1]; a.cv2[p] = q[2]; a.cv3[p] = q[3]; a.cv4[p] = q[4];
}

// per block: min, max, sum, sum of squares of each of the 12 sample columns
__global__ void __launch_bounds__(256) k_ws_stats(const float *set, long long n, double *part)
{
    double mn[kWsSample], mx[kWsSample], s1[kWsSample], s2[kWsSample];
    for (int c = 0; c < kWsSample; c++) { mn[c] = 1e300; mx[c] = -1e300; s1[c] = 0.0; s2[c] = 0.0; }
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        for (int c = 0; c < kWsSample; c++) {
            const double v = set[i * kWsSample + c];
            mn[c] = fmin(mn[c], v); mx[c] = fmax(mx[c], v); s1[c] += v; s2[c] += v * v;
        }
    __shared__ double sh[256];
    for (int c = 0; c < kWsSample; c++)
        for (int kind = 0; kind < 4; kind++) {
            double v = kind == 0 ? mn[c] : kind == 1 ? mx[c] : kind == 2 ? s1[c] : s2[c];
            sh[threadIdx.x] = v;
            __syncthreads();
            for (int w = 128; w > 0; w >>= 1) {
                if ((int)threadIdx.x < w) {
                    const double o = sh[threadIdx.x + w];
                    sh[threadIdx.x] = kind == 0 ? fmin(sh[threadIdx.x], o) : kind == 1 ? fmax(sh[threadIdx.x], o) : sh[threadIdx.x] + o;
                }
                __syncthreads();
            }
            if (threadIdx.x == 0) part[((size_t)blockIdx.x * kWsSample + c) * 4 + kind] = sh[0];
            __syncthreads();
        }
}

// ---------------------------------------------------------------- host side
// 2D tensor map of a row-major BF16 matrix [rows x cols] (row stride ld elements) read in boxes
// of 8 columns (16 bytes) x box_rows rows; rows past the end read as zeros
static CUtensorMap tensor_map_rows(const bf16 *base, long long rows, int cols, long long ld, int box_rows)
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        WCK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q));
        if (!f || q != cudaDriverEntryPointSuccess) throw std::runtime_error("cuTensorMapEncodeTiled is not available");
        encode = (PFN_cuTensorMapEncodeTiled_v12000)f;
    }
    if (((uintptr_t)base & 15) || ((ld * 2) & 15) || (cols & 7) || box_rows < 1 || box_rows > 256)
        throw std::runtime_error("tensor map: misaligned matrix or box");
    CUtensorMap m;
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {8u, (cuuint32_t)box_rows};
    const cuuint32_t es[2] = {1u, 1u};
    const CUresult r = encode(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void *)base, dims, strides, box, es,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed");
    return m;
}

static const int kN[kWsLayers] = {kWsHidden, kWsHidden, kWsHidden, kWsHidden, kWsHidden, kWsOut};
static const int kK[kWsLayers] = {kWsIn, kWsHidden, kWsHidden, kWsHidden, kWsHidden, kWsHidden};

static size_t w_off(int l)
{
    size_t o = 0;
    for (int q = 0; q < l; q++) o += (size_t)kN[q] * kK[q] + kN[q];
    return o;
}
static size_t b_off(int l) { return w_off(l) + (size_t)kN[l] * kK[l]; }

struct WarmStart::Impl {
    cudaStream_t st = nullptr;
    int n_sm = 0;
    float *P = nullptr, *G = nullptr, *Mo = nullptr, *Vo = nullptr;
    bf16 *Wb[kWsLayers] = {}, *Wt[kWsLayers] = {};
    int *err = nullptr;
    float *nrm_d = nullptr;
    float nrm[kWsNorm] = {};
    bool have_norm = false;
    int adam_t = 0;
    // activations for up to cap rows
    long long cap = 0;
    bf16 *X0 = nullptr, *Z[5] = {}, *H[5] = {}, *dY = nullptr, *dZa = nullptr, *dZb = nullptr;
    float *Y = nullptr, *T = nullptr, *part = nullptr, *cpart = nullptr, *lpart = nullptr;
    size_t part_n = 0;
    // training set
    float *set = nullptr;
    long long set_cap = 0;
    unsigned long long rng = 0;

    void ensure(long long M)
    {
        if (M <= cap) return;
        release_acts();
        cap = std::max(M, (long long)4096);
        auto abf = [&](long long n) { bf16 *p; WCK(cudaMalloc(&p, sizeof(bf16) * n)); return p; };
        auto af = [&](long long n) { float *p; WCK(cudaMalloc(&p, sizeof(float) * n)); return p; };
        X0 = abf(cap * kWsIn);
        for (int l = 0; l < 5; l++) { Z[l] = abf(cap * kWsHidden); H[l] = abf(cap * kWsHidden); }
        dY = abf(cap * kWsOut);
        dZa = abf(cap * kWsHidden);
        dZb = abf(cap * kWsHidden);
        Y = af(cap * kWsOut);
        T = af(cap * 8);
        lpart = af((cap + 255) / 256);
    }
    void release_acts()
    {
        cudaFree(X0); X0 = nullptr;
        for (int l = 0; l < 5; l++) { cudaFree(Z[l]); cudaFree(H[l]); Z[l] = H[l] = nullptr; }
        cudaFree(dY); cudaFree(dZa); cudaFree(dZb); cudaFree(Y); cudaFree(T); cudaFree(lpart);
        dY = dZa = dZb = nullptr; Y = T = lpart = nullptr;
        cap = 0;
    }

    template <int EPI>
    void gemm(const bf16 *A, long long lda, int l_w, bool transposed, long long M, int N, int K, const float *bias, bf16 *Zo,
              bf16 *Ho, float *Yo, long long ldo, const bf16 *Zp, bf16 *dZ)
    {
        if (M <= 0) return;
        GemmArgs g{};
        g.M = M; g.N = N; g.K = K;
        g.bias = bias; g.Z = Zo; g.H = Ho; g.Y = Yo; g.ldo = ldo; g.Zp = Zp; g.dZ = dZ; g.err = err;
        const CUtensorMap ta = tensor_map_rows(A, M, K, lda, 128);
        const CUtensorMap tb = tensor_map_rows(transposed ? Wt[l_w] : Wb[l_w], N, K, K, N);
        const long long tiles = (M + 127) / 128;
        const int grid = (int)std::min<long long>(tiles, n_sm);
        k_mlp_gemm<EPI><<<grid, 32 * (kEpiWarps + 2), kTcSmem, st>>>(ta, tb, g);
        WCK(cudaGetLastError());
    }

    void wgrad(const bf16 *Xa, long long lda, const bf16 *Xb, int Nb, long long M, float scale, int trans, float *dst)
    {
        const int Wa = kWsHidden;                           // every weight gradient has 256 rows on one side
        const int gy = Wa / 128;
        int gx = std::max(1, n_sm / gy);
        long long chunk = ((M + gx - 1) / gx + 63) / 64 * 64;
        gx = (int)((M + chunk - 1) / chunk);
        const size_t need = (size_t)gy * gx * 128 * Nb;
        if (need > part_n) {
            cudaFree(part);
            WCK(cudaMalloc(&part, sizeof(float) * need));
            part_n = need;
        }
        WgradArgs g{};
        g.M = M; g.Nb = Nb; g.chunk = chunk; g.part = part; g.err = err;
        const CUtensorMap ta = tensor_map_rows(Xa, M, Wa, lda, kWgCells);
        const CUtensorMap tb = tensor_map_rows(Xb, M, Nb, Nb, kWgCells);
        k_mlp_wgrad<<<dim3(gx, gy), 192, kTcSmem, st>>>(ta, tb, g);
        WCK(cudaGetLastError());
        k_wgrad_reduce<<<(Wa * Nb + 255) / 256, 256, 0, st>>>(part, gx, Wa, Nb, scale, trans, dst);
    }

    void colsum(const bf16 *X, long long M, int W, float scale, float *dst)
    {
        const int nb = (int)std::min<long long>(std::max<long long>(1, (M + 255) / 256), 512);
        const long long rows = (M + nb - 1) / nb;
        if (!cpart) WCK(cudaMalloc(&cpart, sizeof(float) * 512 * 256));
        k_colsum_partial<<<nb, 256, 0, st>>>(X, M, W, rows, cpart);
        k_colsum_reduce<<<1, 256, 0, st>>>(cpart, nb, W, scale, dst);
    }

    void refresh_bf16()
    {
        for (int l = 0; l < kWsLayers; l++)
            k_ws_weights_bf16<<<(kN[l] * kK[l] + 255) / 256, 256, 0, st>>>(P + w_off(l), kN[l], kK[l], Wb[l], Wt[l]);
    }

    // rows of X0 -> Y with every layer fused in one kernel (inference: no activations kept)
    void infer(long long M)
    {
        if (M <= 0) return;
        InferArgs g{};
        g.M = M; g.Y = Y; g.err = err;
        for (int l = 0; l < kWsLayers; l++) g.bias[l] = P + b_off(l);
        const CUtensorMap tx = tensor_map_rows(X0, M, kWsIn, kWsIn, 128);
        CUtensorMap tw[kWsLayers];
        for (int l = 0; l < kWsLayers; l++) tw[l] = tensor_map_rows(Wb[l], kN[l], kK[l], kK[l], kN[l]);
        const long long tiles = (M + 127) / 128;
        const int grid = (int)std::min<long long>(tiles, n_sm);
        k_mlp_infer<<<grid, 32 * (kEpiWarps + 2), kInfSmem, st>>>(tx, tw[0], tw[1], tw[2], tw[3], tw[4], tw[5], g);
        WCK(cudaGetLastError());
    }

    // rows of X0 -> Y (and the hidden activations, which training needs)
    void forward(long long M)
    {
        const bf16 *in = X0;
        long long ld = kWsIn;
        for (int l = 0; l < 5; l++) {
            gemm<0>(in, ld, l, false, M, kN[l], kK[l], P + b_off(l), Z[l], H[l], nullptr, kWsHidden, nullptr, nullptr);
            in = H[l];
            ld = kWsHidden;
        }
        gemm<1>(in, ld, 5, false, M, kWsOut, kWsHidden, P + b_off(5), nullptr, nullptr, Y, kWsOut, nullptr, nullptr);
    }

    // from dY: every gradient into G (mean over the M rows)
    void backward(long long M)
    {
        const float sc = 1.0f / (float)M;
        wgrad(H[4], kWsHidden, dY, kWsOut, M, sc, 1, G + w_off(5));             // dW6 (stored transposed)
        colsum(dY, M, kWsOut, sc, G + b_off(5));
        // dZ5 = (dY . W6) * SiLU'(Z5)
        gemm<2>(dY, kWsOut, 5, true, M, kWsHidden, kWsOut, nullptr, nullptr, nullptr, nullptr, kWsHidden, Z[4], dZa);
        bf16 *cur = dZa, *nxt = dZb;
        for (int l = 4; l >= 1; l--) {
            wgrad(cur, kWsHidden, H[l - 1], kWsHidden, M, sc, 0, G + w_off(l));
            colsum(cur, M, kWsHidden, sc, G + b_off(l));
            gemm<2>(cur, kWsHidden, l, true, M, kWsHidden, kWsHidden, nullptr, nullptr, nullptr, nullptr, kWsHidden, Z[l - 1], nxt);
            std::swap(cur, nxt);
        }
        wgrad(cur, kWsHidden, X0, kWsIn, M, sc, 0, G + w_off(0));
        colsum(cur, M, kWsHidden, sc, G + b_off(0));
    }

    float loss(long long M)
    {
        const int nb = (int)((M + 255) / 256);
        k_ws_loss<<<nb, 256, 0, st>>>(Y, T, M, dY, lpart);
        std::vector<float> h(nb);
        WCK(cudaMemcpyAsync(h.data(), lpart, sizeof(float) * nb, cudaMemcpyDeviceToHost, st));
        WCK(cudaStreamSynchronize(st));
        double s = 0.0;
        for (float v : h) s += v;
        return (float)(s / ((double)M * kWsOutUsed));
    }
};

size_t WarmStart::n_params() { return w_off(kWsLayers); }

WarmStart::WarmStart(unsigned seed) : d(new Impl)
{
    int dev = 0;
    WCK(cudaGetDevice(&dev));
    WCK(cudaDeviceGetAttribute(&d->n_sm, cudaDevAttrMultiProcessorCount, dev));
    WCK(cudaStreamCreateWithFlags(&d->st, cudaStreamNonBlocking));
    WCK(cudaFuncSetAttribute(k_mlp_gemm<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
    WCK(cudaFuncSetAttribute(k_mlp_gemm<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
    WCK(cudaFuncSetAttribute(k_mlp_gemm<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
    WCK(cudaFuncSetAttribute(k_mlp_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
    WCK(cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, kInfSmem));
    const size_t np = n_params();
    WCK(cudaMalloc(&d->P, sizeof(float) * np));
    WCK(cudaMalloc(&d->G, sizeof(float) * np));
    WCK(cudaMalloc(&d->Mo, sizeof(float) * np));
    WCK(cudaMalloc(&d->Vo, sizeof(float) * np));
    WCK(cudaMemset(d->G, 0, sizeof(float) * np));
    WCK(cudaMemset(d->Mo, 0, sizeof(float) * np));
    WCK(cudaMemset(d->Vo, 0, sizeof(float) * np));
    for (int l = 0; l < kWsLayers; l++) {
        WCK(cudaMalloc(&d->Wb[l], sizeof(bf16) * kN[l] * kK[l]));
        WCK(cudaMalloc(&d->Wt[l], sizeof(bf16) * kN[l] * kK[l]));
    }
    WCK(cudaMalloc(&d->err, sizeof(int)));
    WCK(cudaMemset(d->err, 0, sizeof(int)));
    WCK(cudaMalloc(&d->nrm_d, sizeof(float) * kWsNorm));
    // Glorot-uniform weights, zero biases; the padded outputs 6..15 stay zero (their gradient is zero)
    std::mt19937 rng(seed);
    std::vector<float> h(np, 0.0f);
    for (int l = 0; l < kWsLayers; l++) {
        const float a = std::sqrt(6.0f / (float)(kK[l] + kN[l]));
        std::uniform_real_distribution<float> u(-a, a);
        for (int n = 0; n < kN[l]; n++)
            for (int k = 0; k < kK[l]; k++) {
                const float v = u(rng);
                h[w_off(l) + (size_t)n * kK[l] + k] = (l == kWsLayers - 1 && n >= kWsOutUsed) ? 0.0f : v;
            }
    }
    WCK(cudaMemcpy(d->P, h.data(), sizeof(float) * np, cudaMemcpyHostToDevice));
    d->refresh_bf16();
    d->rng = ((unsigned long long)seed << 32) ^ 0x5DEECE66Dull;
    for (int q = 0; q < kWsNorm; q++) d->nrm[q] = (q >= 3 && q < 6) || q >= 9 ? 1.0f : 0.0f;
    WCK(cudaMemcpy(d->nrm_d, d->nrm, sizeof(d->nrm), cudaMemcpyHostToDevice));
    WCK(cudaStreamSynchronize(d->st));
}

WarmStart::~WarmStart()
{
    if (!d) return;
    cudaStreamSynchronize(d->st);
    d->release_acts();
    cudaFree(d->P); cudaFree(d->G); cudaFree(d->Mo); cudaFree(d->Vo);
    for (int l = 0; l < kWsLayers; l++) { cudaFree(d->Wb[l]); cudaFree(d->Wt[l]); }
    cudaFree(d->err); cudaFree(d->nrm_d); cudaFree(d->part); cudaFree(d->cpart); cudaFree(d->set);
    cudaStreamDestroy(d->st);
    delete d;
}

int WarmStart::error_flag()
{
    int e = 0;
    WCK(cudaMemcpy(&e, d->err, sizeof(int), cudaMemcpyDeviceToHost));
    return e;
}

static CellsArgs cells_args(const FineView &v, const long long *off, const int *slot_case, const float *params)
{
    CellsArgs a{};
    a.lv = v.lv_dev; a.off = off; a.nslot = v.nslot; a.slot_case = slot_case; a.params = params;
    a.cc0 = v.cc[0]; a.cc1 = v.cc[1]; a.cc2 = v.cc[2];
    a.cv0 = v.cv[0]; a.cv1 = v.cv[1]; a.cv2 = v.cv[2]; a.cv3 = v.cv[3]; a.cv4 = v.cv[4];
    a.mut = v.mut; a.fp32 = v.fp32 ? 1 : 0;
    return a;
}

// device tables of a solver's fine cells: prefix counts per slot, slot -> case, case parameters
struct CellTables {
    DevBuf mem;
    long long *off = nullptr;
    int *slot_case = nullptr;
    float *params = nullptr;
    long long total = 0;
    CellTables(SolverBase &s, const FineView &v, const float *params_h)
    {
        std::vector<long long> off_h(v.nslot + 1, 0);
        for (int q = 0; q < v.nslot; q++)
            off_h[q + 1] = off_h[q] + (long long)(v.lv[q].IM - 1) * (v.lv[q].JM - 1) * (v.lv[q].KM - 1);
        total = off_h[v.nslot];
        std::vector<int> sc(v.nslot, 0);
        for (int c = 0; c < s.ncase; c++)
            for (int b = 0; b < s.case_nblk[c]; b++) sc[s.case_first[c] + b] = c;
        mem.bytes = sizeof(long long) * off_h.size() + 256 + sizeof(int) * sc.size() + 256 + sizeof(float) * kWsParams * s.ncase + 256;
        WCK(cudaMalloc(&mem.p, mem.bytes));
        char *q = (char *)mem.p;
        off = (long long *)q; q += (sizeof(long long) * off_h.size() + 255) & ~(size_t)255;
        slot_case = (int *)q; q += (sizeof(int) * sc.size() + 255) & ~(size_t)255;
        params = (float *)q;
        WCK(cudaMemcpy(off, off_h.data(), sizeof(long long) * off_h.size(), cudaMemcpyHostToDevice));
        WCK(cudaMemcpy(slot_case, sc.data(), sizeof(int) * sc.size(), cudaMemcpyHostToDevice));
        WCK(cudaMemcpy(params, params_h, sizeof(float) * kWsParams * s.ncase, cudaMemcpyHostToDevice));
    }
};

void WarmStart::add_solves(SolverBase &s, const float *params)
{
    WCK(cudaStreamSynchronize(s.stream));
    FineView v = s.fine_view();
    CellTables t(s, v, params);
    if (n_set + t.total > d->set_cap) {
        long long cap = std::max(n_set + t.total, 2 * d->set_cap);
        float *p;
        WCK(cudaMalloc(&p, sizeof(float) * kWsSample * cap));
        if (d->set && n_set) WCK(cudaMemcpy(p, d->set, sizeof(float) * kWsSample * n_set, cudaMemcpyDeviceToDevice));
        cudaFree(d->set);
        d->set = p;
        d->set_cap = cap;
    }
    CellsArgs a = cells_args(v, t.off, t.slot_case, t.params);
    k_ws_collect<<<(unsigned)((t.total + 255) / 256), 256, 0, d->st>>>(a, 0, t.total, d->set + n_set * kWsSample);
    WCK(cudaGetLastError());
    WCK(cudaStreamSynchronize(d->st));
    n_set += t.total;
}

float WarmStart::train(int steps, int batch, float lr)
{
    if (n_set <= 0) throw std::runtime_error("the training set is empty");
    if (batch < 128) throw std::invalid_argument("batch below 128 samples");
    Impl &m = *d;
    if (!m.have_norm) {
        const int nb = 256;
        DevBuf pb;
        pb.bytes = sizeof(double) * nb * kWsSample * 4;
        WCK(cudaMalloc(&pb.p, pb.bytes));
        k_ws_stats<<<nb, 256, 0, m.st>>>(m.set, n_set, (double *)pb.p);
        std::vector<double> h(nb * kWsSample * 4);
        WCK(cudaMemcpyAsync(h.data(), pb.p, pb.bytes, cudaMemcpyDeviceToHost, m.st));
        WCK(cudaStreamSynchronize(m.st));
        double mn[kWsSample], mx[kWsSample], s1[kWsSample], s2[kWsSample];
        for (int c = 0; c < kWsSample; c++) { mn[c] = 1e300; mx[c] = -1e300; s1[c] = s2[c] = 0.0; }
        for (int b = 0; b < nb; b++)
            for (int c = 0; c < kWsSample; c++) {
                const double *q = &h[((size_t)b * kWsSample + c) * 4];
                mn[c] = std::min(mn[c], q[0]); mx[c] = std::max(mx[c], q[1]); s1[c] += q[2]; s2[c] += q[3];
            }
        const double N = (double)n_set;
        for (int c = 0; c < 3; c++) {
            m.nrm[c] = (float)mn[c];
            m.nrm[3 + c] = (float)(mx[c] - mn[c] > 1e-12 ? mx[c] : mn[c] + 1.0);
        }
        for (int c = 0; c < 3 + kWsOutUsed; c++) {
            const double mean = s1[3 + c] / N, var = std::max(0.0, s2[3 + c] / N - mean * mean);
            const double sd = std::sqrt(var) > 1e-6 * std::max(1.0, std::fabs(mean)) ? std::sqrt(var) : 1.0;
            if (c < 3) { m.nrm[6 + c] = (float)mean; m.nrm[9 + c] = (float)sd; }
            else { m.nrm[12 + c - 3] = (float)mean; m.nrm[18 + c - 3] = (float)sd; }
        }
        WCK(cudaMemcpy(m.nrm_d, m.nrm, sizeof(m.nrm), cudaMemcpyHostToDevice));
        m.have_norm = true;
    }
    m.ensure(batch);
    const size_t np = n_params();
    double acc = 0.0;
    int nacc = 0;
    for (int it = 0; it < steps; it++) {
        m.rng = m.rng * 6364136223846793005ull + 1442695040888963407ull;
        k_ws_gather<<<(batch + 255) / 256, 256, 0, m.st>>>(m.set, n_set, m.rng, batch, m.nrm_d, m.X0, m.T);
        m.forward(batch);
        const float l = m.loss(batch);
        m.backward(batch);
        m.adam_t++;
        const float c1 = 1.0f - std::pow(0.9f, (float)m.adam_t), c2 = 1.0f - std::pow(0.999f, (float)m.adam_t);
        k_adam<<<(unsigned)((np + 255) / 256), 256, 0, m.st>>>(m.P, m.G, m.Mo, m.Vo, (long long)np, lr, 0.9f, 0.999f, 1e-8f, c1, c2);
        m.refresh_bf16();
        if (it >= steps - 20) { acc += l; nacc++; }
    }
    WCK(cudaStreamSynchronize(m.st));
    WCK(cudaGetLastError());
    if (error_flag()) throw std::runtime_error("a tensor-core wait of the warm-start network ran out");
    return nacc ? (float)(acc / nacc) : 0.0f;
}

void WarmStart::apply(SolverBase &s, const float *params, int *used, double *res_warm, double *res_uniform)
{
    if (!d->have_norm) throw std::runtime_error("the network has no normalisation constants (train or set_norm first)");
    Impl &m = *d;
    s.init_uniform();
    s.save_fine_state();
    s.fill_uniform_fine({});
    s.fine_primitive();
    std::vector<double> r_uni, r_warm;
    s.fine_residual(r_uni);
    FineView v = s.fine_view();
    CellTables t(s, v, params);
    CellsArgs a = cells_args(v, t.off, t.slot_case, t.params);
    const long long chunk = 1 << 19;
    m.ensure(std::min(chunk, std::max(t.total, 1LL)));
    for (long long t0 = 0; t0 < t.total; t0 += chunk) {
        const long long n = std::min(chunk, t.total - t0);
        k_ws_cell_features<<<(unsigned)((n + 255) / 256), 256, 0, m.st>>>(a, t0, n, m.nrm_d, m.X0);
        m.infer(n);
        k_ws_write_cv<<<(unsigned)((n + 255) / 256), 256, 0, m.st>>>(a, t0, n, m.nrm_d, m.Y);
    }
    WCK(cudaStreamSynchronize(m.st));
    WCK(cudaGetLastError());
    if (error_flag()) throw std::runtime_error("a tensor-core wait of the warm-start network ran out");
    s.fine_primitive();
    s.fine_residual(r_warm);
    std::vector<int> back;
    int n_used = 0;
    for (int c = 0; c < s.ncase; c++) {
        const bool ok = std::isfinite(r_warm[c]) && r_warm[c] < r_uni[c];
        used[c] = ok ? 1 : 0;
        n_used += ok;
        if (res_warm) res_warm[c] = r_warm[c];
        if (res_uniform) res_uniform[c] = r_uni[c];
        if (!ok)
            for (int b = 0; b < s.case_nblk[c]; b++) back.push_back(s.case_first[c] + b);
    }
    if (n_used == 0) {
        s.restore_fine_state(true);              // every case on the plain start-up, as init_uniform left it
        return;
    }
    s.restore_fine_state(false);
    if (!back.empty()) {
        s.fill_uniform_fine(back);
        s.fine_primitive();
    }
    WCK(cudaStreamSynchronize(s.stream));
    s.start_from_fine_state();
}

void WarmStart::get_params(float *out)
{
    WCK(cudaStreamSynchronize(d->st));
    WCK(cudaMemcpy(out, d->P, sizeof(float) * n_params(), cudaMemcpyDeviceToHost));
}
void WarmStart::set_params(const float *in)
{
    WCK(cudaStreamSynchronize(d->st));
    WCK(cudaMemcpy(d->P, in, sizeof(float) * n_params(), cudaMemcpyHostToDevice));
    d->refresh_bf16();
    WCK(cudaStreamSynchronize(d->st));
}
void WarmStart::get_norm(float *out) const { std::memcpy(out, d->nrm, sizeof(d->nrm)); }
void WarmStart::set_norm(const float *in)
{
    std::memcpy(d->nrm, in, sizeof(d->nrm));
    WCK(cudaMemcpy(d->nrm_d, d->nrm, sizeof(d->nrm), cudaMemcpyHostToDevice));
    d->have_norm = true;
}

void WarmStart::forward(const float *feat, int M, float *y)
{
    Impl &m = *d;
    m.ensure(M);
    DevBuf f;
    f.bytes = sizeof(float) * (size_t)M * kWsIn;
    WCK(cudaMalloc(&f.p, f.bytes));
    WCK(cudaMemcpy(f.p, feat, f.bytes, cudaMemcpyHostToDevice));
    k_f32_to_bf16<<<(unsigned)(((size_t)M * kWsIn + 255) / 256), 256, 0, m.st>>>((const float *)f.p, (long long)M * kWsIn, m.X0);
    m.infer(M);
    WCK(cudaMemcpyAsync(y, m.Y, sizeof(float) * (size_t)M * kWsOut, cudaMemcpyDeviceToHost, m.st));
    WCK(cudaStreamSynchronize(m.st));
    if (error_flag()) throw std::runtime_error("a tensor-core wait of the warm-start network ran out");
}

float WarmStart::forward_backward(const float *feat, const float *target, int M, float *grad)
{
    Impl &m = *d;
    m.ensure(M);
    DevBuf f;
    f.bytes = sizeof(float) * (size_t)M * kWsIn;
    WCK(cudaMalloc(&f.p, f.bytes));
    WCK(cudaMemcpy(f.p, feat, f.bytes, cudaMemcpyHostToDevice));
    k_f32_to_bf16<<<(unsigned)(((size_t)M * kWsIn + 255) / 256), 256, 0, m.st>>>((const float *)f.p, (long long)M * kWsIn, m.X0);
    std::vector<float> t8((size_t)M * 8, 0.0f);
    for (int r = 0; r < M; r++)
        for (int o = 0; o < kWsOutUsed; o++) t8[(size_t)r * 8 + o] = target[(size_t)r * kWsOutUsed + o];
    WCK(cudaMemcpyAsync(m.T, t8.data(), sizeof(float) * t8.size(), cudaMemcpyHostToDevice, m.st));
    m.forward(M);
    const float l = m.loss(M);
    m.backward(M);
    WCK(cudaMemcpyAsync(grad, m.G, sizeof(float) * n_params(), cudaMemcpyDeviceToHost, m.st));
    WCK(cudaStreamSynchronize(m.st));
    if (error_flag()) throw std::runtime_error("a tensor-core wait of the warm-start network ran out");
    return l;
}

__global__ void k_ws_random_rows(long long M, unsigned long long seed, bf16 *X0, float *T)
{
    const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    for (int c = 0; c < kWsIn; c++) {
        const unsigned long long h = mix64(seed ^ ((unsigned long long)m * kWsIn + c));
        X0[m * kWsIn + c] = __float2bfloat16_rn((float)(h >> 40) * (2.0f / 16777216.0f) - 1.0f);
    }
    for (int o = 0; o < 8; o++) {
        const unsigned long long h = mix64(~seed ^ ((unsigned long long)m * 8 + o));
        T[m * 8 + o] = o < kWsOutUsed ? (float)(h >> 40) * (2.0f / 16777216.0f) - 1.0f : 0.0f;
    }
}

void WarmStart::benchmark(long long M, int iters, float *ms_forward, float *ms_step, float *ms_infer, double *max_diff)
{
    if (M < 128 || iters < 1) throw std::invalid_argument("benchmark: at least 128 rows and one iteration");
    Impl &m = *d;
    m.ensure(M);
    k_ws_random_rows<<<(unsigned)((M + 255) / 256), 256, 0, m.st>>>(M, 12345ull, m.X0, m.T);
    cudaEvent_t e0, e1;
    WCK(cudaEventCreate(&e0));
    WCK(cudaEventCreate(&e1));
    m.forward(M);                                        // warm-up
    WCK(cudaEventRecord(e0, m.st));
    for (int i = 0; i < iters; i++) m.forward(M);
    WCK(cudaEventRecord(e1, m.st));
    WCK(cudaEventSynchronize(e1));
    float t = 0.f;
    WCK(cudaEventElapsedTime(&t, e0, e1));
    *ms_forward = t / iters;
    // the fused inference: timed, and its outputs against the layer-by-layer pass's (the same bits)
    std::vector<float> y_layers((size_t)M * kWsOut), y_fused((size_t)M * kWsOut);
    WCK(cudaMemcpyAsync(y_layers.data(), m.Y, sizeof(float) * y_layers.size(), cudaMemcpyDeviceToHost, m.st));
    m.infer(M);                                          // warm-up
    WCK(cudaEventRecord(e0, m.st));
    for (int i = 0; i < iters; i++) m.infer(M);
    WCK(cudaEventRecord(e1, m.st));
    WCK(cudaEventSynchronize(e1));
    WCK(cudaEventElapsedTime(&t, e0, e1));
    if (ms_infer) *ms_infer = t / iters;
    WCK(cudaMemcpyAsync(y_fused.data(), m.Y, sizeof(float) * y_fused.size(), cudaMemcpyDeviceToHost, m.st));
    WCK(cudaStreamSynchronize(m.st));
    double dmax = 0.0;
    for (size_t q = 0; q < y_fused.size(); q++) {
        const double dq = std::fabs((double)y_fused[q] - (double)y_layers[q]);
        dmax = (dq > dmax || dq != dq) ? dq : dmax;
    }
    if (max_diff) *max_diff = dmax;
    const int nb = (int)((M + 255) / 256);
    WCK(cudaEventRecord(e0, m.st));
    for (int i = 0; i < iters; i++) {
        m.forward(M);
        k_ws_loss<<<nb, 256, 0, m.st>>>(m.Y, m.T, M, m.dY, m.lpart);
        m.backward(M);
    }
    WCK(cudaEventRecord(e1, m.st));
    WCK(cudaEventSynchronize(e1));
    WCK(cudaEventElapsedTime(&t, e0, e1));
    *ms_step = t / iters;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (error_flag()) throw std::runtime_error("a tensor-core wait of the warm-start network ran out");
}

}  // namespace gbt
