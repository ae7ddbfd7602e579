// Face stage of the mixed form with each tile of faces staged in shared memory by the tensor
// memory accelerator (TMA): one CTA per tile of 128 faces of one family, a single thread issues
// one cp.async.bulk.tensor.3d copy per input field -- the cell fields over the tile plus its
// stencil halo (two cells along the face normal each way for MUSCL and the reference's dummy-layer
// switch, one cell tangentially for the viscous gradients) and the per-face geometry of the tile --
// all completing on one mbarrier; every thread then computes one face from shared memory with the
// arithmetic of the plain face kernel (face_body.cuh) and stores its fluxes.
//
// The stencil arithmetic is source/Upwind_Convective.cpp:31-97 (gather), source/Reconstruction.cpp
// (MUSCL3 on primitives), source/Flux_Split_Scheme.cpp:568-635 (Roe), source/WallFlux.cpp:70-175
// and source/ViscousFlux.cpp:9-269, as in k_face. Used for the default scheme of the mixed form
// when every block's padded k extent (KM + 7) is a multiple of four, so that every tensor row and
// every box start is 16-byte aligned (KM = 4n + 1: every multigrid-coarsenable mesh); otherwise the
// plain kernel runs.
//
// Tensor maps: one per (slot, field), built once per level on the host and kept in device memory;
// they cover only this GPU's own pools (no multicast).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cstdint>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>
#include "gbt_common.cuh"
#include "kernels.hpp"
#include "face_body.cuh"
#include "solver.hpp"

namespace gbt {
namespace {

constexpr int kCellFields = 7;                    // six primitives and mu_t
constexpr int kGeoFields = 24;                    // S(3) s nrm(3) t1(3) t2(3) qe m(9) and the wall flag
constexpr int kMapsPerSlot = 3 * kCellFields + 3 * kGeoFields;
constexpr int KT = 32;                            // faces of a tile along k (the contiguous index)

template <int F, bool GEO> struct Tile {
    static constexpr int JT = F == 0 ? 1 : 4, IT = F == 0 ? 4 : 1;            // faces along j, i
    static constexpr int KW = KT + 8;                                          // cells along k: k0-4 .. k0+35
    static constexpr int JW = JT + (F == 1 ? 5 : 2), IW = IT + (F == 0 ? 5 : 2);
    static constexpr int JLO = F == 1 ? 3 : 1, ILO = F == 0 ? 3 : 1;          // halo below j0, i0
    static constexpr int CELLS = KW * JW * IW;
    static constexpr int CELL_STRIDE = ((CELLS * 4 + 127) / 128) * 32;         // floats, 128-byte multiples
    static constexpr int FACES = KT * JT * IT;                                 // 128
    static constexpr int NGEO = GEO ? kGeoFields : 0;                          // geometry staged too, or read straight
    static constexpr int TX_BYTES = kCellFields * CELLS * 4 + NGEO * FACES * 4;
    static constexpr int SMEM = kCellFields * CELL_STRIDE * 4 + NGEO * FACES * 4 + 128 + 128;
};

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
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
// about a second at most
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity)
{
    for (int t = 0; t < (1 << 22); t++) {
        if (mbar_try_wait(bar, parity)) return true;
        if (t > 16) __nanosleep(64);
    }
    return false;
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

// GEO: the per-face geometry staged by TMA as well (true) or read by each thread straight from
// HBM with coalesced loads (false), which leaves shared memory to the haloed cell fields alone
template <int F, bool GEO>
__global__ void __launch_bounds__(128, GEO ? 5 : 7) k_face_tma(Batch B, Phys P, PhysW<float> PC, GeoW<float> G,
                                                             Flow<float> W, const DevWall *walls, const CUtensorMap *maps)
{
    using Tl = Tile<F, GEO>;
    extern __shared__ unsigned char smem_raw[];
    const int s = blockIdx.y;
    const Lvl L = B.lv[s];
    int ni, nj, nk;
    face_extent(L, F, ni, nj, nk);
    const int tk = (nk + KT - 1) / KT, tj = (nj + Tl::JT - 1) / Tl::JT, ti = (ni + Tl::IT - 1) / Tl::IT;
    const int b = blockIdx.x;
    if (b >= tk * tj * ti) return;                 // the whole CTA: a smaller block of the batch
    const int k0 = 1 + (b % tk) * KT, j0 = 1 + ((b / tk) % tj) * Tl::JT, i0 = 1 + (b / (tk * tj)) * Tl::IT;

    // 128-byte aligned carve-up: cell fields, geometry, mbarrier
    const uint32_t raw = (uint32_t)__cvta_generic_to_shared(smem_raw);
    const uint32_t base = (raw + 127u) & ~127u;
    float *cell = reinterpret_cast<float *>(smem_raw + (base - raw));
    float *geo = cell + kCellFields * Tl::CELL_STRIDE;
    const uint32_t bar = base + (uint32_t)(kCellFields * Tl::CELL_STRIDE + Tl::NGEO * Tl::FACES) * 4u;
    const CUtensorMap *mp = maps + (size_t)s * kMapsPerSlot;

    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        mbar_expect_tx(bar, (uint32_t)Tl::TX_BYTES);
    }
    __syncthreads();                               // the barrier is armed before any copy or poll
    if (threadIdx.x < kCellFields + Tl::NGEO) {
        // one copy per lane of the first warp, issued side by side; tensor coordinates are box
        // indices + PAD, and x = k0 - 1 and x = k0 + 3 are multiples of four
        const int c = threadIdx.x;
        if (c < kCellFields)
            tma_load_3d(base + (uint32_t)(c * Tl::CELL_STRIDE) * 4u, mp + F * kCellFields + c, k0 - 4 + PAD,
                        j0 - Tl::JLO + PAD, i0 - Tl::ILO + PAD, bar);
        else
            tma_load_3d(base + (uint32_t)(kCellFields * Tl::CELL_STRIDE + (c - kCellFields) * Tl::FACES) * 4u,
                        mp + 3 * kCellFields + F * kGeoFields + (c - kCellFields), k0 + PAD, j0 + PAD, i0 + PAD, bar);
    }
    if (!mbar_wait_bounded(bar, 0)) {
        // the copies did not complete within the limit: report it, give them once more the same
        // time before the tile's shared memory is released, and leave the tile
        if (threadIdx.x == 0) atomicOr(&B.st[s].status, GBT_STATUS_WAIT_TIMEOUT);
        mbar_wait_bounded(bar, 0);
        return;
    }
    const int kk = threadIdx.x & (KT - 1), r = threadIdx.x / KT;
    const int ii = F == 0 ? r : 0, jj = F == 0 ? 0 : r;
    const int i = i0 + ii, j = j0 + jj, k = k0 + kk;
    if (i > ni || j > nj || k > nk) return;
    const long long sJ = Tl::KW, sI = (long long)Tl::JW * Tl::KW;
    const long long p = (long long)(i - (i0 - Tl::ILO)) * sI + (long long)(j - (j0 - Tl::JLO)) * sJ + (k - (k0 - 4));
    CellSrc<float> C;
#pragma unroll
    for (int c = 0; c < NPV; c++) C.pv[c] = cell + c * Tl::CELL_STRIDE;
    C.mut = cell + 6 * Tl::CELL_STRIDE;
    const long long pg = ix(L, i, j, k);
    FaceGeo<float> g;
    int wq;
    if constexpr (GEO) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            g.S[c] = geo + c * Tl::FACES;
            g.nrm[c] = geo + (4 + c) * Tl::FACES;
            g.t1[c] = geo + (7 + c) * Tl::FACES;
            g.t2[c] = geo + (10 + c) * Tl::FACES;
        }
        g.s = geo + 3 * Tl::FACES;
        g.qe = geo + 13 * Tl::FACES;
#pragma unroll
        for (int c = 0; c < 9; c++) g.m[c] = geo + (14 + c) * Tl::FACES;
        g.q = (ii * Tl::JT + jj) * KT + kk;
        wq = reinterpret_cast<const int *>(geo + 23 * Tl::FACES)[g.q];
    } else {
#pragma unroll
        for (int c = 0; c < 3; c++) { g.S[c] = G.S[F][c]; g.nrm[c] = G.nrm[F][c]; g.t1[c] = G.t1[F][c]; g.t2[c] = G.t2[F][c]; }
        g.s = G.s[F];
        g.qe = G.qe[F];
#pragma unroll
        for (int c = 0; c < 9; c++) g.m[c] = G.m[F][c];
        g.q = pg;
        wq = W.wallf[F][pg];
    }
    float rot = 0.f, cxf = 0.f, cyf = 0.f;
    if (wq) {
        rot = walls[wq - 1].rotate ? (float)B.sc[s].w_rot : 0.f;
        cxf = G.c[F][0][pg];
        cyf = G.c[F][1][pg];
    }
    float out[10];
    face_body<float, F, 1>(P, PC, C, nullptr, p, sI, sJ, 1, i, j, k, L.IM, L.JM, L.KM, g, wq, rot, cxf, cyf, out);
#pragma unroll
    for (int c = 0; c < NQ; c++) W.Ff[F][c][pg] = out[c];
    if (!P.equation_ns) return;
#pragma unroll
    for (int c = 0; c < NQ; c++) W.Vf[F][c][pg] = out[5 + c];
}

PFN_cuTensorMapEncodeTiled_v12000 encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        check_cuda(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q),
                   "cudaGetDriverEntryPointByVersion(cuTensorMapEncodeTiled)");
        if (!f || q != cudaDriverEntryPointSuccess) throw std::runtime_error("cuTensorMapEncodeTiled is not available");
        encode = (PFN_cuTensorMapEncodeTiled_v12000)f;
    }
    return encode;
}

// 3D tensor map over one slot's padded box (x = k, y = j, z = i), boxes of bx x by x bz elements;
// boxes that reach past the box read zeros
CUtensorMap box_map(const void *slot_base, bool is_int, const Lvl &v, int bx, int by, int bz)
{
    const int NI = v.IM + 1 + 2 * PAD;
    if (((uintptr_t)slot_base & 15) || ((v.NK * 4) & 15)) throw std::runtime_error("face tile: misaligned tensor");
    CUtensorMap m;
    const cuuint64_t dims[3] = {(cuuint64_t)v.NK, (cuuint64_t)v.NJ, (cuuint64_t)NI};
    const cuuint64_t strides[2] = {(cuuint64_t)v.NK * 4, (cuuint64_t)v.NK * v.NJ * 4};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz};
    const cuuint32_t es[3] = {1u, 1u, 1u};
    const CUresult r = encoder()(&m, is_int ? CU_TENSOR_MAP_DATA_TYPE_INT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                                 const_cast<void *>(slot_base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                 CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed (face tile)");
    return m;
}

template <int F>
void add_family_maps(std::vector<CUtensorMap> &cellm, std::vector<CUtensorMap> &geom, const Lvl &v,
                     const GeoW<float> &G, const Flow<float> &W)
{
    using Tl = Tile<F, true>;
    for (int c = 0; c < NPV; c++) cellm.push_back(box_map(W.pv[c] + v.base, false, v, Tl::KW, Tl::JW, Tl::IW));
    cellm.push_back(box_map(W.mut + v.base, false, v, Tl::KW, Tl::JW, Tl::IW));
    const float *ga[kGeoFields - 1] = {G.S[F][0], G.S[F][1], G.S[F][2], G.s[F], G.nrm[F][0], G.nrm[F][1], G.nrm[F][2],
                                       G.t1[F][0], G.t1[F][1], G.t1[F][2], G.t2[F][0], G.t2[F][1], G.t2[F][2], G.qe[F],
                                       G.m[F][0], G.m[F][1], G.m[F][2], G.m[F][3], G.m[F][4], G.m[F][5], G.m[F][6],
                                       G.m[F][7], G.m[F][8]};
    for (int g = 0; g < kGeoFields - 1; g++) geom.push_back(box_map(ga[g] + v.base, false, v, KT, Tl::JT, Tl::IT));
    geom.push_back(box_map(W.wallf[F] + v.base, true, v, KT, Tl::JT, Tl::IT));
}

}  // namespace

bool face_tma_eligible(const std::vector<Lvl> &lv)
{
    const char *e = std::getenv("GBTURBO_FACE_TMA");
    if (e && e[0] == '0') return false;
    // every box row and box start 16-byte aligned, and every slot's box at least one tile's halo
    // box wide in each direction
    for (const Lvl &v : lv)
        if (v.NK % 4 != 0 || v.base % 4 != 0 || v.NK < KT + 8 || v.NJ < 9 || v.IM + 1 + 2 * PAD < 9) return false;
    return true;
}

void *build_face_tma(const std::vector<Lvl> &lv, const GeoW<float> &G, const Flow<float> &W, size_t *bytes)
{
    std::vector<CUtensorMap> all;
    all.reserve(lv.size() * kMapsPerSlot);
    for (const Lvl &v : lv) {
        std::vector<CUtensorMap> cellm, geom;
        add_family_maps<0>(cellm, geom, v, G, W);
        add_family_maps<1>(cellm, geom, v, G, W);
        add_family_maps<2>(cellm, geom, v, G, W);
        // per slot: the 3 x 7 cell maps (family after family), then the 3 x 24 geometry maps
        all.insert(all.end(), cellm.begin(), cellm.end());
        all.insert(all.end(), geom.begin(), geom.end());
    }
    void *d = nullptr;
    *bytes = sizeof(CUtensorMap) * all.size();
    check_cuda(cudaMalloc(&d, *bytes), "cudaMalloc(face tile tensor maps)");
    check_cuda(cudaMemcpy(d, all.data(), *bytes, cudaMemcpyHostToDevice), "cudaMemcpy(face tile tensor maps)");
    return d;
}

void launch_face_tma(const LaunchCtx &ctx, const Phys &P, const PhysW<float> &PC, const GeoW<float> &GW, Flow<float> W,
                     const DevWall *walls)
{
    const Batch &B = ctx.batch;
    const CUtensorMap *maps = (const CUtensorMap *)ctx.face_tma;
    auto tiles = [&](int F, int JT, int IT) {
        const int ni = ctx.maxIM - 1 + (F == 0), nj = ctx.maxJM - 1 + (F == 1), nk = ctx.maxKM - 1 + (F == 2);
        return (unsigned)(((nk + KT - 1) / KT) * ((nj + JT - 1) / JT) * ((ni + IT - 1) / IT));
    };
    // a slot smaller than the largest has fewer tiles along every direction, so the largest
    // extents bound every slot's tile count
    const char *e = std::getenv("GBTURBO_FACE_TMA");
    if (e && e[0] == '2') {
        k_face_tma<0, true><<<dim3(tiles(0, Tile<0, true>::JT, Tile<0, true>::IT), B.nsolve), 128, Tile<0, true>::SMEM, ctx.stream>>>(B, P, PC, GW, W, walls, maps);
        k_face_tma<1, true><<<dim3(tiles(1, Tile<1, true>::JT, Tile<1, true>::IT), B.nsolve), 128, Tile<1, true>::SMEM, ctx.stream>>>(B, P, PC, GW, W, walls, maps);
        k_face_tma<2, true><<<dim3(tiles(2, Tile<2, true>::JT, Tile<2, true>::IT), B.nsolve), 128, Tile<2, true>::SMEM, ctx.stream>>>(B, P, PC, GW, W, walls, maps);
    } else {
        k_face_tma<0, false><<<dim3(tiles(0, Tile<0, false>::JT, Tile<0, false>::IT), B.nsolve), 128, Tile<0, false>::SMEM, ctx.stream>>>(B, P, PC, GW, W, walls, maps);
        k_face_tma<1, false><<<dim3(tiles(1, Tile<1, false>::JT, Tile<1, false>::IT), B.nsolve), 128, Tile<1, false>::SMEM, ctx.stream>>>(B, P, PC, GW, W, walls, maps);
        k_face_tma<2, false><<<dim3(tiles(2, Tile<2, false>::JT, Tile<2, false>::IT), B.nsolve), 128, Tile<2, false>::SMEM, ctx.stream>>>(B, P, PC, GW, W, walls, maps);
    }
}

}  // namespace gbt
