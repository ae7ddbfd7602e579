// Face stage of the mixed form with tiles of faces whose cell fields are staged in shared memory
// by the tensor memory accelerator (TMA): per tile, one cp.async.bulk.tensor.3d copy per cell field
// (the six primitives and mu_t) brings the tile plus its stencil halo -- two cells along the face
// normal each way for MUSCL and the reference's dummy-layer switch, one cell tangentially for the
// viscous gradients -- completing on an mbarrier; every thread then computes one face from shared
// memory with the arithmetic of the plain face kernel (face_body.cuh), streaming the per-face
// geometry (read once, no reuse) with coalesced loads, and stores its fluxes.
//
// Two forms:
//  - one-shot: one CTA of 128 threads per tile of 128 faces, which waits for its own copies;
//  - pipelined: persistent CTAs of 256 threads over tiles of 256 faces, two buffers: the copies of
//    a CTA's next tile are in flight while it computes the current one.
//
// The stencil arithmetic is source/Upwind_Convective.cpp:31-97 (gather), source/Reconstruction.cpp
// (MUSCL3 on primitives), source/Flux_Split_Scheme.cpp:568-635 (Roe), source/WallFlux.cpp:70-175
// and source/ViscousFlux.cpp:9-269, as in k_face. Used for the default scheme of the mixed form
// when every block's padded k extent (KM + 7) is a multiple of four, so that every tensor row and
// every box start is 16-byte aligned (KM = 4n + 1: every multigrid-coarsenable mesh).
//
// Tensor maps: one per (slot, cell field, family, form), built once per level on the host and kept
// in device memory; they cover only this GPU's own pools (no multicast).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
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
constexpr int kMapsPerSlot = 2 * 3 * kCellFields; // two forms x three families x seven fields
constexpr int KT = 32;                            // faces of a tile along k (the contiguous index)

// tile geometry of form PIPE (0 one-shot, 1 pipelined) for face family F
template <int F, int PIPE> struct Tile {
    static constexpr int R = PIPE ? 8 : 4;                                     // face rows of 32 (one per warp)
    static constexpr int JT = F == 0 ? 1 : R, IT = F == 0 ? R : 1;             // faces along j, i
    static constexpr int KW = KT + 8;                                          // cells along k: k0-4 .. k0+35
    static constexpr int JW = JT + (F == 1 ? 5 : 2), IW = IT + (F == 0 ? 5 : 2);
    static constexpr int JLO = F == 1 ? 3 : 1, ILO = F == 0 ? 3 : 1;          // halo below j0, i0
    static constexpr int CELLS = KW * JW * IW;
    static constexpr int CELL_STRIDE = ((CELLS * 4 + 127) / 128) * 32;         // floats, 128-byte multiples
    static constexpr int BUF = kCellFields * CELL_STRIDE;                      // floats per buffer
    static constexpr int THREADS = 32 * R;
    static constexpr int TX_BYTES = kCellFields * CELLS * 4;
    static constexpr int NBUF = PIPE ? 2 : 1;
    static constexpr int SMEM = NBUF * BUF * 4 + 128 + 128;
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

// a tile's origin (first face of the tile, node indices) from its index within its slot
template <int F, int PIPE>
__device__ __forceinline__ void tile_origin(const Lvl &L, int b, int &i0, int &j0, int &k0)
{
    using Tl = Tile<F, PIPE>;
    int ni, nj, nk;
    face_extent(L, F, ni, nj, nk);
    const int tk = (nk + KT - 1) / KT, tj = (nj + Tl::JT - 1) / Tl::JT;
    k0 = 1 + (b % tk) * KT;
    j0 = 1 + ((b / tk) % tj) * Tl::JT;
    i0 = 1 + (b / (tk * tj)) * Tl::IT;
}

// the copies of one tile: lane c < 7 of the calling warp copies cell field c (the armed barrier
// counts the bytes of all seven); tensor coordinates are box indices + PAD, x = k0 - 1 a multiple of 4
template <int F, int PIPE>
__device__ __forceinline__ void issue_tile(const CUtensorMap *mp, uint32_t dst, uint32_t bar, int i0, int j0, int k0)
{
    using Tl = Tile<F, PIPE>;
    const int c = threadIdx.x & 31;
    if (c < kCellFields)
        tma_load_3d(dst + (uint32_t)(c * Tl::CELL_STRIDE) * 4u, mp + (PIPE * 3 + F) * kCellFields + c, k0 - 4 + PAD,
                    j0 - Tl::JLO + PAD, i0 - Tl::ILO + PAD, bar);
}

// one face of a staged tile: thread t takes face (row t / 32, k0 + t % 32) of the tile
template <int F, int PIPE>
__device__ __forceinline__ void tile_face(const Batch &B, const Phys &P, const PhysW<float> &PC, const GeoW<float> &G,
                                          Flow<float> &W, const DevWall *walls, int s, const Lvl &L, const float *cell,
                                          int i0, int j0, int k0)
{
    using Tl = Tile<F, PIPE>;
    int ni, nj, nk;
    face_extent(L, F, ni, nj, nk);
    const int kk = threadIdx.x & (KT - 1), r = threadIdx.x / KT;
    const int i = i0 + (F == 0 ? r : 0), j = j0 + (F == 0 ? 0 : r), k = k0 + kk;
    if (i > ni || j > nj || k > nk) return;
    const int sJ = Tl::KW, sI = Tl::JW * Tl::KW;
    const int p = (i - (i0 - Tl::ILO)) * sI + (j - (j0 - Tl::JLO)) * sJ + (k - (k0 - 4));
    CellSrc<float> C;
#pragma unroll
    for (int c = 0; c < NPV; c++) C.pv[c] = cell + c * Tl::CELL_STRIDE;
    C.mut = cell + 6 * Tl::CELL_STRIDE;
    const int pg = (int)ix(L, i, j, k);
    FaceGeo<float> g;
#pragma unroll
    for (int c = 0; c < 3; c++) { g.S[c] = G.S[F][c]; g.nrm[c] = G.nrm[F][c]; g.t1[c] = G.t1[F][c]; g.t2[c] = G.t2[F][c]; }
    g.s = G.s[F];
    g.qe = G.qe[F];
#pragma unroll
    for (int c = 0; c < 9; c++) g.m[c] = G.m[F][c];
    g.q = pg;
    const int wq = W.wallf[F][pg];
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

// 128-byte aligned start of the dynamic shared memory
__device__ __forceinline__ uint32_t smem_base(unsigned char *raw_ptr, float *&buf)
{
    const uint32_t raw = (uint32_t)__cvta_generic_to_shared(raw_ptr);
    const uint32_t base = (raw + 127u) & ~127u;
    buf = reinterpret_cast<float *>(raw_ptr + (base - raw));
    return base;
}

// one-shot form: one CTA per tile of 128 faces; grid (tiles of the largest slot, slots)
template <int F>
__global__ void __launch_bounds__(128, 7) k_face_tile(Batch B, Phys P, PhysW<float> PC, GeoW<float> G, Flow<float> W,
                                                     const DevWall *walls, const CUtensorMap *maps)
{
    using Tl = Tile<F, 0>;
    extern __shared__ unsigned char smem_raw[];
    const int s = blockIdx.y;
    const Lvl L = B.lv[s];
    int ni, nj, nk;
    face_extent(L, F, ni, nj, nk);
    const int ntile = ((nk + KT - 1) / KT) * ((nj + Tl::JT - 1) / Tl::JT) * ((ni + Tl::IT - 1) / Tl::IT);
    if ((int)blockIdx.x >= ntile) return;          // the whole CTA: a smaller block of the batch
    int i0, j0, k0;
    tile_origin<F, 0>(L, blockIdx.x, i0, j0, k0);
    float *cell;
    const uint32_t base = smem_base(smem_raw, cell);
    const uint32_t bar = base + (uint32_t)Tl::BUF * 4u;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        mbar_expect_tx(bar, (uint32_t)Tl::TX_BYTES);
    }
    __syncthreads();                               // the barrier is armed before any copy or poll
    if (threadIdx.x < 32) issue_tile<F, 0>(maps + (size_t)s * kMapsPerSlot, base, bar, i0, j0, k0);
    if (!mbar_wait_bounded(bar, 0)) {
        // the copies did not complete within the limit: report it, give them once more the same
        // time before the tile's shared memory is released, and leave the tile
        if (threadIdx.x == 0) atomicOr(&B.st[s].status, GBT_STATUS_WAIT_TIMEOUT);
        mbar_wait_bounded(bar, 0);
        return;
    }
    tile_face<F, 0>(B, P, PC, G, W, walls, s, L, cell, i0, j0, k0);
}

// slot and tile within the slot of flat tile index t (tile_start: nslot + 1 ascending offsets)
__device__ __forceinline__ void locate_tile(const int *__restrict__ tile_start, int nslot, int t, int &s, int &b)
{
    int lo = 0, hi = nslot;                        // tile_start[lo] <= t < tile_start[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (tile_start[mid] <= t) lo = mid;
        else hi = mid;
    }
    s = lo;
    b = t - tile_start[lo];
}

// pipelined form: persistent CTAs over the flat list of tiles of every slot; the copies of tile
// n + 1 of a CTA are in flight while it computes tile n (two buffers, one mbarrier each; buffer
// n % 2 is refilled with tile n + 2 once every thread has finished tile n)
template <int F>
__global__ void __launch_bounds__(256, 2) k_face_pipe(Batch B, Phys P, PhysW<float> PC, GeoW<float> G, Flow<float> W,
                                                     const DevWall *walls, const CUtensorMap *maps,
                                                     const int *__restrict__ tile_start, int ntiles)
{
    using Tl = Tile<F, 1>;
    extern __shared__ unsigned char smem_raw[];
    float *cell;
    const uint32_t base = smem_base(smem_raw, cell);
    const uint32_t bar0 = base + 2u * (uint32_t)Tl::BUF * 4u, bar1 = bar0 + 8u;
    const int nslot = B.nsolve;
    if (threadIdx.x == 0) {
        mbar_init(bar0, 1);
        mbar_init(bar1, 1);
    }
    __syncthreads();
    // the first warp arms buffer `buf`'s barrier and issues tile t's copies into it
    auto issue = [&](int t, int buf) {
        int s, b, i0, j0, k0;
        locate_tile(tile_start, nslot, t, s, b);
        tile_origin<F, 1>(B.lv[s], b, i0, j0, k0);
        const uint32_t bar = buf ? bar1 : bar0;
        if (threadIdx.x == 0) mbar_expect_tx(bar, (uint32_t)Tl::TX_BYTES);
        __syncwarp();
        issue_tile<F, 1>(maps + (size_t)s * kMapsPerSlot, base + (uint32_t)(buf * Tl::BUF) * 4u, bar, i0, j0, k0);
    };
    const int G0 = (int)gridDim.x;
    if (threadIdx.x < 32) {
        if ((int)blockIdx.x < ntiles) issue(blockIdx.x, 0);
        if ((int)blockIdx.x + G0 < ntiles) issue(blockIdx.x + G0, 1);
    }
    int n = 0;
    for (int t = blockIdx.x; t < ntiles; t += G0, n++) {
        const int buf = n & 1;
        int s, b, i0, j0, k0;
        locate_tile(tile_start, nslot, t, s, b);
        if (!mbar_wait_bounded(buf ? bar1 : bar0, (uint32_t)((n >> 1) & 1))) {
            // report it, then give this tile's copies and the next tile's (if issued) once more the
            // same time before the shared memory is released
            if (threadIdx.x == 0) atomicOr(&B.st[s].status, GBT_STATUS_WAIT_TIMEOUT);
            mbar_wait_bounded(buf ? bar1 : bar0, (uint32_t)((n >> 1) & 1));
            if (t + G0 < ntiles) mbar_wait_bounded(buf ? bar0 : bar1, (uint32_t)(((n + 1) >> 1) & 1));
            return;
        }
        const Lvl L = B.lv[s];
        tile_origin<F, 1>(L, b, i0, j0, k0);
        tile_face<F, 1>(B, P, PC, G, W, walls, s, L, cell + buf * Tl::BUF, i0, j0, k0);
        __syncthreads();                           // every thread is done with this buffer
        if (threadIdx.x < 32 && t + 2 * G0 < ntiles) issue(t + 2 * G0, buf);
    }
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

// 3D tensor map over one slot's padded box of an FP32 field (x = k, y = j, z = i), boxes of
// bx x by x bz elements; boxes that reach past the box read zeros
CUtensorMap box_map(const float *slot_base, const Lvl &v, int bx, int by, int bz)
{
    const int NI = v.IM + 1 + 2 * PAD;
    if (((uintptr_t)slot_base & 15) || ((v.NK * 4) & 15)) throw std::runtime_error("face tile: misaligned tensor");
    CUtensorMap m;
    const cuuint64_t dims[3] = {(cuuint64_t)v.NK, (cuuint64_t)v.NJ, (cuuint64_t)NI};
    const cuuint64_t strides[2] = {(cuuint64_t)v.NK * 4, (cuuint64_t)v.NK * v.NJ * 4};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz};
    const cuuint32_t es[3] = {1u, 1u, 1u};
    const CUresult r = encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(slot_base), dims, strides, box,
                                 es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed (face tile)");
    return m;
}

template <int F, int PIPE>
void add_maps(std::vector<CUtensorMap> &out, const Lvl &v, const Flow<float> &W)
{
    using Tl = Tile<F, PIPE>;
    for (int c = 0; c < NPV; c++) out.push_back(box_map(W.pv[c] + v.base, v, Tl::KW, Tl::JW, Tl::IW));
    out.push_back(box_map(W.mut + v.base, v, Tl::KW, Tl::JW, Tl::IW));
}

template <int F, int PIPE>
int slot_tiles(const Lvl &v)
{
    using Tl = Tile<F, PIPE>;
    const int ni = v.IM - 1 + (F == 0), nj = v.JM - 1 + (F == 1), nk = v.KM - 1 + (F == 2);
    return ((nk + KT - 1) / KT) * ((nj + Tl::JT - 1) / Tl::JT) * ((ni + Tl::IT - 1) / Tl::IT);
}

// device table of a level: the tensor maps (slot after slot), then per family the flat tile
// offsets of the pipelined form (nslot + 1 each), then the pipelined grid sizes
struct TmaTable {
    size_t maps_off = 0, starts_off = 0;
    int ntiles[3] = {0, 0, 0}, grid[3] = {0, 0, 0};
    int form = 1;                                  // 1 one-shot, 2 pipelined (fixed at create)
};

}  // namespace

bool face_tma_eligible(const std::vector<Lvl> &lv)
{
    // opt-in: GBTURBO_FACE_TMA=1 the one-shot form, =2 the pipelined form
    const char *e = std::getenv("GBTURBO_FACE_TMA");
    if (!e || (e[0] != '1' && e[0] != '2')) return false;
    // every box row and box start 16-byte aligned, and every slot's box at least one tile's halo
    // box wide in each direction
    for (const Lvl &v : lv)
        if (v.NK % 4 != 0 || v.base % 4 != 0 || v.NK < KT + 8 || v.NJ < 13 || v.IM + 1 + 2 * PAD < 13) return false;
    return true;
}

void *build_face_tma(const std::vector<Lvl> &lv, const GeoW<float> &, const Flow<float> &W, size_t *bytes,
                     unsigned char host_header[64])
{
    std::vector<CUtensorMap> maps;
    maps.reserve(lv.size() * kMapsPerSlot);
    for (const Lvl &v : lv) {
        add_maps<0, 0>(maps, v, W); add_maps<1, 0>(maps, v, W); add_maps<2, 0>(maps, v, W);
        add_maps<0, 1>(maps, v, W); add_maps<1, 1>(maps, v, W); add_maps<2, 1>(maps, v, W);
    }
    const int nslot = (int)lv.size();
    std::vector<int> starts;
    TmaTable tab;
    const char *e = std::getenv("GBTURBO_FACE_TMA");
    tab.form = (e && e[0] == '2') ? 2 : 1;
    int dev = 0, sms = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
    auto family = [&](auto kernel, int F, int smem, auto tiles_of) {
        check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem), "cudaFuncSetAttribute");
        int per_sm = 0;
        check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, smem), "cudaOccupancyMaxActiveBlocks");
        int acc = 0;
        starts.push_back(0);
        for (const Lvl &v : lv) { acc += tiles_of(v); starts.push_back(acc); }
        tab.ntiles[F] = acc;
        tab.grid[F] = std::max(1, std::min(acc, std::max(per_sm, 1) * sms));
    };
    family(k_face_pipe<0>, 0, Tile<0, 1>::SMEM, slot_tiles<0, 1>);
    family(k_face_pipe<1>, 1, Tile<1, 1>::SMEM, slot_tiles<1, 1>);
    family(k_face_pipe<2>, 2, Tile<2, 1>::SMEM, slot_tiles<2, 1>);
    tab.maps_off = sizeof(TmaTable) <= 64 ? 64 : 128;
    tab.starts_off = tab.maps_off + sizeof(CUtensorMap) * maps.size();
    *bytes = tab.starts_off + sizeof(int) * starts.size();
    std::vector<unsigned char> host(*bytes, 0);
    std::memcpy(host.data(), &tab, sizeof(tab));
    std::memcpy(host.data() + tab.maps_off, maps.data(), sizeof(CUtensorMap) * maps.size());
    std::memcpy(host.data() + tab.starts_off, starts.data(), sizeof(int) * starts.size());
    (void)nslot;
    void *d = nullptr;
    check_cuda(cudaMalloc(&d, *bytes), "cudaMalloc(face tile tables)");
    check_cuda(cudaMemcpy(d, host.data(), *bytes, cudaMemcpyHostToDevice), "cudaMemcpy(face tile tables)");
    // the launches read the table's header on the host: a host copy beside the device one
    static_assert(sizeof(TmaTable) <= 64, "table header");
    std::memcpy(host_header, &tab, sizeof(tab));
    return d;
}

void launch_face_tma(const LaunchCtx &ctx, const Phys &P, const PhysW<float> &PC, const GeoW<float> &GW, Flow<float> W,
                     const DevWall *walls)
{
    const Batch &B = ctx.batch;
    const unsigned char *tbl = (const unsigned char *)ctx.face_tma;
    const TmaTable &tab = *(const TmaTable *)ctx.face_tma_host;
    const CUtensorMap *maps = (const CUtensorMap *)(tbl + tab.maps_off);
    const int *starts = (const int *)(tbl + tab.starts_off);
    if (tab.form == 2) {
        const int ns = B.nsolve + 1;
        k_face_pipe<0><<<tab.grid[0], 256, Tile<0, 1>::SMEM, ctx.stream>>>(B, P, PC, GW, W, walls, maps, starts, tab.ntiles[0]);
        k_face_pipe<1><<<tab.grid[1], 256, Tile<1, 1>::SMEM, ctx.stream>>>(B, P, PC, GW, W, walls, maps, starts + ns, tab.ntiles[1]);
        k_face_pipe<2><<<tab.grid[2], 256, Tile<2, 1>::SMEM, ctx.stream>>>(B, P, PC, GW, W, walls, maps, starts + 2 * ns, tab.ntiles[2]);
        return;
    }
    // a slot smaller than the largest has fewer tiles along every direction, so the largest
    // extents bound every slot's tile count
    auto tiles = [&](int F, int JT, int IT) {
        const int ni = ctx.maxIM - 1 + (F == 0), nj = ctx.maxJM - 1 + (F == 1), nk = ctx.maxKM - 1 + (F == 2);
        return (unsigned)(((nk + KT - 1) / KT) * ((nj + JT - 1) / JT) * ((ni + IT - 1) / IT));
    };
    k_face_tile<0><<<dim3(tiles(0, Tile<0, 0>::JT, Tile<0, 0>::IT), B.nsolve), 128, Tile<0, 0>::SMEM, ctx.stream>>>(B, P, PC, GW, W, walls, maps);
    k_face_tile<1><<<dim3(tiles(1, Tile<1, 0>::JT, Tile<1, 0>::IT), B.nsolve), 128, Tile<1, 0>::SMEM, ctx.stream>>>(B, P, PC, GW, W, walls, maps);
    k_face_tile<2><<<dim3(tiles(2, Tile<2, 0>::JT, Tile<2, 0>::IT), B.nsolve), 128, Tile<2, 0>::SMEM, ctx.stream>>>(B, P, PC, GW, W, walls, maps);
}

}  // namespace gbt
