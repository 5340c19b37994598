// sf_step_tile.cu -- single-grid step kernels over warp tiles (sf_tile.cuh).
//
// k_step_tile:  float4 warp tiles (tile4_run), W warps of 32 k x 4R rows per
//               block; needs nz % 4 == 0, 16-byte aligned fields and 32-bit
//               cell offsets, else the launcher falls back to the first
//               column configuration.
// k_step_tile1: scalar warp tiles (tile1_run), W warps of 32 k x R rows.
// Blocks take i-chunks of ich planes, high to low on alternate steps (a step
// starts on the planes the previous one wrote last, still in L2), and skip
// the tile-aligned region a split ADE step leaves to the per-cell kernel.
#include <cuda_runtime.h>

#include <climits>

#include "sf_common.cuh"
#include "sf_kernels.h"
#include "sf_tile.cuh"

namespace {

// Whether the block whose tile starts at (i0, j0, k0) lies in the
// tile-aligned region that a split ADE step leaves to the per-cell kernel
// (whole blocks only: the region's bounds are multiples of the tile spans).
__device__ __forceinline__ bool in_skip(const SfStepArgs& a, int i0, int j0, int k0) {
    return i0 >= a.skip_lo[0] && i0 < a.skip_hi[0] && j0 >= a.skip_lo[1] && j0 < a.skip_hi[1] &&
           k0 >= a.skip_lo[2] && k0 < a.skip_hi[2];
}

__device__ __forceinline__ SfTileIo tile_io(const SfStepArgs& a) {
    SfTileIo io;
    io.nx = a.nx;
    io.ny = a.ny;
    io.nz = a.nz;
    io.plane = a.plane;
    io.cv = a.cv;
    io.cp = a.cp;
    io.p = a.p;
    io.vx = a.vx;
    io.vy = a.vy;
    io.vz = a.vz;
    io.po = a.po;
    io.vxo = a.vxo;
    io.vyo = a.vyo;
    io.vzo = a.vzo;
    io.flags = a.flags;
    io.dx = a.dx;
    io.dy = a.dy;
    io.dz = a.dz;
    io.src_val = a.src_val;
    for (int q = 0; q < 3; ++q) {
        io.nu_cv[q] = a.nu_cv[q];
        io.nu_inv[q] = a.nu_inv[q];
    }
    return io;
}

template <bool GEOM, int R, int W, int MINB, bool PF, bool NU, bool WB>
__global__ void __launch_bounds__(32 * W, MINB) k_step_tile(SfStepArgs a, SfSources src, int ich) {
    const int jw = (blockIdx.y * W + threadIdx.y) * (4 * R);  // the warp's first row
    const int chunk = a.reverse ? (int)(gridDim.z - 1 - blockIdx.z) : (int)blockIdx.z;
    const int i0 = chunk * ich;
    const int i1 = min(i0 + ich, a.nx);
    if (a.trace_prev != nullptr && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0) {
        for (int t = threadIdx.y * 32 + threadIdx.x; t < a.n_probe; t += 32 * W)
            a.trace_prev[t] = a.p[a.probe_cells[t]];
    }
    if (jw >= a.ny) return;  // the whole warp is past the grid (no block barrier follows)
    if (in_skip(a, i0, blockIdx.y * W * 4 * R, blockIdx.x * 32)) return;  // the ADE kernel's cells
    tile4_run<GEOM, R, PF, NU, WB>(tile_io(a), src, i0, i1, jw, blockIdx.x * 32,
                                   SfPlainMem{a.ny * a.nz});
}

// Scalar warp tiles: 32 lanes along k, R rows per lane, W warps along j.
template <bool GEOM, int R, int W, int MINB, bool PF, bool NU>
__global__ void __launch_bounds__(32 * W, MINB) k_step_tile1(SfStepArgs a, SfSources src, int ich) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int jb = (blockIdx.y * W + threadIdx.y) * R;
    const int chunk = a.reverse ? (int)(gridDim.z - 1 - blockIdx.z) : (int)blockIdx.z;
    const int i0 = chunk * ich;
    const int i1 = min(i0 + ich, a.nx);
    if (a.trace_prev != nullptr && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0) {
        for (int t = threadIdx.y * 32 + threadIdx.x; t < a.n_probe; t += 32 * W)
            a.trace_prev[t] = a.p[a.probe_cells[t]];
    }
    if (jb >= a.ny) return;  // the whole warp is past the grid
    if (in_skip(a, i0, blockIdx.y * W * R, blockIdx.x * 32)) return;  // the ADE kernel's cells
    tile1_run<GEOM, R, PF, NU>(tile_io(a), src, i0, i1, jb, k);
}

template <int R, int W, int MINB, bool PF>
int launch1(const SfStepArgs& a, const SfSources& src, bool geom, int ich, cudaStream_t st) {
    dim3 blk(32, W, 1);
    dim3 grd((a.nz + 31) / 32, (a.ny + R * W - 1) / (R * W), (a.nx + ich - 1) / ich);
    if (a.nu_cv[0] != nullptr) {
        if (geom) k_step_tile1<true, R, W, MINB, PF, true><<<grd, blk, 0, st>>>(a, src, ich);
        else k_step_tile1<false, R, W, MINB, PF, true><<<grd, blk, 0, st>>>(a, src, ich);
    } else {
        if (geom) k_step_tile1<true, R, W, MINB, PF, false><<<grd, blk, 0, st>>>(a, src, ich);
        else k_step_tile1<false, R, W, MINB, PF, false><<<grd, blk, 0, st>>>(a, src, ich);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_step_tile1 launch failed");
}

template <int R, int W, int MINB, bool PF, bool WB = false>
int launch(const SfStepArgs& a, const SfSources& src, bool geom, int ich, cudaStream_t st) {
    dim3 blk(32, W, 1);
    const int rows = 4 * R * W;
    dim3 grd((a.nz + 31) / 32, (a.ny + rows - 1) / rows, (a.nx + ich - 1) / ich);
    if (a.nu_cv[0] != nullptr) {
        if (geom) k_step_tile<true, R, W, MINB, PF, true, WB><<<grd, blk, 0, st>>>(a, src, ich);
        else k_step_tile<false, R, W, MINB, PF, true, WB><<<grd, blk, 0, st>>>(a, src, ich);
    } else {
        if (geom) k_step_tile<true, R, W, MINB, PF, false, WB><<<grd, blk, 0, st>>>(a, src, ich);
        else k_step_tile<false, R, W, MINB, PF, false, WB><<<grd, blk, 0, st>>>(a, src, ich);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_step_tile launch failed");
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

// Warp-tile configurations (index = SF_CFG_COL_FIRST + kSfColConfigCount + position).
const SfTileConfig kSfTileConfigs[] = {
    // cells per lane along k, rows per lane, warps per block, min blocks, prefetch, name
    {4, 1, 4, 6, 1, "tile_r1_w4_pf"},
    {4, 1, 8, 3, 1, "tile_r1_w8_pf"},
    {4, 1, 4, 8, 0, "tile_r1_w4"},
    {4, 2, 4, 4, 0, "tile_r2_w4"},
    {4, 2, 2, 8, 0, "tile_r2_w2"},
    {4, 1, 2, 16, 0, "tile_r1_w2"},
    {4, 1, 8, 4, 0, "tile_r1_w8"},
    {4, 1, 4, 6, 0, "tile_r1_w4_m6"},
    {1, 4, 4, 4, 0, "tile1_r4_w4"},
    {1, 2, 8, 3, 1, "tile1_r2_w8_pf"},
    {1, 2, 4, 8, 0, "tile1_r2_w4"},
    {1, 2, 8, 4, 0, "tile1_r2_w8"},
    {1, 1, 8, 4, 1, "tile1_r1_w8_pf"},
    {1, 2, 4, 6, 1, "tile1_r2_w4_pf"},
    {4, 1, 4, 6, 0, "tile_r1_w4_m6_wb"},
    {4, 1, 8, 4, 0, "tile_r1_w8_wb"},
};
const int kSfTileConfigCount = sizeof(kSfTileConfigs) / sizeof(kSfTileConfigs[0]);

bool sf_tile_supported(const SfStepArgs& a, int vec) {
    if (vec == 1) return (long long)a.ny * a.nz + a.nz + 64 < (long long)INT_MAX;
    const long long n = (long long)a.nx * a.ny * a.nz;
    if (a.nz % 4 != 0 || n + 2LL * a.ny * a.nz + 8 >= (long long)INT_MAX) return false;
    return aligned16(a.p) && aligned16(a.vx) && aligned16(a.vy) && aligned16(a.vz) &&
           aligned16(a.po) && aligned16(a.vxo) && aligned16(a.vyo) && aligned16(a.vzo) &&
           (a.flags == nullptr || (reinterpret_cast<uintptr_t>(a.flags) & 3u) == 0);
}

int sf_launch_step_tile_cfg(const SfStepArgs& a, const SfSources& src, bool geom, int cfg, int ich,
                            cudaStream_t st) {
    if (ich < 1) ich = 1;
    if (cfg < 0 || cfg >= kSfTileConfigCount) return sf_fail("k_step_tile: bad configuration");
    if (!sf_tile_supported(a, kSfTileConfigs[cfg].vec))
        return sf_launch_step_col_cfg(a, src, geom, 0, ich, st);
    switch (cfg) {
        case 0: return launch<1, 4, 6, true>(a, src, geom, ich, st);
        case 1: return launch<1, 8, 3, true>(a, src, geom, ich, st);
        case 2: return launch<1, 4, 8, false>(a, src, geom, ich, st);
        case 3: return launch<2, 4, 4, false>(a, src, geom, ich, st);
        case 4: return launch<2, 2, 8, false>(a, src, geom, ich, st);
        case 5: return launch<1, 2, 16, false>(a, src, geom, ich, st);
        case 6: return launch<1, 8, 4, false>(a, src, geom, ich, st);
        case 7: return launch<1, 4, 6, false>(a, src, geom, ich, st);
        case 8: return launch1<4, 4, 4, false>(a, src, geom, ich, st);
        case 9: return launch1<2, 8, 3, true>(a, src, geom, ich, st);
        case 10: return launch1<2, 4, 8, false>(a, src, geom, ich, st);
        case 11: return launch1<2, 8, 4, false>(a, src, geom, ich, st);
        case 12: return launch1<1, 8, 4, true>(a, src, geom, ich, st);
        case 13: return launch1<2, 4, 6, true>(a, src, geom, ich, st);
        case 14: return launch<1, 4, 6, false, true>(a, src, geom, ich, st);
        case 15: return launch<1, 8, 4, false, true>(a, src, geom, ich, st);
    }
    return sf_fail("k_step_tile: bad configuration");
}
