// sf_step_tb.cu -- two time steps per pass over the state (temporal
// blocking with overlapped warp tiles, sf_tb.cuh).
//
// One launch advances the state by two steps: HBM sees one read of the
// input set and one write of the output set per two steps.  Warps of W per
// block are stacked along j (R output rows each); blocks cover windows of 28
// output cells along k (overlapping by 4) and chunks of planes along i,
// high to low on alternate launches.  The level-1 probe row is written by
// the warps owning the probe cells; the level-2 one is gathered from the
// output set like a single step's.  Uniform grids without ADE poles,
// microphones, plane boundaries or weighted sources, at most 32 probes
// (the caller falls back to single steps otherwise).
#include <cuda_runtime.h>

#include <climits>

#include "sf_common.cuh"
#include "sf_kernels.h"
#include "sf_tb.cuh"

namespace {

template <bool GEOM, int R, int W, int MINB>
__global__ void __launch_bounds__(32 * W, MINB) k_step_tb2(SfStepArgs a, SfSources src, int ich,
                                                           float* trace1) {
    const int chunk = a.reverse ? (int)(gridDim.z - 1 - blockIdx.z) : (int)blockIdx.z;
    const int i0 = chunk * ich;
    const int i1 = min(i0 + ich, a.nx);
    if (a.trace_prev != nullptr && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0) {
        for (int q = threadIdx.y * 32 + threadIdx.x; q < a.n_probe; q += 32 * W)
            a.trace_prev[q] = a.p[a.probe_cells[q]];
    }
    const int jw = (blockIdx.y * W + threadIdx.y) * R;
    if (jw >= a.ny) return;  // the whole warp is past the grid (no block barrier follows)
    SfTbIo io;
    io.nx = a.nx;
    io.ny = a.ny;
    io.nz = a.nz;
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
    io.val1 = a.src_val;
    io.val2 = a.src_val != nullptr ? a.src_val + src.n : nullptr;
    io.n_probe = a.n_probe;
    io.probe_cells = a.probe_cells;
    io.trace1 = trace1;
    const int W0 = (int)blockIdx.x * 28 - 2;
    if (tb2_interior(io, R, jw, W0)) tb2_warp_run<GEOM, R, false>(io, src, i0, i1, jw, W0);
    else tb2_warp_run<GEOM, R, true>(io, src, i0, i1, jw, W0);
}

template <int R, int W, int MINB>
int launch_tb(const SfStepArgs& a, const SfSources& src, bool geom, int ich, float* trace1,
              cudaStream_t st) {
    dim3 blk(32, W, 1);
    dim3 grd((a.nz + 27) / 28, (a.ny + R * W - 1) / (R * W), (a.nx + ich - 1) / ich);
    if (geom) k_step_tb2<true, R, W, MINB><<<grd, blk, 0, st>>>(a, src, ich, trace1);
    else k_step_tb2<false, R, W, MINB><<<grd, blk, 0, st>>>(a, src, ich, trace1);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_step_tb2 launch failed");
}

}  // namespace

// Two-step configurations: output rows per warp, warps per block, min blocks.
const SfTbConfig kSfTbConfigs[] = {
    {4, 4, 3, "tb2_r4_w4"},
    {6, 4, 2, "tb2_r6_w4"},
    {4, 8, 1, "tb2_r4_w8"},
    {2, 8, 2, "tb2_r2_w8"},
};
const int kSfTbConfigCount = sizeof(kSfTbConfigs) / sizeof(kSfTbConfigs[0]);

bool sf_tb_supported(const SfStepArgs& a) {
    return a.nu_cv[0] == nullptr && a.n_probe <= 32 &&
           (long long)a.ny * a.nz + 64 < (long long)INT_MAX;
}

int sf_launch_step_tb(const SfStepArgs& a, const SfSources& src, bool geom, int cfg, int ich,
                      float* trace1, cudaStream_t st) {
    if (ich < 1) ich = 1;
    switch (cfg) {
        case 0: return launch_tb<4, 4, 3>(a, src, geom, ich, trace1, st);
        case 1: return launch_tb<6, 4, 2>(a, src, geom, ich, trace1, st);
        case 2: return launch_tb<4, 8, 1>(a, src, geom, ich, trace1, st);
        case 3: return launch_tb<2, 8, 2>(a, src, geom, ich, trace1, st);
    }
    return sf_fail("k_step_tb2: bad configuration");
}
