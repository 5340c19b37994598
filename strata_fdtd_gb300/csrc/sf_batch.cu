// sf_batch.cu -- many independent grids of different sizes, stepped together.
//
// A batch gathers plans (each a complete single-grid solve: fields, flags,
// PML, sources, probes, ADE) and advances them with one persistent launch
// per time step.  Every grid is cut into work items (i-chunk x a block of
// rows x 32 columns); the warps of the persistent kernel claim items one at a
// time from a device-wide work queue (one atomic counter, no block
// barriers), so uneven grids load-balance across the SMs.  Items that meet a
// grid's material box run the ADE column path (the arithmetic and order of
// core/solver.py:2135-2193 and ade.cpp); the others run the batch's plain
// path: thread columns or warp tiles (sf_tile.cuh).  Every path is the
// per-cell arithmetic of k_step, so a grid's result is bit-identical alone
// or in the batch.
//
// Per step the batch enqueues: the ADE density pre-pass over the material
// boxes (if any grid has density poles), the persistent kernel, the probe
// gather, and a one-thread kernel that advances the device step counter and
// resets the queue.  The kernels read the step number from device memory, so
// a run of steps can be captured once as a CUDA graph and replayed.  Grids
// drop out of the work when they reach their own step count: members are
// listed longest run first, so a finished grid's items end their segment of
// the queue, and the first warp to claim one skips the rest of the segment.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "sf_common.cuh"
#include "sf_kernels.h"
#include "sf_plan_internal.h"
#include "sf_tile.cuh"

struct SfGridDev {
    int nx, ny, nz, ich;
    int jspan;  // rows per tile
    int vec4;   // plain tiles run as float4 warp tiles (nz % 4 == 0, aligned, 32-bit offsets)
    long long plane, n_steps;
    float cv, cp;
    int cur0, n_probe;
    float* f[2][4];
    const uint8_t* flags;
    const float* dx;
    const float* dy;
    const float* dz;
    const double* src_val;
    const long long* probe_cells;
    float* trace;
    const uint8_t* mat;
    int ade_lo[3], ade_hi[3];
    SfSources src;
    SfPoles poles;
    // nonuniform grid (warp-tile items only): per-face velocity coefficients
    // and per-cell inverse spacings per axis, or null
    const float* nu_cv[3];
    const float* nu_inv[3];
    // microphone rows sampled after each step (k_mic_gather's arithmetic)
    int n_mic;
    const int* mic_field;
    const long long* mic_idx;
    const float* mic_w;
    float* mic_trace;
};

namespace {

__device__ __forceinline__ float ade_face_g(float v, const SfPoles& P, uint8_t m_lo, uint8_t m_hi,
                                            long long lo, long long hi) {
    if (m_lo == 0 || m_lo != m_hi) return v;
    for (int q = 0; q < P.n; ++q) {
        const sf_pole& pl = P.p[q];
        if (pl.target == 0 && pl.material_id == m_lo)
            v = f_add(v, f_mul(pl.corr, f_sub(pl.J[hi], pl.J[lo])));
    }
    return v;
}

// One row of an item: lane l of the warp walks cells (i0..i1-1, j, kb*32 + l)
// of grid g at step s, as k_step_col does.
template <bool GEOM, bool ADE>
__device__ void batch_column(const SfGridDev& g, long long s, int chunk, int j, int kb,
                             bool trial) {
    const int k = kb * 32 + (threadIdx.x & 31);
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    if (k >= nz || j >= ny) return;
    const int i0 = chunk * g.ich;
    const int i1 = min(i0 + g.ich, nx);
    const int in = (int)((g.cur0 + s) & 1);
    const float* __restrict__ P = g.f[in][0];
    const float* __restrict__ VX = g.f[in][1];
    const float* __restrict__ VY = g.f[in][2];
    const float* __restrict__ VZ = g.f[in][3];
    float* __restrict__ PO = g.f[1 - in][0];
    float* __restrict__ VXO = g.f[1 - in][1];
    float* __restrict__ VYO = g.f[1 - in][2];
    float* __restrict__ VZO = g.f[1 - in][3];
    const uint8_t* __restrict__ F = g.flags;
    const uint8_t* __restrict__ M = g.mat;
    const float* __restrict__ DX = g.dx;
    constexpr bool geom = GEOM;
    constexpr bool ade = ADE;
    const long long plane = g.plane;
    const float cv = g.cv, cp = g.cp;
    const float dj = g.dy[j], dk = g.dz[k];
    const double* sv = g.src_val + s * g.src.n;

    unsigned smask = 0;
    for (int q = 0; q < g.src.n; ++q) {
        const sf_source& S = g.src.s[q];
        bool can;
        if (S.kind == 0) can = (S.b == j) && (S.c == k);
        else if (S.a == 0) can = true;
        else if (S.a == 1) can = (S.b == j);
        else can = (S.b == k);
        if (can) smask |= 1u << q;
    }

    long long c = (long long)i0 * plane + (long long)j * nz + k;
    float pc = P[c], vxc = VX[c], vyc = VY[c], vzc = VZ[c];
    uint8_t fc = geom ? F[c] : (uint8_t)SF_ALL;
    float pn = (i0 + 1 < nx) ? P[c + plane] : 0.0f;
    float vxm = 0.0f;
    if (i0 > 0) {
        const long long m = c - plane;
        vxm = face_update(VX[m], cv, pc, P[m]);
        if (ade) vxm = ade_face_g(vxm, g.poles, M[m], M[c], m, c);
        if (geom && !(F[m] & SF_OPX)) vxm = 0.0f;
    }

    for (int i = i0; i < i1; ++i, c += plane) {
        float pnn = 0.0f, vxn = 0.0f, vyn = 0.0f, vzn = 0.0f;
        uint8_t fnn = SF_ALL;
        if (i + 1 < i1) {
            vxn = VX[c + plane];
            vyn = VY[c + plane];
            vzn = VZ[c + plane];
            if (geom) fnn = F[c + plane];
            if (i + 2 < nx) pnn = P[c + 2 * plane];
        }
        const uint8_t mc = ade ? M[c] : (uint8_t)0;

        float ux = vxc, uy = vyc, uz = vzc;
        if (i < nx - 1) {
            ux = face_update(vxc, cv, pn, pc);
            if (ade) ux = ade_face_g(ux, g.poles, mc, M[c + plane], c, c + plane);
            if (geom && !(fc & SF_OPX)) ux = 0.0f;
        }
        if (j < ny - 1) {
            uy = face_update(vyc, cv, P[c + nz], pc);
            if (ade) uy = ade_face_g(uy, g.poles, mc, M[c + nz], c, c + nz);
            if (geom && !(fc & SF_OPY)) uy = 0.0f;
        }
        if (k < nz - 1) {
            uz = face_update(vzc, cv, P[c + 1], pc);
            if (ade) uz = ade_face_g(uz, g.poles, mc, M[c + 1], c, c + 1);
            if (geom && !(fc & SF_OPZ)) uz = 0.0f;
        }
        float uym = 0.0f, uzm = 0.0f;
        if (j > 0) {
            const long long m = c - nz;
            uym = face_update(VY[m], cv, pc, P[m]);
            if (ade) uym = ade_face_g(uym, g.poles, M[m], mc, m, c);
            if (geom && !(F[m] & SF_OPY)) uym = 0.0f;
        }
        if (k > 0) {
            const long long m = c - 1;
            uzm = face_update(VZ[m], cv, pc, P[m]);
            if (ade) uzm = ade_face_g(uzm, g.poles, M[m], mc, m, c);
            if (geom && !(F[m] & SF_OPZ)) uzm = 0.0f;
        }

        const bool air = (fc & SF_AIR) != 0;
        const float ddx = f_sub(ux, vxm), ddy = f_sub(uy, uym), ddz = f_sub(uz, uzm);
        float pnew = air ? f_add(pc, f_mul(cp, f_add(f_add(ddx, ddy), ddz))) : 0.0f;
        if (ade && mc != 0 && g.poles.n_modulus > 0) {
            const float sc = g.poles.inv_dx;
            const float div = f_add(f_add(f_mul(ddx, sc), f_mul(ddy, sc)), f_mul(ddz, sc));
            for (int q = 0; q < g.poles.n; ++q) {
                const sf_pole& pl = g.poles.p[q];
                if (pl.target != 1 || pl.material_id != mc) continue;
                const float j0 = pl.J[c];
                float jn;
                if (pl.kind == 0) {
                    jn = f_add(f_mul(pl.c0, j0), f_mul(pl.c1, div));
                } else {
                    const float jp = pl.J_prev[c];
                    jn = f_add(f_add(f_mul(pl.c0, j0), f_mul(pl.c1, jp)), f_mul(pl.c2, div));
                    if (!trial) pl.J_prev[c] = j0;
                }
                if (!trial) pl.J[c] = jn;
                pnew = f_add(pnew, f_mul(pl.corr, jn));
            }
            if (!air) pnew = 0.0f;
        }
        const float di = DX[i];
        VXO[c] = f_mul(ux, di);
        VYO[c] = f_mul(uy, dj);
        VZO[c] = f_mul(uz, dk);
        pnew = f_mul(f_mul(f_mul(pnew, di), dj), dk);
        for (unsigned mm = smask; mm != 0; mm &= mm - 1) {
            const int q = __ffs(mm) - 1;
            const sf_source& S = g.src.s[q];
            const bool hit = (S.kind == 0) ? (i == S.a) : (S.a == 0 ? (i == S.b) : true);
            if (hit && air) pnew = __double2float_rn(d_add((double)pnew, sv[q]));
        }
        PO[c] = pnew;

        vxm = ux;
        pc = pn;
        pn = pnn;
        vxc = vxn;
        vyc = vyn;
        vzc = vzn;
        fc = fnn;
    }
}

// Does the tile (with a one-cell margin, for the neighbours' faces) reach
// the grid's material box?  Outside it every ADE term is absent, so such
// tiles go to the plain kernel.
__host__ __device__ __forceinline__ bool tile_meets_box(const SfGridDev& g, int chunk, int jb,
                                                        int kb) {
    const int by = g.jspan;
    const int i0 = chunk * g.ich - 1, i1 = chunk * g.ich + g.ich + 1;
    const int j0 = jb * by - 1, j1 = jb * by + by + 1;
    const int k0 = kb * 32 - 1, k1 = kb * 32 + 33;
    return i1 > g.ade_lo[0] && i0 < g.ade_hi[0] && j1 > g.ade_lo[1] && j0 < g.ade_hi[1] &&
           k1 > g.ade_lo[2] && k0 < g.ade_hi[2];
}

// Persistent warp loop over the step's work items (grid, i-chunk, row block,
// k block).  Every warp claims items on its own -- one atomic per item, no
// block barrier -- so items of all sizes and kinds balance across the SMs.
// Items that meet a grid's material box come first in the list and run the
// ADE column path; the others run the batch's plain path: thread columns
// (KIND 0) or warp tiles (sf_tile.cuh; KIND 1, and 2 with the next plane
// loaded ahead; 3 the same with fewer registers and more resident warps),
// float4 tiles where the grid's fields allow them.  The grid
// descriptor is read in place (global memory, L1-resident while a warp
// works through its items).
template <int W, int MINB, int KIND>
__global__ void __launch_bounds__(32 * W, MINB) k_batch_warp(
    const SfGridDev* __restrict__ grids, const int4* __restrict__ items, int n_items, int n_ade,
    int* __restrict__ queue, const long long* __restrict__ step_ptr, int trial) {
    constexpr bool PF = KIND >= 2;
    const int lane = threadIdx.x;
    const long long s = *step_ptr;
    for (;;) {
        int it = 0;
        if (lane == 0) {
            it = atomicAdd(queue, 1);
            // members are listed longest run first, so a finished member's
            // item is followed by finished members' items only: skip to the
            // plain items, or stop after them
            if (it < n_items && s >= grids[items[it].x].n_steps) {
                if (it < n_ade) {
                    atomicMax(queue, n_ade);
                    it = -1;
                } else {
                    it = n_items;
                }
            }
        }
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= n_items) return;  // warp-uniform
        if (it < 0) continue;
        const int4 T = items[it];   // grid, i-chunk, row block, k block
        const SfGridDev& g = grids[T.x];
        if (s >= g.n_steps) continue;
        const bool geom = g.flags != nullptr;
        const int j0 = T.z * g.jspan;
        if (it < n_ade || KIND == 0) {
            const int j_end = min(j0 + g.jspan, g.ny);
            const bool ade = it < n_ade;
#pragma unroll 1
            for (int j = j0; j < j_end; ++j) {
                if (geom) {
                    if (ade) batch_column<true, true>(g, s, T.y, j, T.w, trial != 0);
                    else batch_column<true, false>(g, s, T.y, j, T.w, trial != 0);
                } else {
                    if (ade) batch_column<false, true>(g, s, T.y, j, T.w, trial != 0);
                    else batch_column<false, false>(g, s, T.y, j, T.w, trial != 0);
                }
            }
            continue;
        }
        const int in = (int)((g.cur0 + s) & 1);
        SfTileIo io;
        io.nx = g.nx;
        io.ny = g.ny;
        io.nz = g.nz;
        io.plane = g.plane;
        io.cv = g.cv;
        io.cp = g.cp;
        io.p = g.f[in][0];
        io.vx = g.f[in][1];
        io.vy = g.f[in][2];
        io.vz = g.f[in][3];
        io.po = g.f[1 - in][0];
        io.vxo = g.f[1 - in][1];
        io.vyo = g.f[1 - in][2];
        io.vzo = g.f[1 - in][3];
        io.flags = g.flags;
        io.dx = g.dx;
        io.dy = g.dy;
        io.dz = g.dz;
        io.src_val = g.src_val + s * g.src.n;
        const int i0 = T.y * g.ich;
        const int i1 = min(i0 + g.ich, g.nx);
        if (g.vec4) {
            const SfPlainMem mem{io.ny * io.nz};
            if (geom) tile4_run<true, 1, PF, false, true>(io, g.src, i0, i1, j0, T.w * 32, mem);
            else tile4_run<false, 1, PF, false, true>(io, g.src, i0, i1, j0, T.w * 32, mem);
        } else {
            const int k = T.w * 32 + lane;
            if (geom) tile1_run<true, 2, PF>(io, g.src, i0, i1, j0, k);
            else tile1_run<false, 2, PF>(io, g.src, i0, i1, j0, k);
        }
    }
}

// The items of nonuniform members (no ADE), in a persistent kernel of their
// own: the warp tiles with per-face coefficients and per-cell divergence
// scales (NU variants of sf_tile.cuh), from the queue's second counter.
// Keeping them out of k_batch_warp keeps its register allocation as it is.
template <int W, int MINB>
__global__ void __launch_bounds__(32 * W, MINB) k_batch_warp_nu(
    const SfGridDev* __restrict__ grids, const int4* __restrict__ items, int n_items,
    int* __restrict__ queue, const long long* __restrict__ step_ptr) {
    const int lane = threadIdx.x;
    const long long s = *step_ptr;
    for (;;) {
        int it = 0;
        if (lane == 0) {
            it = atomicAdd(queue, 1);
            // a finished member's item: only finished members' items follow
            if (it < n_items && s >= grids[items[it].x].n_steps) it = n_items;
        }
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= n_items) return;  // warp-uniform
        const int4 T = items[it];
        const SfGridDev& g = grids[T.x];
        if (s >= g.n_steps) continue;
        const bool geom = g.flags != nullptr;
        const int j0 = T.z * g.jspan;
        const int in = (int)((g.cur0 + s) & 1);
        SfTileIo io;
        io.nx = g.nx;
        io.ny = g.ny;
        io.nz = g.nz;
        io.plane = g.plane;
        io.cv = g.cv;
        io.cp = g.cp;
        io.p = g.f[in][0];
        io.vx = g.f[in][1];
        io.vy = g.f[in][2];
        io.vz = g.f[in][3];
        io.po = g.f[1 - in][0];
        io.vxo = g.f[1 - in][1];
        io.vyo = g.f[1 - in][2];
        io.vzo = g.f[1 - in][3];
        io.flags = g.flags;
        io.dx = g.dx;
        io.dy = g.dy;
        io.dz = g.dz;
        io.src_val = g.src_val + s * g.src.n;
        for (int q = 0; q < 3; ++q) {
            io.nu_cv[q] = g.nu_cv[q];
            io.nu_inv[q] = g.nu_inv[q];
        }
        const int i0 = T.y * g.ich;
        const int i1 = min(i0 + g.ich, g.nx);
        if (g.vec4) {
            const SfPlainMem mem{io.ny * io.nz};
            if (geom) tile4_run<true, 1, false, true, true>(io, g.src, i0, i1, j0, T.w * 32, mem);
            else tile4_run<false, 1, false, true, true>(io, g.src, i0, i1, j0, T.w * 32, mem);
        } else {
            const int k = T.w * 32 + lane;
            if (geom) tile1_run<true, 2, false, true>(io, g.src, i0, i1, j0, k);
            else tile1_run<false, 2, false, true>(io, g.src, i0, i1, j0, k);
        }
    }
}

constexpr int kBatchWarps = 4;  // warps per block of the persistent kernel

// ADE density poles of every grid that has them, over its material box
// (ade.cpp:25-68 and 118-170), from the step's input pressure.
__global__ void k_batch_ade_density(const SfGridDev* __restrict__ grids, const int* __restrict__ ids,
                                    const long long* __restrict__ step_ptr) {
    const long long s = *step_ptr;
    const SfGridDev& g = grids[ids[blockIdx.y]];
    if (s >= g.n_steps || g.poles.n_density == 0) return;
    const float* __restrict__ P = g.f[(g.cur0 + s) & 1][0];
    const int ex = g.ade_hi[0] - g.ade_lo[0], ey = g.ade_hi[1] - g.ade_lo[1],
              ez = g.ade_hi[2] - g.ade_lo[2];
    const long long total = (long long)ex * ey * ez;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = g.ade_lo[0] + (int)(t / ((long long)ey * ez));
        const int r = (int)(t % ((long long)ey * ez));
        const int j = g.ade_lo[1] + r / ez, k = g.ade_lo[2] + r % ez;
        const long long c = (long long)i * g.plane + (long long)j * g.nz + k;
        const uint8_t mc = g.mat[c];
        if (mc == 0) continue;
        const float pc = P[c];
        for (int q = 0; q < g.poles.n; ++q) {
            const sf_pole& pl = g.poles.p[q];
            if (pl.target != 0 || pl.material_id != mc) continue;
            const float j0 = pl.J[c];
            if (pl.kind == 0) {
                pl.J[c] = f_add(f_mul(pl.c0, j0), f_mul(pl.c1, pc));
            } else {
                const float jp = pl.J_prev[c];
                pl.J[c] = f_add(f_add(f_mul(pl.c0, j0), f_mul(pl.c1, jp)), f_mul(pl.c2, pc));
                pl.J_prev[c] = j0;
            }
        }
    }
}

// Probe samples of every grid after the step (core/solver.py:2435-2439), and
// its microphone rows: 8 weighted corner values of p or a velocity
// component, summed from 0 in corner order (the arithmetic of k_mic_gather).
__global__ void k_batch_post(const SfGridDev* __restrict__ grids, const long long* __restrict__ step_ptr) {
    const long long s = *step_ptr;
    const SfGridDev& g = grids[blockIdx.x];
    if (s >= g.n_steps) return;
    float* const* f = g.f[(g.cur0 + s + 1) & 1];
    if (g.n_probe > 0 && g.trace != nullptr)
        for (int t = threadIdx.x; t < g.n_probe; t += blockDim.x)
            g.trace[s * g.n_probe + t] = f[0][g.probe_cells[t]];
    if (g.n_mic > 0 && g.mic_trace != nullptr) {
        for (int m = threadIdx.x; m < g.n_mic; m += blockDim.x) {
            const int fi = g.mic_field ? g.mic_field[m] : 0;
            const float* __restrict__ src = f[fi >= 0 && fi <= 3 ? fi : 0];
            float acc = 0.0f;
#pragma unroll
            for (int q = 0; q < 8; ++q)
                acc = f_add(acc, f_mul(g.mic_w[8 * m + q], src[g.mic_idx[8 * m + q]]));
            g.mic_trace[s * g.n_mic + m] = acc;
        }
    }
}

__global__ void k_batch_advance(long long* step_ptr, int* queue) {
    *step_ptr += 1;
    queue[0] = 0;
    queue[1] = 0;
}

}  // namespace

// ---------------------------------------------------------------------------

struct sf_batch {
    struct Member {
        sf_plan* plan;
        long long steps;
        const double* src;
        float* trace;
        float* mic_trace;
    };
    std::vector<Member> members;
    int rows = 8;
    int plain_kernel = 2;  // plain items: 0 thread columns, 1 warp tiles, 2 warp tiles + prefetch
    int i_chunk = 0;
    int device = 0;
    bool built = false;
    SfGridDev* d_grids = nullptr;
    int4* d_tiles = nullptr;  // work items: those meeting a material box first
    int n_tiles = 0;          // all work items
    int n_tiles_ade = 0;      // items that meet a material box
    int n_tiles_nu = 0;       // items of nonuniform members, after the others in d_tiles
    int blocks_nu = 0;        // persistent grid size of k_batch_warp_nu
    int* d_ade_ids = nullptr;
    int n_ade = 0;
    int ade_blocks = 1;
    int* d_queue = nullptr;   // [0] work-queue head ([1] spare)
    long long* d_step = nullptr;
    int blocks = 0;      // persistent grid size
    long long max_steps = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_steps = 0;
};

namespace {

void free_device(sf_batch* B) {
    sf_defer_graph(B->graph_exec, B->graph);  // released later, without a device-wide wait
    B->graph_exec = nullptr;
    B->graph = nullptr;
    B->graph_steps = 0;
    sf_defer_free(B->d_grids, 0);
    sf_defer_free(B->d_tiles, 0);
    sf_defer_free(B->d_ade_ids, 0);
    sf_defer_free(B->d_queue, 0);
    sf_defer_free(B->d_step, 0);
    B->d_grids = nullptr;
    B->d_tiles = nullptr;
    B->d_ade_ids = nullptr;
    B->d_queue = nullptr;
    B->d_step = nullptr;
    B->built = false;
}

int chunk_for_grid(const sf_batch* B, const sf_plan* P) {
    if (B->i_chunk > 0) return B->i_chunk;
    // about 16 planes per tile, fewer for thin grids
    return P->d.nx < 32 ? (P->d.nx + 1) / 2 : 16;
}

template <typename K>
int occupancy_blocks(K kernel, int threads, int* out) {
    int dev = 0, sms = 0, per = 0;
    SF_CUDA_OK(cudaGetDevice(&dev));
    SF_CUDA_OK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SF_CUDA_OK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0));
    *out = sms * (per > 0 ? per : 1);
    return 0;
}

// Resident blocks of 4 warps asked of the compiler: 6 caps registers at 85
// per thread (24 warps per SM), 8 at 64 (32 warps).
constexpr int kMinBlocksColumn = 6, kMinBlocksTile = 6, kMinBlocksLean = 8;

int occupancy_warp(sf_batch* B) {
    constexpr int W = kBatchWarps;
    if (B->plain_kernel == 1)
        return occupancy_blocks(k_batch_warp<W, kMinBlocksTile, 1>, 32 * W, &B->blocks);
    if (B->plain_kernel == 2)
        return occupancy_blocks(k_batch_warp<W, kMinBlocksTile, 2>, 32 * W, &B->blocks);
    if (B->plain_kernel == 3)
        return occupancy_blocks(k_batch_warp<W, kMinBlocksLean, 3>, 32 * W, &B->blocks);
    return occupancy_blocks(k_batch_warp<W, kMinBlocksColumn, 0>, 32 * W, &B->blocks);
}

int build(sf_batch* B) {
    free_device(B);
    if (B->members.empty()) return sf_fail("sf_batch: no members");
    std::vector<SfGridDev> grids;
    std::vector<int4> tiles, tiles_ade, tiles_nu;
    std::vector<int> ade_ids;
    // members by step count, longest first (then the largest work first):
    // at every step the items of the members still running are a prefix of
    // each segment (ADE, plain, nonuniform), so the kernels stop at the
    // first item of a finished member
    std::vector<int> order(B->members.size());
    for (size_t q = 0; q < order.size(); ++q) order[q] = (int)q;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const auto &ma = B->members[a], &mb = B->members[b];
        if (ma.steps != mb.steps) return ma.steps > mb.steps;
        return ma.plan->n * ma.steps > mb.plan->n * mb.steps;
    });
    B->max_steps = 0;
    long long ade_cells = 0;
    for (int q : order) {
        const auto& m = B->members[q];
        const sf_plan* P = m.plan;
        SfGridDev g{};
        g.nx = P->d.nx;
        g.ny = P->d.ny;
        g.nz = P->d.nz;
        g.ich = chunk_for_grid(B, P);
        // warp-tile plain kernels: float4 tiles where the fields allow them
        const long long n_cells = (long long)P->d.nx * P->d.ny * P->d.nz;
        bool aligned = true;
        for (int a = 0; a < 2; ++a)
            for (int f = 0; f < 4; ++f)
                aligned = aligned && (reinterpret_cast<uintptr_t>(P->f[a][f]) & 15u) == 0;
        g.vec4 = (B->plain_kernel != 0 || P->nu != nullptr) && P->d.nz % 4 == 0 && aligned &&
                 (P->flags == nullptr || (reinterpret_cast<uintptr_t>(P->flags) & 3u) == 0) &&
                 n_cells + 2LL * P->d.ny * P->d.nz + 8 < 0x7fffffffLL;
        // rows per item; a nonuniform member always takes the warp tiles
        g.jspan = (B->plain_kernel == 0 && !P->nu) ? B->rows : (g.vec4 ? 4 : 2);
        g.plane = (long long)P->d.ny * P->d.nz;
        g.n_steps = m.steps;
        g.cv = P->d.coeff_v;
        g.cp = P->d.coeff_p;
        g.cur0 = P->cur;
        g.n_probe = m.trace ? P->n_probe : 0;
        for (int a = 0; a < 2; ++a)
            for (int f = 0; f < 4; ++f) g.f[a][f] = P->f[a][f];
        g.flags = P->flags;
        g.dx = P->decay[0];
        g.dy = P->decay[1];
        g.dz = P->decay[2];
        g.src_val = m.src;
        g.probe_cells = P->probe_cells;
        g.trace = m.trace;
        g.mat = P->mat;
        for (int a = 0; a < 3; ++a) {
            g.ade_lo[a] = P->ade_lo[a];
            g.ade_hi[a] = P->ade_hi[a];
        }
        g.src = P->src;
        g.poles = P->poles;
        if (P->nu) {  // face coefficients x, y, z, then cell inverse spacings x, y, z
            const int n3[3] = {P->d.nx, P->d.ny, P->d.nz};
            long long off = 0;
            for (int a = 0; a < 3; off += n3[a], ++a) g.nu_cv[a] = P->nu + off;
            for (int a = 0; a < 3; off += n3[a], ++a) g.nu_inv[a] = P->nu + off;
        }
        g.n_mic = m.mic_trace ? P->n_mic : 0;
        g.mic_field = P->mic_field;
        g.mic_idx = P->mic_idx;
        g.mic_w = P->mic_w;
        g.mic_trace = m.mic_trace;
        const int gi = (int)grids.size();
        grids.push_back(g);
        if (g.poles.n > 0 && g.poles.n_density > 0) {
            ade_ids.push_back(gi);
            ade_cells = std::max(ade_cells, (long long)(g.ade_hi[0] - g.ade_lo[0]) *
                                                (g.ade_hi[1] - g.ade_lo[1]) * (g.ade_hi[2] - g.ade_lo[2]));
        }
        B->max_steps = std::max(B->max_steps, m.steps);
        const int nch = (g.nx + g.ich - 1) / g.ich, njb = (g.ny + g.jspan - 1) / g.jspan,
                  nkb = (g.nz + 31) / 32;
        for (int ch = 0; ch < nch; ++ch)
            for (int jb = 0; jb < njb; ++jb)
                for (int kb = 0; kb < nkb; ++kb) {
                    const bool ade = g.poles.n > 0 && tile_meets_box(g, ch, jb, kb);
                    if (g.nu_cv[0] != nullptr) tiles_nu.push_back(make_int4(gi, ch, jb, kb));
                    else (ade ? tiles_ade : tiles).push_back(make_int4(gi, ch, jb, kb));
                }
    }
    if (tiles.size() + tiles_ade.size() + tiles_nu.size() > 0x7fffffff)
        return sf_fail("sf_batch: too many tiles");
    // items meeting a material box first: they are the slowest, so they
    // start early and the step ends on short plain items
    B->n_tiles_ade = (int)tiles_ade.size();
    tiles_ade.insert(tiles_ade.end(), tiles.begin(), tiles.end());
    tiles.swap(tiles_ade);
    B->n_tiles = (int)tiles.size();
    B->n_tiles_nu = (int)tiles_nu.size();
    tiles.insert(tiles.end(), tiles_nu.begin(), tiles_nu.end());
    B->n_ade = (int)ade_ids.size();
    B->ade_blocks = (int)std::min<long long>(std::max<long long>(1, (ade_cells + 255) / 256), 512);
    SF_CUDA_OK(cudaMalloc(&B->d_grids, sizeof(SfGridDev) * grids.size()));
    SF_CUDA_OK(cudaMemcpy(B->d_grids, grids.data(), sizeof(SfGridDev) * grids.size(),
                          cudaMemcpyHostToDevice));
    SF_CUDA_OK(cudaMalloc(&B->d_tiles, sizeof(int4) * tiles.size()));
    SF_CUDA_OK(cudaMemcpy(B->d_tiles, tiles.data(), sizeof(int4) * tiles.size(), cudaMemcpyHostToDevice));
    if (!ade_ids.empty()) {
        SF_CUDA_OK(cudaMalloc(&B->d_ade_ids, sizeof(int) * ade_ids.size()));
        SF_CUDA_OK(cudaMemcpy(B->d_ade_ids, ade_ids.data(), sizeof(int) * ade_ids.size(),
                              cudaMemcpyHostToDevice));
    }
    SF_CUDA_OK(cudaMalloc(&B->d_queue, 2 * sizeof(int)));
    SF_CUDA_OK(cudaMalloc(&B->d_step, sizeof(long long)));
    if (int rc = occupancy_warp(B)) return rc;
    if (B->n_tiles_nu > 0)
        if (int rc = occupancy_blocks(k_batch_warp_nu<kBatchWarps, kMinBlocksTile>, 32 * kBatchWarps,
                                      &B->blocks_nu))
            return rc;
    B->built = true;
    return 0;
}

int launch_step_kernel(sf_batch* B, cudaStream_t st, int trial) {
    constexpr int W = kBatchWarps;
    if (B->n_tiles_nu > 0 && !trial) {  // nonuniform members: their own persistent kernel
        const int blocks = std::min(B->blocks_nu, (B->n_tiles_nu + W - 1) / W);
        k_batch_warp_nu<W, kMinBlocksTile><<<blocks, dim3(32, W), 0, st>>>(
            B->d_grids, B->d_tiles + B->n_tiles, B->n_tiles_nu, B->d_queue + 1, B->d_step);
        if (cudaGetLastError() != cudaSuccess) return sf_fail("k_batch_warp_nu launch failed");
    }
    if (B->n_tiles == 0) return 0;
    const dim3 blk(32, W);
    if (B->plain_kernel == 1)
        k_batch_warp<W, kMinBlocksTile, 1><<<B->blocks, blk, 0, st>>>(
            B->d_grids, B->d_tiles, B->n_tiles, B->n_tiles_ade, B->d_queue, B->d_step, trial);
    else if (B->plain_kernel == 2)
        k_batch_warp<W, kMinBlocksTile, 2><<<B->blocks, blk, 0, st>>>(
            B->d_grids, B->d_tiles, B->n_tiles, B->n_tiles_ade, B->d_queue, B->d_step, trial);
    else if (B->plain_kernel == 3)
        k_batch_warp<W, kMinBlocksLean, 3><<<B->blocks, blk, 0, st>>>(
            B->d_grids, B->d_tiles, B->n_tiles, B->n_tiles_ade, B->d_queue, B->d_step, trial);
    else
        k_batch_warp<W, kMinBlocksColumn, 0><<<B->blocks, blk, 0, st>>>(
            B->d_grids, B->d_tiles, B->n_tiles, B->n_tiles_ade, B->d_queue, B->d_step, trial);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_batch_warp launch failed");
}

// One batch step: ADE density pass, step, probes, advance.
int enqueue_step(sf_batch* B, cudaStream_t st) {
    if (B->n_ade > 0)
        k_batch_ade_density<<<dim3(B->ade_blocks, B->n_ade), 256, 0, st>>>(B->d_grids, B->d_ade_ids,
                                                                           B->d_step);
    if (int rc = launch_step_kernel(B, st, 0)) return rc;
    k_batch_post<<<(int)B->members.size(), 64, 0, st>>>(B->d_grids, B->d_step);
    k_batch_advance<<<1, 1, 0, st>>>(B->d_step, B->d_queue);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("sf_batch: launch failed");
}

}  // namespace

extern "C" {

int sf_batch_create(sf_batch** out) {
    if (!out) return sf_fail("sf_batch_create: NULL argument");
    auto* B = new sf_batch();
    cudaGetDevice(&B->device);
    *out = B;
    return 0;
}

int sf_batch_destroy(sf_batch* B) {
    if (!B) return 0;
    DeviceGuard g(B->device);
    free_device(B);
    delete B;
    return 0;
}

int sf_batch_add(sf_batch* B, sf_plan* P, int64_t n_steps, const double* src_values_dev,
                 float* trace_dev) {
    return sf_batch_add_ex(B, P, n_steps, src_values_dev, trace_dev, nullptr);
}

int sf_batch_add_ex(sf_batch* B, sf_plan* P, int64_t n_steps, const double* src_values_dev,
                    float* trace_dev, float* mic_trace_dev) {
    if (!B || !P) return sf_fail("sf_batch_add: NULL argument");
    if (!P->bound) return sf_fail("sf_batch_add: plan fields not bound");
    if (P->device != B->device) return sf_fail("sf_batch_add: plan on another device");
    if (P->nu && P->poles.n > 0)
        return sf_fail("sf_batch_add: nonuniform grids with ADE materials are stepped alone");
    if (P->n_mic > 0 && n_steps > 0 && !mic_trace_dev)
        return sf_fail("sf_batch_add: microphone rows need a microphone trace");
    if (P->n_plane) return sf_fail("sf_batch_add: plane boundaries are stepped alone");
    for (int q = 0; q < P->src.n; ++q)
        if (P->src.s[q].kind == 2) return sf_fail("sf_batch_add: membrane sources are stepped alone");
    if (n_steps < 0) return sf_fail("sf_batch_add: negative step count");
    if (P->src.n > 0 && n_steps > 0 && !src_values_dev)
        return sf_fail("sf_batch_add: sources need src_values");
    B->members.push_back({P, n_steps, src_values_dev, trace_dev, mic_trace_dev});
    B->built = false;
    return 0;
}

int sf_batch_clear(sf_batch* B) {
    if (!B) return sf_fail("sf_batch_clear: NULL batch");
    DeviceGuard g(B->device);
    free_device(B);
    B->members.clear();
    return 0;
}

int sf_batch_set_tiles(sf_batch* B, int rows, int i_chunk) {
    if (!B) return sf_fail("sf_batch_set_tiles: NULL batch");
    if (rows != 4 && rows != 8 && rows != 16) return sf_fail("sf_batch_set_tiles: rows must be 4, 8 or 16");
    if (i_chunk < 0) return sf_fail("sf_batch_set_tiles: negative i_chunk");
    B->rows = rows;
    B->i_chunk = i_chunk;
    B->built = false;
    return 0;
}

int sf_batch_tiles(const sf_batch* B) { return B ? B->n_tiles : -1; }

int sf_batch_set_kernel(sf_batch* B, int kind) {
    if (!B) return sf_fail("sf_batch_set_kernel: NULL batch");
    if (kind < 0 || kind > 3) return sf_fail("sf_batch_set_kernel: kind must be 0 .. 3");
    B->plain_kernel = kind;
    B->built = false;
    return 0;
}

int sf_batch_run(sf_batch* B, int64_t n_steps, int graph_steps, void* stream) {
    if (!B) return sf_fail("sf_batch_run: NULL batch");
    DeviceGuard g(B->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (!B->built)
        if (int rc = build(B)) return rc;
    if (n_steps <= 0) return 0;
    SF_CUDA_OK(cudaMemsetAsync(B->d_step, 0, sizeof(long long), st));
    SF_CUDA_OK(cudaMemsetAsync(B->d_queue, 0, 2 * sizeof(int), st));
    int64_t done = 0;
    if (graph_steps > 0 && n_steps >= graph_steps) {
        if (!B->graph_exec || B->graph_steps != graph_steps) {
            if (B->graph_exec) cudaGraphExecDestroy(B->graph_exec);
            if (B->graph) cudaGraphDestroy(B->graph);
            B->graph_exec = nullptr;
            B->graph = nullptr;
            cudaStream_t cap;
            SF_CUDA_OK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
            int rc = 0;
            if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                rc = sf_fail("sf_batch_run: stream capture failed to begin");
            } else {
                for (int q = 0; q < graph_steps && !rc; ++q) rc = enqueue_step(B, cap);
                if (cudaStreamEndCapture(cap, &B->graph) != cudaSuccess && !rc)
                    rc = sf_fail("sf_batch_run: stream capture failed");
            }
            cudaStreamDestroy(cap);
            if (rc) return rc;
            SF_CUDA_OK(cudaGraphInstantiate(&B->graph_exec, B->graph, 0));
            B->graph_steps = graph_steps;
        }
        while (n_steps - done >= graph_steps) {
            SF_CUDA_OK(cudaGraphLaunch(B->graph_exec, st));
            done += graph_steps;
        }
    }
    for (; done < n_steps; ++done)
        if (int rc = enqueue_step(B, st)) return rc;
    // the members' current sets and step counts move with the batch
    for (auto& m : B->members) {
        const long long ran = std::min<long long>(m.steps, n_steps);
        m.plan->cur = (int)((m.plan->cur + ran) & 1);
        m.plan->steps_done += ran;
        m.steps -= ran;
        if (m.src) m.src += ran * m.plan->src.n;
        if (m.trace) m.trace += ran * m.plan->n_probe;
    }
    B->built = false;  // descriptors carry cur0 / remaining steps
    return 0;
}

int sf_batch_autotune(sf_batch* B, int launches, void* stream, float* ms_out, int* best_rows,
                      int* best_chunk) {
    if (!B) return sf_fail("sf_batch_autotune: NULL batch");
    if (launches < 1) launches = 1;
    DeviceGuard g(B->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int rows_c[3] = {4, 8, 16};
    const int chunk_c[3] = {8, 16, 32};
    cudaEvent_t e0, e1;
    SF_CUDA_OK(cudaEventCreate(&e0));
    SF_CUDA_OK(cudaEventCreate(&e1));
    float best = -1.0f;
    int br = B->rows, bc = B->i_chunk;
    int rc = 0;
    for (int a = 0; a < 3 && !rc; ++a)
        for (int b = 0; b < 3 && !rc; ++b) {
            B->rows = rows_c[a];
            B->i_chunk = chunk_c[b];
            if ((rc = build(B))) break;
            // trial launches: step 0 of every member, out of place, no J writes,
            // no probes and no step advance -- the members' state is untouched
            if (cudaMemsetAsync(B->d_step, 0, sizeof(long long), st) != cudaSuccess) {
                rc = sf_fail("sf_batch_autotune: memset failed");
                break;
            }
            float ms = 0.0f;
            for (int q = 0; q <= launches && !rc; ++q) {
                if (q == 1) cudaEventRecord(e0, st);
                cudaMemsetAsync(B->d_queue, 0, 2 * sizeof(int), st);
                rc = launch_step_kernel(B, st, 1);
            }
            if (rc) break;
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                rc = sf_fail("sf_batch_autotune: timing failed");
                break;
            }
            cudaEventElapsedTime(&ms, e0, e1);
            ms /= launches;
            if (ms_out) ms_out[a * 3 + b] = ms;
            if (best < 0 || ms < best) {
                best = ms;
                br = rows_c[a];
                bc = chunk_c[b];
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    B->rows = br;
    B->i_chunk = bc;
    B->built = false;
    if (rc) return rc;
    if (best_rows) *best_rows = br;
    if (best_chunk) *best_chunk = bc;
    return 0;
}

}  // extern "C"
