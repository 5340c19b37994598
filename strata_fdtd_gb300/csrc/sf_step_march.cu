// sf_step_march.cu -- the fused step as a 2.5-D slab march along i.
//
// Same per-cell arithmetic as k_step in sf_step.cu (and so as the reference
// passes listed there), organised for HBM: a block owns a TJ x TK tile of
// (j, k) and walks a chunk of i planes.
//   * p(i+1), vx, vy, vz and the flag byte of the next plane are loaded one
//     plane ahead into registers, so each field crosses HBM once per step;
//   * the new x-face velocity of plane i is carried in a register to plane
//     i+1 (it is that cell's low x face);
//   * the pressure plane is staged in shared memory with a one-cell j/k halo
//     for the +y and +z faces; the low y face comes from the row above
//     through shared memory, the low z face from the lane to the left by a
//     warp shuffle; only tile-edge threads recompute a neighbour's face.
// Each cell therefore reads 17 bytes (p, vx, vy, vz, flags) and writes 16
// (p, vx, vy, vz) of DRAM per step; the tile halos and the first plane of
// each chunk are re-read from L2.
#include <cuda_runtime.h>

#include "sf_common.cuh"

namespace {

constexpr int TK = 32;  // lanes along k (one warp per tile row)
constexpr int TJ = 8;   // tile rows along j

template <bool GEOM>
__global__ void __launch_bounds__(TK* TJ) k_step_march(SfStepArgs a, SfSources src, int ich) {
    __shared__ float s_p[TJ + 2][TK + 2];
    __shared__ float s_vy[TJ][TK];

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int k0 = blockIdx.x * TK, j0 = blockIdx.y * TJ;
    const int k = k0 + tx, j = j0 + ty;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int i0 = blockIdx.z * ich;
    const int i1 = min(i0 + ich, nx);

    if (a.trace_prev != nullptr && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0) {
        for (int t = ty * TK + tx; t < a.n_probe; t += TK * TJ)
            a.trace_prev[t] = a.p[a.probe_cells[t]];
    }

    const bool in = (k < nz) && (j < ny);
    const long long plane = a.plane;
    const long long col = (long long)j * nz + k;
    const float cv = a.cv, cp = a.cp;
    const float dj = in ? a.dy[j] : 1.0f;
    const float dk = in ? a.dz[k] : 1.0f;

    // plane i0 (current) and i0+1 (next) in registers
    float pc = 0.f, vxc = 0.f, vyc = 0.f, vzc = 0.f;
    uint8_t fc = SF_ALL;
    float pn = 0.f, vxn = 0.f, vyn = 0.f, vzn = 0.f;
    uint8_t fn = SF_ALL;
    float vxm = 0.0f;  // new x-face velocity of plane i-1 (low x face of plane i)
    if (in) {
        const long long c = (long long)i0 * plane + col;
        pc = a.p[c];
        vxc = a.vx[c];
        vyc = a.vy[c];
        vzc = a.vz[c];
        if (GEOM) fc = a.flags[c];
        if (i0 + 1 < nx) {
            pn = a.p[c + plane];
            if (i0 + 1 < i1) {
                vxn = a.vx[c + plane];
                vyn = a.vy[c + plane];
                vzn = a.vz[c + plane];
                if (GEOM) fn = a.flags[c + plane];
            }
        }
        if (i0 > 0) {  // chunk start: recompute the low x face from plane i0-1
            const long long m = c - plane;
            vxm = face_update(a.vx[m], cv, pc, a.p[m]);
            if (GEOM && !(a.flags[m] & SF_OPX)) vxm = 0.0f;
        }
    }

    for (int i = i0; i < i1; ++i) {
        const long long c = (long long)i * plane + col;
        // prefetch plane i+2
        float pnn = 0.f, vxnn = 0.f, vynn = 0.f, vznn = 0.f;
        uint8_t fnn = SF_ALL;
        if (in && i + 2 < nx && i + 2 <= i1) {
            const long long q = c + 2 * plane;
            pnn = a.p[q];
            if (i + 2 < i1) {
                vxnn = a.vx[q];
                vynn = a.vy[q];
                vznn = a.vz[q];
                if (GEOM) fnn = a.flags[q];
            }
        }

        // stage p(i) with its j/k halo
        s_p[ty + 1][tx + 1] = pc;
        if (ty == 0) s_p[0][tx + 1] = (k < nz && j0 > 0 && j0 - 1 < ny) ? a.p[c - nz] : 0.0f;
        if (ty == TJ - 1)
            s_p[TJ + 1][tx + 1] = (k < nz && j + 1 < ny) ? a.p[c + nz] : 0.0f;
        if (tx == 0) s_p[ty + 1][0] = (j < ny && k0 > 0) ? a.p[c - 1] : 0.0f;
        if (tx == TK - 1) s_p[ty + 1][TK + 1] = (j < ny && k + 1 < nz) ? a.p[c + 1] : 0.0f;
        __syncthreads();

        // high faces of this cell
        float ux = vxc, uy = vyc, uz = vzc;
        if (in) {
            if (i < nx - 1) {
                ux = face_update(vxc, cv, pn, pc);
                if (GEOM && !(fc & SF_OPX)) ux = 0.0f;
            }
            if (j < ny - 1) {
                uy = face_update(vyc, cv, s_p[ty + 2][tx + 1], pc);
                if (GEOM && !(fc & SF_OPY)) uy = 0.0f;
            }
            if (k < nz - 1) {
                uz = face_update(vzc, cv, s_p[ty + 1][tx + 2], pc);
                if (GEOM && !(fc & SF_OPZ)) uz = 0.0f;
            }
        }
        // low z face: from the lane to the left, or recomputed at the tile edge
        float uzm = __shfl_up_sync(0xffffffffu, uz, 1);
        if (tx == 0) {
            uzm = 0.0f;
            if (in && k > 0) {
                uzm = face_update(a.vz[c - 1], cv, pc, s_p[ty + 1][0]);
                if (GEOM && !(a.flags[c - 1] & SF_OPZ)) uzm = 0.0f;
            }
        }
        s_vy[ty][tx] = uy;
        __syncthreads();
        // low y face: from the row above, or recomputed at the tile edge
        float uym = 0.0f;
        if (in && j > 0) {
            if (ty > 0) {
                uym = s_vy[ty - 1][tx];
            } else {
                uym = face_update(a.vy[c - nz], cv, pc, s_p[0][tx + 1]);
                if (GEOM && !(a.flags[c - nz] & SF_OPY)) uym = 0.0f;
            }
        }

        if (in) {
            const bool air = (fc & SF_AIR) != 0;
            float pnew = air ? f_add(pc, f_mul(cp, f_add(f_add(f_sub(ux, vxm), f_sub(uy, uym)),
                                                          f_sub(uz, uzm))))
                             : 0.0f;
            const float di = a.dx[i];
            a.vxo[c] = f_mul(ux, di);
            a.vyo[c] = f_mul(uy, dj);
            a.vzo[c] = f_mul(uz, dk);
            pnew = f_mul(f_mul(f_mul(pnew, di), dj), dk);
#pragma unroll 1
            for (int q = 0; q < src.n; ++q) {
                const sf_source& S = src.s[q];
                bool hit;
                if (S.kind == 0)
                    hit = (i == S.a) && (j == S.b) && (k == S.c);
                else
                    hit = (S.a == 0) ? (i == S.b) : ((S.a == 1) ? (j == S.b) : (k == S.b));
                if (hit && air) pnew = __double2float_rn(d_add((double)pnew, a.src_val[q]));
            }
            a.po[c] = pnew;
        }

        vxm = ux;
        pc = pn;
        vxc = vxn;
        vyc = vyn;
        vzc = vzn;
        fc = fn;
        pn = pnn;
        vxn = vxnn;
        vyn = vynn;
        vzn = vznn;
        fn = fnn;
    }
}

}  // namespace

int sf_launch_step_march(const SfStepArgs& a, const SfSources& src, bool geom, int ich,
                         cudaStream_t st) {
    if (ich < 1) ich = 1;
    dim3 blk(TK, TJ, 1);
    dim3 grd((a.nz + TK - 1) / TK, (a.ny + TJ - 1) / TJ, (a.nx + ich - 1) / ich);
    if (geom)
        k_step_march<true><<<grd, blk, 0, st>>>(a, src, ich);
    else
        k_step_march<false><<<grd, blk, 0, st>>>(a, src, ich);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_step_march launch failed");
}
