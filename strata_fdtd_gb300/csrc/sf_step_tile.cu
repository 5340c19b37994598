// sf_step_tile.cu -- the fused step with warp tiles and register neighbours.
//
// Same per-cell arithmetic as k_step (sf_step.cu), which restates the
// reference passes listed there.  The column kernels (sf_step_col.cu) spend
// most of their issue slots re-deriving the low y and z faces of every cell
// from global memory; here a warp owns a 32 (k) x 4R (j) patch of every
// plane of its i-chunk and passes neighbour values between lanes instead:
//   * lane (lx, ly) holds 4 consecutive k cells (one float4 per field) of R
//     consecutive rows; lx = lane & 7 runs along k, ly = lane >> 3 along j;
//   * the +k pressure of a thread's last cell and the -k face of its first
//     cell come from the neighbouring lane (shuffle by 1), the +j pressure
//     of its last row and the -j face of its first row from the lane group
//     above/below (shuffle by 8).  Only the warp's edge lanes read them from
//     global memory (mostly L1/L2 hits): lx == 0 / 7 for k, ly == 0 / 3 for j;
//   * the x-face velocity and pressure of plane i are carried in registers
//     into plane i+1 (and, with PF, plane i+1's velocities, flags and p(i+2)
//     are loaded one plane ahead).
// A face value taken from a neighbour lane is the value that lane computed
// for its own high face with the same operations, so the result is
// bit-identical to the per-cell kernel.
//
// Needs nz % 4 == 0, 16-byte aligned fields and nx*ny*nz + 2*ny*nz < 2^31
// (32-bit cell offsets); the launcher falls back to the first column
// configuration otherwise.  The scalar form (k_step_tile1, one cell per lane,
// sf_tile1.cuh) has no such needs beyond ny*nz < 2^31.
#include <cuda_runtime.h>

#include <climits>

#include "sf_common.cuh"
#include "sf_kernels.h"
#include "sf_tile1.cuh"

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ void ld4(const float* __restrict__ base, int c, float (&v)[4]) {
    const float4 t = __ldg(reinterpret_cast<const float4*>(base + c));
    v[0] = t.x;
    v[1] = t.y;
    v[2] = t.z;
    v[3] = t.w;
}

__device__ __forceinline__ uint32_t ldflags(const uint8_t* __restrict__ base, int c) {
    return __ldg(reinterpret_cast<const unsigned int*>(base + c));
}

__device__ __forceinline__ void st4(float* __restrict__ base, int c, const float (&v)[4]) {
    __stcs(reinterpret_cast<float4*>(base + c), make_float4(v[0], v[1], v[2], v[3]));
}

// Flag bit `bit` of byte e of a packed 4-cell flag word.
template <int E>
__device__ __forceinline__ bool fbit(uint32_t f, uint32_t bit) {
    return (f & (bit << (8 * E))) != 0;
}

template <bool GEOM, int R, int W, int MINB, bool PF>
__global__ void __launch_bounds__(32 * W, MINB) k_step_tile(SfStepArgs a, SfSources src, int ich) {
    const int lane = threadIdx.x;
    const int lx = lane & 7, ly = lane >> 3;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int k0 = blockIdx.x * 32 + lx * 4;
    const int jw = (blockIdx.y * W + threadIdx.y) * (4 * R);  // the warp's first row
    const int jb = jw + ly * R;                               // this lane's first row
    // On alternate steps the chunks are dispatched from high i to low i, so a
    // step starts on the planes the previous step wrote last (still in L2).
    const int chunk = a.reverse ? (int)(gridDim.z - 1 - blockIdx.z) : (int)blockIdx.z;
    const int i0 = chunk * ich;
    const int i1 = min(i0 + ich, nx);

    if (a.trace_prev != nullptr && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0) {
        for (int t = threadIdx.y * 32 + threadIdx.x; t < a.n_probe; t += 32 * W)
            a.trace_prev[t] = a.p[a.probe_cells[t]];
    }
    if (jw >= ny) return;  // the whole warp is past the grid (no block barrier follows)

    const int plane = ny * nz;
    const bool kact = k0 < nz;
    bool ract[R];
    int roff[R];
    float dj[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        ract[r] = kact && (jb + r < ny);
        roff[r] = (jb + r) * nz + k0;
        dj[r] = ract[r] ? a.dy[jb + r] : 1.0f;
    }
    float dk[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) dk[e] = kact ? a.dz[k0 + e] : 1.0f;
    const float cv = a.cv, cp = a.cp;

    // Sources that can reach this lane's cells, in source order.
    unsigned smask = 0;
    if (kact) {
        for (int q = 0; q < src.n; ++q) {
            const sf_source& S = src.s[q];
            bool can;
            if (S.kind == 0) can = S.b >= jb && S.b < jb + R && S.c >= k0 && S.c < k0 + 4;
            else if (S.a == 0) can = true;
            else if (S.a == 1) can = S.b >= jb && S.b < jb + R;
            else can = S.b >= k0 && S.b < k0 + 4;
            if (can) smask |= 1u << q;
        }
    }

    float pc[R][4], pn[R][4], vx[R][4], vy[R][4], vz[R][4], vxm[R][4];
    uint32_t fc[R];
    float pnn[R][4], vxn[R][4], vyn[R][4], vzn[R][4];
    uint32_t fnn[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        fc[r] = fnn[r] = 0x0f0f0f0fu;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            pc[r][e] = pn[r][e] = vx[r][e] = vy[r][e] = vz[r][e] = vxm[r][e] = 0.0f;
            pnn[r][e] = vxn[r][e] = vyn[r][e] = vzn[r][e] = 0.0f;
        }
        if (!ract[r]) continue;
        const int c = i0 * plane + roff[r];
        ld4(a.p, c, pc[r]);
        if (i0 + 1 < nx) ld4(a.p, c + plane, pn[r]);
        if (PF) {
            ld4(a.vx, c, vx[r]);
            ld4(a.vy, c, vy[r]);
            ld4(a.vz, c, vz[r]);
            if (GEOM) fc[r] = ldflags(a.flags, c);
        }
        if (i0 > 0) {  // chunk start: low x face from plane i0-1
            float pm[4], vm[4];
            ld4(a.p, c - plane, pm);
            ld4(a.vx, c - plane, vm);
            const uint32_t fm = GEOM ? ldflags(a.flags, c - plane) : 0x0f0f0f0fu;
            vxm[r][0] = face_update(vm[0], cv, pc[r][0], pm[0]);
            vxm[r][1] = face_update(vm[1], cv, pc[r][1], pm[1]);
            vxm[r][2] = face_update(vm[2], cv, pc[r][2], pm[2]);
            vxm[r][3] = face_update(vm[3], cv, pc[r][3], pm[3]);
            if (GEOM) {
                if (!fbit<0>(fm, SF_OPX)) vxm[r][0] = 0.0f;
                if (!fbit<1>(fm, SF_OPX)) vxm[r][1] = 0.0f;
                if (!fbit<2>(fm, SF_OPX)) vxm[r][2] = 0.0f;
                if (!fbit<3>(fm, SF_OPX)) vxm[r][3] = 0.0f;
            }
        }
    }

    for (int i = i0; i < i1; ++i) {
        const int ci = i * plane;
        if (PF) {  // plane i+1's velocities and flags, p at i+2 (used next iteration)
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (ract[r] && i + 1 < i1) {
                    const int c = ci + plane + roff[r];
                    ld4(a.vx, c, vxn[r]);
                    ld4(a.vy, c, vyn[r]);
                    ld4(a.vz, c, vzn[r]);
                    if (GEOM) fnn[r] = ldflags(a.flags, c);
                    if (i + 2 < nx) ld4(a.p, c + plane, pnn[r]);
                }
            }
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (ract[r]) {
                    const int c = ci + roff[r];
                    ld4(a.vx, c, vx[r]);
                    ld4(a.vy, c, vy[r]);
                    ld4(a.vz, c, vz[r]);
                    if (GEOM) fc[r] = ldflags(a.flags, c);
                    if (i > i0 && i + 1 < nx) ld4(a.p, c + plane, pn[r]);
                }
            }
        }
        // edge-lane neighbours from global memory, others from the lanes
        float pup[4] = {0.0f, 0.0f, 0.0f, 0.0f};  // p at row jb+R (last row's +j)
        if (ly == 3 && ract[R - 1] && jb + R < ny) ld4(a.p, ci + roff[R - 1] + nz, pup);
        float pkp[R];  // p at k0+4 (last cell's +k), per row
        float pkm[R], vzkm[R];
        uint32_t fkm[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            pkp[r] = pkm[r] = vzkm[r] = 0.0f;
            fkm[r] = SF_ALL;
            if (lx == 7 && ract[r] && k0 + 4 < nz) pkp[r] = __ldg(a.p + ci + roff[r] + 4);
            if (lx == 0 && ract[r] && k0 > 0) {
                pkm[r] = __ldg(a.p + ci + roff[r] - 1);
                vzkm[r] = __ldg(a.vz + ci + roff[r] - 1);
                if (GEOM) fkm[r] = __ldg(a.flags + ci + roff[r] - 1);
            }
        }
        float pjm[4] = {0.0f, 0.0f, 0.0f, 0.0f}, vyjm[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        uint32_t fjm = 0x0f0f0f0fu;
        const bool jlow = (ly == 0) && ract[0] && jb > 0;
        if (jlow) {
            ld4(a.p, ci + roff[0] - nz, pjm);
            ld4(a.vy, ci + roff[0] - nz, vyjm);
            if (GEOM) fjm = ldflags(a.flags, ci + roff[0] - nz);
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float t = __shfl_down_sync(kFull, pc[0][e], 8);
            if (ly != 3) pup[e] = t;
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const float t = __shfl_down_sync(kFull, pc[r][0], 1);
            if (lx != 7) pkp[r] = t;
        }

        // high faces
        float ux[R][4], uy[R][4], uz[R][4];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const bool jhi = jb + r < ny - 1;
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                ux[r][e] = vx[r][e];
                if (i < nx - 1) ux[r][e] = face_update(vx[r][e], cv, pn[r][e], pc[r][e]);
                const float ph = (r + 1 < R) ? pc[r + 1 < R ? r + 1 : r][e] : pup[e];
                uy[r][e] = jhi ? face_update(vy[r][e], cv, ph, pc[r][e]) : vy[r][e];
                const float pk = (e < 3) ? pc[r][e < 3 ? e + 1 : e] : pkp[r];
                uz[r][e] = (k0 + e < nz - 1) ? face_update(vz[r][e], cv, pk, pc[r][e]) : vz[r][e];
            }
            if (GEOM) {
                const uint32_t f = fc[r];
                if (i < nx - 1) {
                    if (!fbit<0>(f, SF_OPX)) ux[r][0] = 0.0f;
                    if (!fbit<1>(f, SF_OPX)) ux[r][1] = 0.0f;
                    if (!fbit<2>(f, SF_OPX)) ux[r][2] = 0.0f;
                    if (!fbit<3>(f, SF_OPX)) ux[r][3] = 0.0f;
                }
                if (jhi) {
                    if (!fbit<0>(f, SF_OPY)) uy[r][0] = 0.0f;
                    if (!fbit<1>(f, SF_OPY)) uy[r][1] = 0.0f;
                    if (!fbit<2>(f, SF_OPY)) uy[r][2] = 0.0f;
                    if (!fbit<3>(f, SF_OPY)) uy[r][3] = 0.0f;
                }
                if (!fbit<0>(f, SF_OPZ) && k0 + 0 < nz - 1) uz[r][0] = 0.0f;
                if (!fbit<1>(f, SF_OPZ) && k0 + 1 < nz - 1) uz[r][1] = 0.0f;
                if (!fbit<2>(f, SF_OPZ) && k0 + 2 < nz - 1) uz[r][2] = 0.0f;
                if (!fbit<3>(f, SF_OPZ) && k0 + 3 < nz - 1) uz[r][3] = 0.0f;
            }
        }
        // low faces of the first row / first cell: neighbour lanes or global
        float uym0[4], uzm0[R];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float t = __shfl_up_sync(kFull, uy[R - 1][e], 8);
            uym0[e] = (ly != 0) ? t : 0.0f;
            if (jlow) uym0[e] = face_update(vyjm[e], cv, pc[0][e], pjm[e]);
        }
        if (GEOM && jlow) {
            if (!fbit<0>(fjm, SF_OPY)) uym0[0] = 0.0f;
            if (!fbit<1>(fjm, SF_OPY)) uym0[1] = 0.0f;
            if (!fbit<2>(fjm, SF_OPY)) uym0[2] = 0.0f;
            if (!fbit<3>(fjm, SF_OPY)) uym0[3] = 0.0f;
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const float t = __shfl_up_sync(kFull, uz[r][3], 1);
            uzm0[r] = (lx != 0) ? t : 0.0f;
            if (lx == 0 && ract[r] && k0 > 0) {
                uzm0[r] = face_update(vzkm[r], cv, pc[r][0], pkm[r]);
                if (GEOM && !(fkm[r] & SF_OPZ)) uzm0[r] = 0.0f;
            }
        }

        const float di = a.dx[i];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            float po[4], ox[4], oy[4], oz[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const bool air = !GEOM || ((fc[r] >> (8 * e)) & SF_AIR);
                const float uym = (r > 0) ? uy[r > 0 ? r - 1 : 0][e] : uym0[e];
                const float uzm = (e > 0) ? uz[r][e > 0 ? e - 1 : 0] : uzm0[r];
                float pnew = air ? f_add(pc[r][e], f_mul(cp, f_add(f_add(f_sub(ux[r][e], vxm[r][e]),
                                                                         f_sub(uy[r][e], uym)),
                                                                   f_sub(uz[r][e], uzm))))
                                 : 0.0f;
                ox[e] = f_mul(ux[r][e], di);
                oy[e] = f_mul(uy[r][e], dj[r]);
                oz[e] = f_mul(uz[r][e], dk[e]);
                pnew = f_mul(f_mul(f_mul(pnew, di), dj[r]), dk[e]);
                if (smask != 0) {
                    for (unsigned m = smask; m != 0; m &= m - 1) {
                        const int q = __ffs(m) - 1;
                        const sf_source& S = src.s[q];
                        bool hit;
                        if (S.kind == 0)
                            hit = (i == S.a) && (jb + r == S.b) && (k0 + e == S.c);
                        else if (S.a == 0)
                            hit = (i == S.b);
                        else if (S.a == 1)
                            hit = (jb + r == S.b);
                        else
                            hit = (k0 + e == S.b);
                        if (hit && air) pnew = __double2float_rn(d_add((double)pnew, a.src_val[q]));
                    }
                }
                po[e] = pnew;
            }
            if (ract[r]) {
                const int c = ci + roff[r];
                st4(a.vxo, c, ox);
                st4(a.vyo, c, oy);
                st4(a.vzo, c, oz);
                st4(a.po, c, po);
            }
        }

#pragma unroll
        for (int r = 0; r < R; ++r) {
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                vxm[r][e] = ux[r][e];
                pc[r][e] = pn[r][e];
                if (PF) {
                    pn[r][e] = pnn[r][e];
                    vx[r][e] = vxn[r][e];
                    vy[r][e] = vyn[r][e];
                    vz[r][e] = vzn[r][e];
                }
            }
            if (PF) fc[r] = fnn[r];
        }
    }
}

// Scalar warp tiles: 32 lanes along k, R rows per lane, W warps along j.
template <bool GEOM, int R, int W, int MINB, bool PF>
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
    Tile1Io io;
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
    tile1_run<GEOM, R, PF>(io, src, i0, i1, jb, k);
}

template <int R, int W, int MINB, bool PF>
int launch1(const SfStepArgs& a, const SfSources& src, bool geom, int ich, cudaStream_t st) {
    dim3 blk(32, W, 1);
    dim3 grd((a.nz + 31) / 32, (a.ny + R * W - 1) / (R * W), (a.nx + ich - 1) / ich);
    if (geom) k_step_tile1<true, R, W, MINB, PF><<<grd, blk, 0, st>>>(a, src, ich);
    else k_step_tile1<false, R, W, MINB, PF><<<grd, blk, 0, st>>>(a, src, ich);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_step_tile1 launch failed");
}

template <int R, int W, int MINB, bool PF>
int launch(const SfStepArgs& a, const SfSources& src, bool geom, int ich, cudaStream_t st) {
    dim3 blk(32, W, 1);
    const int rows = 4 * R * W;
    dim3 grd((a.nz + 31) / 32, (a.ny + rows - 1) / rows, (a.nx + ich - 1) / ich);
    if (geom) k_step_tile<true, R, W, MINB, PF><<<grd, blk, 0, st>>>(a, src, ich);
    else k_step_tile<false, R, W, MINB, PF><<<grd, blk, 0, st>>>(a, src, ich);
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
    }
    return sf_fail("k_step_tile: bad configuration");
}
