// sf_tile1.cuh -- one warp's share of a fused step, one cell per lane along k.
//
// The scalar counterpart of the float4 warp tiles in sf_step_tile.cu, for
// any nz and any alignment: the 32 lanes of a warp hold 32 consecutive k
// cells of R consecutive rows (jb .. jb+R-1) and walk planes i0 .. i1-1.
//   * +k pressure and -k face come from the neighbouring lane (shuffle by
//     1); lane 31 / lane 0 read them from global memory;
//   * +j pressure and -j face of inner rows come from the lane's own
//     registers; the first row's -j face and the last row's +j pressure are
//     read from global memory (L1/L2 hits);
//   * the x-face velocity and the pressure are carried into the next plane;
//     with PF the next plane's velocities, flags and p(i+2) are loaded before
//     the current plane's arithmetic (more bytes in flight per warp).
// Per-cell arithmetic and its order are those of k_step (sf_step.cu), so the
// result is bit-identical.  Every lane of the warp must call tile1_run with
// the same jb, i0 and i1 (the shuffles need all 32 lanes), including lanes
// whose k is past the grid.  Used by the single-grid kernel k_step_tile1 and
// the batched plain-tile kernel.
#pragma once
#include "sf_common.cuh"

struct Tile1Io {
    int nx, ny, nz;
    long long plane;
    float cv, cp;
    const float* __restrict__ p;
    const float* __restrict__ vx;
    const float* __restrict__ vy;
    const float* __restrict__ vz;
    float* __restrict__ po;
    float* __restrict__ vxo;
    float* __restrict__ vyo;
    float* __restrict__ vzo;
    const uint8_t* __restrict__ flags;
    const float* __restrict__ dx;
    const float* __restrict__ dy;
    const float* __restrict__ dz;
    const double* __restrict__ src_val;
};

template <bool GEOM, int R, bool PF = false>
__device__ __forceinline__ void tile1_run(const Tile1Io& io, const SfSources& src, int i0, int i1,
                                          int jb, int k) {
    constexpr unsigned kFull1 = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int nx = io.nx, ny = io.ny, nz = io.nz;
    const long long plane = io.plane;
    const float cv = io.cv, cp = io.cp;
    const bool kact = k < nz;
    bool ract[R];
    int roff[R];  // offset within a plane (ny * nz < 2^31)
    float dj[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        ract[r] = kact && (jb + r < ny);
        roff[r] = (jb + r) * nz + k;
        dj[r] = ract[r] ? io.dy[jb + r] : 1.0f;
    }
    const float dk = kact ? io.dz[k] : 1.0f;

    unsigned smask = 0;
    if (kact) {
        for (int q = 0; q < src.n; ++q) {
            const sf_source& S = src.s[q];
            bool can;
            if (S.kind == 0) can = S.b >= jb && S.b < jb + R && S.c == k;
            else if (S.a == 0) can = true;
            else if (S.a == 1) can = S.b >= jb && S.b < jb + R;
            else can = S.b == k;
            if (can) smask |= 1u << q;
        }
    }

    float pc[R], pn[R], vxm[R];
    float vx[R], vy[R], vz[R];  // plane i (with PF: loaded one plane ahead)
    uint8_t fc[R];
    {
        const float* P0 = io.p + (long long)i0 * plane;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            pc[r] = pn[r] = vxm[r] = 0.0f;
            vx[r] = vy[r] = vz[r] = 0.0f;
            fc[r] = SF_ALL;
            if (!ract[r]) continue;
            pc[r] = __ldg(P0 + roff[r]);
            if (i0 + 1 < nx) pn[r] = __ldg(P0 + plane + roff[r]);
            if (PF) {
                const long long c0 = (long long)i0 * plane + roff[r];
                vx[r] = __ldg(io.vx + c0);
                vy[r] = __ldg(io.vy + c0);
                vz[r] = __ldg(io.vz + c0);
                if (GEOM) fc[r] = __ldg(io.flags + c0);
            }
            if (i0 > 0) {  // chunk start: low x face from plane i0-1
                const float pm = __ldg(P0 - plane + roff[r]);
                const float vm = __ldg(io.vx + (long long)(i0 - 1) * plane + roff[r]);
                vxm[r] = face_update(vm, cv, pc[r], pm);
                if (GEOM && !(__ldg(io.flags + (long long)(i0 - 1) * plane + roff[r]) & SF_OPX))
                    vxm[r] = 0.0f;
            }
        }
    }

    for (int i = i0; i < i1; ++i) {
        const long long base = (long long)i * plane;
        const float* __restrict__ P = io.p + base;
        const float* __restrict__ VX = io.vx + base;
        const float* __restrict__ VY = io.vy + base;
        const float* __restrict__ VZ = io.vz + base;
        const uint8_t* __restrict__ F = GEOM ? io.flags + base : nullptr;
        float vxn[R], vyn[R], vzn[R], pnn[R];
        uint8_t fnn[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            vxn[r] = vyn[r] = vzn[r] = pnn[r] = 0.0f;
            fnn[r] = SF_ALL;
            if (!ract[r]) continue;
            if (PF) {  // plane i+1 for the next iteration, p at i+2
                if (i + 1 < i1) {
                    vxn[r] = __ldg(VX + plane + roff[r]);
                    vyn[r] = __ldg(VY + plane + roff[r]);
                    vzn[r] = __ldg(VZ + plane + roff[r]);
                    if (GEOM) fnn[r] = __ldg(F + plane + roff[r]);
                    if (i + 2 < nx) pnn[r] = __ldg(P + 2 * plane + roff[r]);
                }
            } else {
                vx[r] = __ldg(VX + roff[r]);
                vy[r] = __ldg(VY + roff[r]);
                vz[r] = __ldg(VZ + roff[r]);
                if (GEOM) fc[r] = __ldg(F + roff[r]);
                if (i > i0 && i + 1 < nx) pn[r] = __ldg(P + plane + roff[r]);
            }
        }
        // neighbours outside the lane's registers
        float pup = 0.0f;  // p at row jb+R
        if (ract[R - 1] && jb + R < ny) pup = __ldg(P + roff[R - 1] + nz);
        const bool jlow = ract[0] && jb > 0;
        float pjm = 0.0f, vyjm = 0.0f;
        uint8_t fjm = SF_ALL;
        if (jlow) {
            pjm = __ldg(P + roff[0] - nz);
            vyjm = __ldg(VY + roff[0] - nz);
            if (GEOM) fjm = __ldg(F + roff[0] - nz);
        }
        float pkp[R], pkm[R], vzkm[R];
        uint8_t fkm[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            pkp[r] = pkm[r] = vzkm[r] = 0.0f;
            fkm[r] = SF_ALL;
            if (lane == 31 && ract[r] && k + 1 < nz) pkp[r] = __ldg(P + roff[r] + 1);
            if (lane == 0 && ract[r] && k > 0) {
                pkm[r] = __ldg(P + roff[r] - 1);
                vzkm[r] = __ldg(VZ + roff[r] - 1);
                if (GEOM) fkm[r] = __ldg(F + roff[r] - 1);
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const float t = __shfl_down_sync(kFull1, pc[r], 1);
            if (lane != 31) pkp[r] = t;
        }

        float ux[R], uy[R], uz[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            ux[r] = vx[r];
            if (i < nx - 1) {
                ux[r] = face_update(vx[r], cv, pn[r], pc[r]);
                if (GEOM && !(fc[r] & SF_OPX)) ux[r] = 0.0f;
            }
            uy[r] = vy[r];
            if (jb + r < ny - 1) {
                uy[r] = face_update(vy[r], cv, (r + 1 < R) ? pc[r + 1 < R ? r + 1 : r] : pup, pc[r]);
                if (GEOM && !(fc[r] & SF_OPY)) uy[r] = 0.0f;
            }
            uz[r] = vz[r];
            if (k < nz - 1) {
                uz[r] = face_update(vz[r], cv, pkp[r], pc[r]);
                if (GEOM && !(fc[r] & SF_OPZ)) uz[r] = 0.0f;
            }
        }
        float uzm[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const float t = __shfl_up_sync(kFull1, uz[r], 1);
            uzm[r] = (lane != 0) ? t : 0.0f;
            if (lane == 0 && ract[r] && k > 0) {
                uzm[r] = face_update(vzkm[r], cv, pc[r], pkm[r]);
                if (GEOM && !(fkm[r] & SF_OPZ)) uzm[r] = 0.0f;
            }
        }
        float uym0 = 0.0f;
        if (jlow) {
            uym0 = face_update(vyjm, cv, pc[0], pjm);
            if (GEOM && !(fjm & SF_OPY)) uym0 = 0.0f;
        }

        const float di = io.dx[i];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const bool air = !GEOM || (fc[r] & SF_AIR);
            const float uym = (r > 0) ? uy[r > 0 ? r - 1 : 0] : uym0;
            float pnew = air ? f_add(pc[r], f_mul(cp, f_add(f_add(f_sub(ux[r], vxm[r]),
                                                                  f_sub(uy[r], uym)),
                                                            f_sub(uz[r], uzm[r]))))
                             : 0.0f;
            const float ox = f_mul(ux[r], di), oy = f_mul(uy[r], dj[r]), oz = f_mul(uz[r], dk);
            pnew = f_mul(f_mul(f_mul(pnew, di), dj[r]), dk);
            if (smask != 0) {
                for (unsigned m = smask; m != 0; m &= m - 1) {
                    const int q = __ffs(m) - 1;
                    const sf_source& S = src.s[q];
                    bool hit;
                    if (S.kind == 0) hit = (i == S.a) && (jb + r == S.b);
                    else if (S.a == 0) hit = (i == S.b);
                    else if (S.a == 1) hit = (jb + r == S.b);
                    else hit = true;
                    if (hit && air) pnew = __double2float_rn(d_add((double)pnew, io.src_val[q]));
                }
            }
            if (ract[r]) {
                const long long c = base + roff[r];
                __stcs(io.vxo + c, ox);
                __stcs(io.vyo + c, oy);
                __stcs(io.vzo + c, oz);
                __stcs(io.po + c, pnew);
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            vxm[r] = ux[r];
            pc[r] = pn[r];
            if (PF) {
                pn[r] = pnn[r];
                vx[r] = vxn[r];
                vy[r] = vyn[r];
                vz[r] = vzn[r];
                fc[r] = fnn[r];
            }
        }
    }
}
