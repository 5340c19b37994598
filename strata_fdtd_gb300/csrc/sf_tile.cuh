// sf_tile.cuh -- one warp's share of a fused step over a tile of planes.
//
// Same per-cell arithmetic as k_step (sf_step.cu), which restates the
// reference passes listed there.  A warp owns a patch of every plane
// i0 .. i1-1 of its tile and passes neighbour values between lanes instead
// of re-deriving them from global memory (the thread-column kernels of
// sf_step_col.cu spend most of their issue slots doing that):
//
// tile4_run -- 32 (k) x 4R (j) cells per warp: lane (lx, ly) holds 4
//   consecutive k cells (one float4 per field) of R consecutive rows,
//   lx = lane & 7 along k, ly = lane >> 3 along j.  The +k pressure of a
//   lane's last cell and the -k face of its first come from the neighbouring
//   lane (shuffle by 1), the +j pressure of its last row and the -j face of
//   its first row from the lane group above / below (shuffle by 8); only the
//   warp's edge lanes read them from global memory (L1/L2 hits).  Needs
//   nz % 4 == 0, 16-byte aligned fields and nx*ny*nz + 2*ny*nz < 2^31
//   (32-bit cell offsets).
// tile1_run -- 32 (k) x R (j) cells per warp, one cell per lane, for any nz
//   and alignment (ny*nz < 2^31): k neighbours by shuffles, j neighbours of
//   inner rows from the lane's own registers.
//
// Both carry the x-face velocity and the pressure in registers into the next
// plane (2.5-D register blocking); with PF the next plane's velocities, flags
// and p(i+2) are loaded before the current plane's arithmetic.  A face value
// taken from a neighbour lane is the value that lane computed for its own
// high face with the same operations, so the result is bit-identical to the
// per-cell kernel.  Every lane of a warp must call with the same tile
// (the shuffles need all 32 lanes), including lanes past the grid.  Used by
// the single-grid kernels (sf_step_tile.cu) and the batched tile loop
// (sf_batch.cu).
#pragma once
#include "sf_common.cuh"

struct SfTileIo {
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
    // nonuniform grids (NU kernels only): per-face velocity coefficients
    // float(coeff_v_base * inv_face) and per-cell inverse spacings, per axis
    const float* __restrict__ nu_cv[3];
    const float* __restrict__ nu_inv[3];
};

namespace sf_tile {

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

// Streaming (evict-first) stores, or ordinary write-back ones with WB.
template <bool WB = false>
__device__ __forceinline__ void st4(float* __restrict__ base, int c, const float (&v)[4]) {
    if (WB) *reinterpret_cast<float4*>(base + c) = make_float4(v[0], v[1], v[2], v[3]);
    else __stcs(reinterpret_cast<float4*>(base + c), make_float4(v[0], v[1], v[2], v[3]));
}

// Flag bit `bit` of byte e of a packed 4-cell flag word.
template <int E>
__device__ __forceinline__ bool fbit(uint32_t f, uint32_t bit) {
    return (f & (bit << (8 * E))) != 0;
}

}  // namespace sf_tile

// Plane addressing of the float4 warp tile: where plane i of the input and
// output fields starts, and how they are read and written.  SfPlainMem is
// the state sets themselves (plane i at i * plane, loads through the
// read-only path, streaming or write-back stores); the multi-step pipeline
// (sf_step_pipe.cu) substitutes ring buffers of planes.  The flag bytes are
// always addressed by i * plane.  before(i) runs ahead of plane i's loads
// (the planes up to i+2 may be read next) and after(i) once plane i is
// stored: hooks for the streaming pipeline's synchronisation, empty here.
struct SfPlainMem {
    int plane;
    __device__ __forceinline__ void before(int) const {}
    __device__ __forceinline__ void after(int) const {}
    __device__ __forceinline__ int in(int i) const { return i * plane; }
    __device__ __forceinline__ int out(int i) const { return i * plane; }
    __device__ __forceinline__ void ld4(const float* __restrict__ b, int c, float (&v)[4]) const {
        sf_tile::ld4(b, c, v);
    }
    __device__ __forceinline__ float ld1(const float* __restrict__ b, int c) const {
        return __ldg(b + c);
    }
    template <bool WB>
    __device__ __forceinline__ void st4(float* __restrict__ b, int c, const float (&v)[4]) const {
        sf_tile::st4<WB>(b, c, v);
    }
};

template <bool GEOM, int R, bool PF, bool NU = false, bool WB = false, class Mem = SfPlainMem>
__device__ __forceinline__ void tile4_run(const SfTileIo& io, const SfSources& src, int i0, int i1,
                                          int jw, int kw, const Mem& mem) {
    using namespace sf_tile;
    const int lane = threadIdx.x & 31;
    const int lx = lane & 7, ly = lane >> 3;
    const int nx = io.nx, ny = io.ny, nz = io.nz;
    const int k0 = kw + lx * 4;
    const int jb = jw + ly * R;  // this lane's first row
    const int plane = mem.plane;  // ny * nz
    const bool kact = k0 < nz;
    bool ract[R];
    int roff[R];
    float dj[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        ract[r] = kact && (jb + r < ny);
        roff[r] = (jb + r) * nz + k0;
        dj[r] = ract[r] ? io.dy[jb + r] : 1.0f;
    }
    float dk[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) dk[e] = kact ? io.dz[k0 + e] : 1.0f;
    const float cv = io.cv, cp = io.cp;
    // face coefficients and cell scales (uniform: cv everywhere, scale 1)
    float cvy[R], sy[R], cvz[4], sz[4], cvy_lo = cv, cvz_lo = cv;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        cvy[r] = cv;
        sy[r] = 1.0f;
        if (NU && ract[r]) {
            cvy[r] = jb + r < ny - 1 ? io.nu_cv[1][jb + r] : 0.0f;
            sy[r] = io.nu_inv[1][jb + r];
        }
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        cvz[e] = cv;
        sz[e] = 1.0f;
        if (NU && kact) {
            cvz[e] = k0 + e < nz - 1 ? io.nu_cv[2][k0 + e] : 0.0f;
            sz[e] = io.nu_inv[2][k0 + e];
        }
    }
    if (NU && kact && jb > 0) cvy_lo = io.nu_cv[1][jb - 1];
    if (NU && kact && k0 > 0) cvz_lo = io.nu_cv[2][k0 - 1];

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
    mem.before(i0);
    for (int r = 0; r < R; ++r) {
        fc[r] = fnn[r] = 0x0f0f0f0fu;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            pc[r][e] = pn[r][e] = vx[r][e] = vy[r][e] = vz[r][e] = vxm[r][e] = 0.0f;
            pnn[r][e] = vxn[r][e] = vyn[r][e] = vzn[r][e] = 0.0f;
        }
        if (!ract[r]) continue;
        const int c = mem.in(i0) + roff[r];
        const int cf = i0 * plane + roff[r];
        mem.ld4(io.p, c, pc[r]);
        if (i0 + 1 < nx) mem.ld4(io.p, mem.in(i0 + 1) + roff[r], pn[r]);
        if (PF) {
            mem.ld4(io.vx, c, vx[r]);
            mem.ld4(io.vy, c, vy[r]);
            mem.ld4(io.vz, c, vz[r]);
            if (GEOM) fc[r] = ldflags(io.flags, cf);
        }
        if (i0 > 0) {  // chunk start: low x face from plane i0-1
            float pm[4], vm[4];
            const int cm = mem.in(i0 - 1) + roff[r];
            mem.ld4(io.p, cm, pm);
            mem.ld4(io.vx, cm, vm);
            const uint32_t fm = GEOM ? ldflags(io.flags, cf - plane) : 0x0f0f0f0fu;
            const float cvm = NU ? io.nu_cv[0][i0 - 1] : cv;
            vxm[r][0] = face_update(vm[0], cvm, pc[r][0], pm[0]);
            vxm[r][1] = face_update(vm[1], cvm, pc[r][1], pm[1]);
            vxm[r][2] = face_update(vm[2], cvm, pc[r][2], pm[2]);
            vxm[r][3] = face_update(vm[3], cvm, pc[r][3], pm[3]);
            if (GEOM) {
                if (!fbit<0>(fm, SF_OPX)) vxm[r][0] = 0.0f;
                if (!fbit<1>(fm, SF_OPX)) vxm[r][1] = 0.0f;
                if (!fbit<2>(fm, SF_OPX)) vxm[r][2] = 0.0f;
                if (!fbit<3>(fm, SF_OPX)) vxm[r][3] = 0.0f;
            }
        }
    }

    for (int i = i0; i < i1; ++i) {
        mem.before(i);
        const int ci = mem.in(i);      // input fields of plane i
        const int cfi = i * plane;     // flag bytes of plane i
        const float cvx = NU ? (i < nx - 1 ? io.nu_cv[0][i] : 0.0f) : cv;
        const float sxi = NU ? io.nu_inv[0][i] : 1.0f;
        if (PF) {  // plane i+1's velocities and flags, p at i+2 (used next iteration)
            const int cn = mem.in(i + 1), cnn = mem.in(i + 2);  // read only when in the grid
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (ract[r] && i + 1 < i1) {
                    const int c = cn + roff[r];
                    mem.ld4(io.vx, c, vxn[r]);
                    mem.ld4(io.vy, c, vyn[r]);
                    mem.ld4(io.vz, c, vzn[r]);
                    if (GEOM) fnn[r] = ldflags(io.flags, cfi + plane + roff[r]);
                    if (i + 2 < nx) mem.ld4(io.p, cnn + roff[r], pnn[r]);
                }
            }
        } else {
            const int cn = mem.in(i + 1);  // read only when in the grid
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (ract[r]) {
                    const int c = ci + roff[r];
                    mem.ld4(io.vx, c, vx[r]);
                    mem.ld4(io.vy, c, vy[r]);
                    mem.ld4(io.vz, c, vz[r]);
                    if (GEOM) fc[r] = ldflags(io.flags, cfi + roff[r]);
                    if (i > i0 && i + 1 < nx) mem.ld4(io.p, cn + roff[r], pn[r]);
                }
            }
        }
        // edge-lane neighbours from global memory, others from the lanes
        float pup[4] = {0.0f, 0.0f, 0.0f, 0.0f};  // p at row jb+R (last row's +j)
        if (ly == 3 && ract[R - 1] && jb + R < ny) mem.ld4(io.p, ci + roff[R - 1] + nz, pup);
        float pkp[R];  // p at k0+4 (last cell's +k), per row
        float pkm[R], vzkm[R];
        uint32_t fkm[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            pkp[r] = pkm[r] = vzkm[r] = 0.0f;
            fkm[r] = SF_ALL;
            if (lx == 7 && ract[r] && k0 + 4 < nz) pkp[r] = mem.ld1(io.p, ci + roff[r] + 4);
            if (lx == 0 && ract[r] && k0 > 0) {
                pkm[r] = mem.ld1(io.p, ci + roff[r] - 1);
                vzkm[r] = mem.ld1(io.vz, ci + roff[r] - 1);
                if (GEOM) fkm[r] = __ldg(io.flags + cfi + roff[r] - 1);
            }
        }
        float pjm[4] = {0.0f, 0.0f, 0.0f, 0.0f}, vyjm[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        uint32_t fjm = 0x0f0f0f0fu;
        const bool jlow = (ly == 0) && ract[0] && jb > 0;
        if (jlow) {
            mem.ld4(io.p, ci + roff[0] - nz, pjm);
            mem.ld4(io.vy, ci + roff[0] - nz, vyjm);
            if (GEOM) fjm = ldflags(io.flags, cfi + roff[0] - nz);
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
                if (i < nx - 1) ux[r][e] = face_update(vx[r][e], cvx, pn[r][e], pc[r][e]);
                const float ph = (r + 1 < R) ? pc[r + 1 < R ? r + 1 : r][e] : pup[e];
                uy[r][e] = jhi ? face_update(vy[r][e], cvy[r], ph, pc[r][e]) : vy[r][e];
                const float pk = (e < 3) ? pc[r][e < 3 ? e + 1 : e] : pkp[r];
                uz[r][e] = (k0 + e < nz - 1) ? face_update(vz[r][e], cvz[e], pk, pc[r][e]) : vz[r][e];
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
            if (jlow) uym0[e] = face_update(vyjm[e], cvy_lo, pc[0][e], pjm[e]);
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
                uzm0[r] = face_update(vzkm[r], cvz_lo, pc[r][0], pkm[r]);
                if (GEOM && !(fkm[r] & SF_OPZ)) uzm0[r] = 0.0f;
            }
        }

        const float di = io.dx[i];
        const int co = mem.out(i);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            float po[4], ox[4], oy[4], oz[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const bool air = !GEOM || ((fc[r] >> (8 * e)) & SF_AIR);
                const float uym = (r > 0) ? uy[r > 0 ? r - 1 : 0][e] : uym0[e];
                const float uzm = (e > 0) ? uz[r][e > 0 ? e - 1 : 0] : uzm0[r];
                float dx_ = f_sub(ux[r][e], vxm[r][e]), dy_ = f_sub(uy[r][e], uym),
                      dz_ = f_sub(uz[r][e], uzm);
                if (NU) {  // update_pressure_nonuniform: each term scaled first
                    dx_ = f_mul(sxi, dx_);
                    dy_ = f_mul(sy[r], dy_);
                    dz_ = f_mul(sz[e], dz_);
                }
                float pnew = air ? f_add(pc[r][e], f_mul(cp, f_add(f_add(dx_, dy_), dz_))) : 0.0f;
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
                        if (hit && air) pnew = __double2float_rn(d_add((double)pnew, io.src_val[q]));
                    }
                }
                po[e] = pnew;
            }
            if (ract[r]) {
                const int c = co + roff[r];
                mem.template st4<WB>(io.vxo, c, ox);
                mem.template st4<WB>(io.vyo, c, oy);
                mem.template st4<WB>(io.vzo, c, oz);
                mem.template st4<WB>(io.po, c, po);
            }
        }
        mem.after(i);

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

template <bool GEOM, int R, bool PF = false, bool NU = false>
__device__ __forceinline__ void tile1_run(const SfTileIo& io, const SfSources& src, int i0, int i1,
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
    // face coefficients and cell scales (uniform: cv everywhere, scale 1)
    float cvy[R], sy[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        cvy[r] = cv;
        sy[r] = 1.0f;
        if (NU && ract[r]) {
            cvy[r] = jb + r < ny - 1 ? io.nu_cv[1][jb + r] : 0.0f;
            sy[r] = io.nu_inv[1][jb + r];
        }
    }
    const float cvz = NU ? (kact && k < nz - 1 ? io.nu_cv[2][k] : 0.0f) : cv;
    const float sz = NU ? (kact ? io.nu_inv[2][k] : 1.0f) : 1.0f;
    const float cvy_lo = NU && kact && jb > 0 ? io.nu_cv[1][jb - 1] : cv;
    const float cvz_lo = NU && kact && k > 0 ? io.nu_cv[2][k - 1] : cv;

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
                vxm[r] = face_update(vm, NU ? io.nu_cv[0][i0 - 1] : cv, pc[r], pm);
                if (GEOM && !(__ldg(io.flags + (long long)(i0 - 1) * plane + roff[r]) & SF_OPX))
                    vxm[r] = 0.0f;
            }
        }
    }

    for (int i = i0; i < i1; ++i) {
        const long long base = (long long)i * plane;
        const float cvx = NU ? (i < nx - 1 ? io.nu_cv[0][i] : 0.0f) : cv;
        const float sxi = NU ? io.nu_inv[0][i] : 1.0f;
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
                ux[r] = face_update(vx[r], cvx, pn[r], pc[r]);
                if (GEOM && !(fc[r] & SF_OPX)) ux[r] = 0.0f;
            }
            uy[r] = vy[r];
            if (jb + r < ny - 1) {
                uy[r] = face_update(vy[r], cvy[r], (r + 1 < R) ? pc[r + 1 < R ? r + 1 : r] : pup,
                                    pc[r]);
                if (GEOM && !(fc[r] & SF_OPY)) uy[r] = 0.0f;
            }
            uz[r] = vz[r];
            if (k < nz - 1) {
                uz[r] = face_update(vz[r], cvz, pkp[r], pc[r]);
                if (GEOM && !(fc[r] & SF_OPZ)) uz[r] = 0.0f;
            }
        }
        float uzm[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const float t = __shfl_up_sync(kFull1, uz[r], 1);
            uzm[r] = (lane != 0) ? t : 0.0f;
            if (lane == 0 && ract[r] && k > 0) {
                uzm[r] = face_update(vzkm[r], cvz_lo, pc[r], pkm[r]);
                if (GEOM && !(fkm[r] & SF_OPZ)) uzm[r] = 0.0f;
            }
        }
        float uym0 = 0.0f;
        if (jlow) {
            uym0 = face_update(vyjm, cvy_lo, pc[0], pjm);
            if (GEOM && !(fjm & SF_OPY)) uym0 = 0.0f;
        }

        const float di = io.dx[i];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const bool air = !GEOM || (fc[r] & SF_AIR);
            const float uym = (r > 0) ? uy[r > 0 ? r - 1 : 0] : uym0;
            float dx_ = f_sub(ux[r], vxm[r]), dy_ = f_sub(uy[r], uym), dz_ = f_sub(uz[r], uzm[r]);
            if (NU) {  // update_pressure_nonuniform: each term scaled first
                dx_ = f_mul(sxi, dx_);
                dy_ = f_mul(sy[r], dy_);
                dz_ = f_mul(sz, dz_);
            }
            float pnew = air ? f_add(pc[r], f_mul(cp, f_add(f_add(dx_, dy_), dz_))) : 0.0f;
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
