// sf_tb.cuh -- one warp's share of a two-step pass (temporal blocking with
// overlapped warp tiles).
//
// A warp owns a window of 32 k cells (one per lane, k = W0 + lane) and
// R + 4 rows j = jw - 2 .. jw + R + 1 (register arrays indexed by row), and
// marches planes along i.  At plane iteration t it computes the first step
// ("level 1") of plane t and the second ("level 2") of plane t-1:
//
//   level-1 faces  x and z on rows jw-1 .. jw+R, y on rows jw-2 .. jw+R
//   level-1 p      rows jw-1 .. jw+R, lanes 1 .. 30
//   level-2 faces  x and z on rows jw .. jw+R-1, y on rows jw-1 .. jw+R-1
//   level-2 p      rows jw .. jw+R-1, lanes 2 .. 29: the output (28 x R
//                  cells per plane), stored to the output set
//
// The k neighbours come from the adjacent lanes by shuffles, the j
// neighbours from the lane's own rows, the x neighbours from the previous
// iteration (carried in registers).  Cells outside the output region are
// recomputed by the neighbouring warps with the same operations, so the
// values they feed into this warp's output equal the neighbours' bit for
// bit, and no warp ever waits for another.  HBM sees one read of the input
// state (plus the halo rows and lanes, mostly L1/L2 hits) and one write of
// the output state per two steps.
//
// The per-cell operations are those of tile4_run / tile1_run (sf_tile.cuh),
// in the same order: FP32 without contraction, faces zeroed by the flag
// bits, PML on p as three rounded products, sources in FP64 rounded once in
// source order on air cells.  Uniform grids only.
#pragma once
#include "sf_common.cuh"

namespace sf_tb {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float pressure(float pc, float cp, float uxh, float uxl, float uyh,
                                          float uyl, float uzh, float uzl, bool air, float di,
                                          float dj, float dk) {
    const float dx_ = f_sub(uxh, uxl), dy_ = f_sub(uyh, uyl), dz_ = f_sub(uzh, uzl);
    const float pn = air ? f_add(pc, f_mul(cp, f_add(f_add(dx_, dy_), dz_))) : 0.0f;
    return f_mul(f_mul(f_mul(pn, di), dj), dk);
}

__device__ __forceinline__ float inject(float pn, const SfSources& src, unsigned smask,
                                       const double* val, int i, int j, int k, bool air) {
    for (unsigned m = smask; m != 0; m &= m - 1) {
        const int q = __ffs(m) - 1;
        const sf_source& S = src.s[q];
        bool hit;
        if (S.kind == 0) hit = (i == S.a) && (j == S.b) && (k == S.c);
        else if (S.a == 0) hit = (i == S.b);
        else if (S.a == 1) hit = (j == S.b);
        else hit = (k == S.b);
        if (hit && air) pn = __double2float_rn(d_add((double)pn, val[q]));
    }
    return pn;
}

}  // namespace sf_tb

// What one warp of a two-step pass reads and writes.
struct SfTbIo {
    int nx, ny, nz;
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
    const double* __restrict__ val1;  // waveform values of the first step (or null)
    const double* __restrict__ val2;  // of the second step
    int n_probe;                      // <= 32
    const long long* __restrict__ probe_cells;
    float* __restrict__ trace1;  // probe row of the state after the first step, or null
};

// Whether the warp's whole window (rows jw-2 .. jw+R+1, k = W0 .. W0+31)
// lies inside the grid and away from its high faces, so that no cell needs
// the grid-edge rules (the EDGE = false instantiation leaves them out).
__device__ __forceinline__ bool tb2_interior(const SfTbIo& io, int R, int jw, int W0) {
    return jw - 2 >= 0 && jw + R + 1 < io.ny - 1 && W0 >= 0 && W0 + 31 < io.nz - 1;
}

// Output planes i0 .. i1-1, output rows jw .. jw+R-1 (clipped to the grid),
// window k = W0 .. W0+31 (output lanes 2 .. 29).  Every lane of the warp
// must call with the same arguments.  EDGE = false only for windows that
// tb2_interior accepts.
template <bool GEOM, int R, bool EDGE>
__device__ __forceinline__ void tb2_warp_run(const SfTbIo& io, const SfSources& src, int i0,
                                             int i1, int jw, int W0) {
    using namespace sf_tb;
    constexpr int NR = R + 4;  // rows jw-2 .. jw+R+1
    const int lane = threadIdx.x & 31;
    const int nx = io.nx, ny = io.ny, nz = io.nz;
    const int plane = ny * nz;
    const int k = W0 + lane;
    const bool kin = k >= 0 && k < nz;
    const float cv = io.cv, cp = io.cp;
    const float dk = kin ? io.dz[k] : 1.0f;
    bool rin[NR];   // row in the grid and k in the grid
    int roff[NR];   // in-plane offset of the lane's cell in each row
    float dj[NR];
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        const int j = jw - 2 + r;
        rin[r] = !EDGE || (kin && j >= 0 && j < ny);
        roff[r] = rin[r] ? j * nz + k : 0;
        dj[r] = rin[r] ? io.dy[j] : 1.0f;
    }
    // sources that can reach the warp's cells, planes i0-1 .. i1
    unsigned smask = 0;
    for (int q = 0; q < src.n; ++q) {
        const sf_source& S = src.s[q];
        bool can;
        if (S.kind == 0)
            can = S.a >= i0 - 1 && S.a <= i1 && S.b >= jw - 2 && S.b < jw + R + 2 && S.c >= W0 &&
                  S.c < W0 + 32;
        else if (S.a == 0) can = S.b >= i0 - 1 && S.b <= i1;
        else if (S.a == 1) can = S.b >= jw - 2 && S.b < jw + R + 2;
        else can = S.b >= W0 && S.b < W0 + 32;
        if (can) smask |= 1u << q;
    }
    // probes whose cell is one of this warp's outputs: lane q holds probe q
    int pq_i = -1, pq_j = 0, pq_k = 0;
    if (io.trace1 != nullptr && lane < io.n_probe) {
        const long long cell = io.probe_cells[lane];
        const int pi = (int)(cell / plane);
        const int rem = (int)(cell - (long long)pi * plane);
        pq_j = rem / nz;
        pq_k = rem - pq_j * nz;
        if (pi >= i0 && pi < i1 && pq_j >= jw && pq_j < jw + R && pq_k >= W0 + 2 && pq_k < W0 + 30)
            pq_i = pi;
    }
    const unsigned pmask = __ballot_sync(kFull, pq_i >= 0);

    auto ld = [&](const float* __restrict__ f, long long base, int r) -> float {
        return (!EDGE || rin[r]) ? __ldg(f + base + roff[r]) : 0.0f;
    };
    auto ldf = [&](long long base, int r) -> uint32_t {
        return (GEOM && (!EDGE || rin[r])) ? (uint32_t)__ldg(io.flags + base + roff[r])
                                           : (uint32_t)SF_ALL;
    };
    // the grid-edge rules: a face on the last plane of an axis is not
    // updated, cells outside the grid hold zeros
    auto jface = [&](int r) { return !EDGE || jw - 2 + r < ny - 1; };
    const bool kface = !EDGE || k < nz - 1;
    auto keep = [&](int r, float v) { return (!EDGE || rin[r]) ? v : 0.0f; };

    const int tstart = i0 > 0 ? i0 - 1 : 0;
    // carried: level-1 x faces and p of the previous plane (rows 1..R+2), its
    // y faces (rows 1..R+1) and z faces (rows 2..R+1), flags (rows 1..R+1);
    // the level-2 x face of the plane before (rows 2..R+1); p0 of the next
    // plane (rows 1..R+2)
    float u1xm[NR], p1m[NR], u1ym[NR], u1zm[NR], u2xm[NR], p0n[NR];
    uint32_t flm[NR];
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        u1xm[r] = p1m[r] = u1ym[r] = u1zm[r] = u2xm[r] = p0n[r] = 0.0f;
        flm[r] = SF_ALL;
    }
    {
        const long long b = (long long)tstart * plane;
#pragma unroll
        for (int r = 1; r <= R + 2; ++r) p0n[r] = ld(io.p, b, r);
        if (tstart > 0) {  // level-1 x face below the first plane
            const long long bm = b - plane;
#pragma unroll
            for (int r = 1; r <= R + 2; ++r) {
                float u = face_update(ld(io.vx, bm, r), cv, p0n[r], ld(io.p, bm, r));
                if (GEOM && !(ldf(bm, r) & SF_OPX)) u = 0.0f;
                u1xm[r] = keep(r, u);
            }
        }
    }

    // the level-0 state of the next plane, loaded one iteration ahead
    float nVX[NR], nVY[NR], nVZ[NR], nE0, nE3;
    uint32_t nFL[NR];
    auto prefetch = [&](int tp) {
        const long long bp = (long long)tp * plane;
#pragma unroll
        for (int r = 0; r <= R + 2; ++r) {
            nVY[r] = ld(io.vy, bp, r);
            nFL[r] = ldf(bp, r);
            if (r >= 1) {
                nVX[r] = ld(io.vx, bp, r);
                nVZ[r] = ld(io.vz, bp, r);
            }
        }
        nE0 = ld(io.p, bp, 0);
        nE3 = ld(io.p, bp, R + 3);
    };
    if (tstart < nx) prefetch(tstart);

    for (int t = tstart; t <= i1; ++t) {
        const bool l1 = t < nx;
        const bool l2 = t >= tstart + 1;
        const bool out = t - 1 >= i0;
        const long long b = (long long)t * plane;
        // level 0 of plane t
        float P0[NR], VX[NR], VY[NR], VZ[NR];
        uint32_t FL[NR];
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            P0[r] = p0n[r];
            VX[r] = nVX[r];
            VY[r] = nVY[r];
            VZ[r] = nVZ[r];
            FL[r] = nFL[r];
        }
        P0[0] = nE0;
        P0[R + 3] = nE3;
        float p1[NR], u1x[NR], u1y[NR], u1z[NR];
#pragma unroll
        for (int r = 0; r < NR; ++r) p1[r] = u1x[r] = u1y[r] = u1z[r] = 0.0f;
        if (l1) {
            // p0 of plane t+1 (rows 1..R+2): the x faces now, carried on;
            // then the rest of plane t+1 for the next iteration
            if (t + 1 < nx) {
#pragma unroll
                for (int r = 1; r <= R + 2; ++r) p0n[r] = ld(io.p, b + plane, r);
                if (t + 1 <= i1) prefetch(t + 1);
            }
            // level-1 faces
#pragma unroll
            for (int r = 0; r <= R + 2; ++r) {
                float uy = VY[r];
                if (jface(r)) {
                    uy = face_update(uy, cv, P0[r + 1], P0[r]);
                    if (GEOM && !(FL[r] & SF_OPY)) uy = 0.0f;
                }
                u1y[r] = keep(r, uy);
                if (r >= 1) {
                    float ux = VX[r];
                    if (t < nx - 1) {
                        ux = face_update(ux, cv, p0n[r], P0[r]);
                        if (GEOM && !(FL[r] & SF_OPX)) ux = 0.0f;
                    }
                    u1x[r] = keep(r, ux);
                    const float pk = __shfl_down_sync(kFull, P0[r], 1);
                    float uz = VZ[r];
                    if (kface) {
                        uz = face_update(uz, cv, pk, P0[r]);
                        if (GEOM && !(FL[r] & SF_OPZ)) uz = 0.0f;
                    }
                    u1z[r] = keep(r, uz);
                }
            }
            // level-1 pressure
            const float di = io.dx[t];
#pragma unroll
            for (int r = 1; r <= R + 2; ++r) {
                const float uzl = __shfl_up_sync(kFull, u1z[r], 1);
                const bool air = !GEOM || (FL[r] & SF_AIR);
                float pn = pressure(P0[r], cp, u1x[r], u1xm[r], u1y[r], u1y[r - 1], u1z[r], uzl,
                                    air, di, dj[r], dk);
                if (smask) pn = inject(pn, src, smask, io.val1, t, jw - 2 + r, k, air);
                p1[r] = keep(r, pn);
            }
            // level-1 probe samples (owner lanes)
            for (unsigned m = pmask; m != 0; m &= m - 1) {
                const int q = __ffs(m) - 1;
                const int qi = __shfl_sync(kFull, pq_i, q);
                const int qj = __shfl_sync(kFull, pq_j, q);
                const int qk = __shfl_sync(kFull, pq_k, q);
                if (qi == t && qk == k) {
                    float v = 0.0f;
#pragma unroll
                    for (int r = 2; r <= R + 1; ++r)
                        if (qj == jw - 2 + r) v = p1[r];
                    io.trace1[q] = v;
                }
            }
        }
        // level 2 of plane t-1
        if (l2) {
            const float dxm = io.dx[t - 1];
            float u2y[NR];
#pragma unroll
            for (int r = 1; r <= R + 1; ++r) {
                float uy = f_mul(u1ym[r], dj[r]);
                if (jface(r)) {
                    uy = face_update(uy, cv, p1m[r + 1], p1m[r]);
                    if (GEOM && !(flm[r] & SF_OPY)) uy = 0.0f;
                }
                u2y[r] = keep(r, uy);
            }
            const long long bo = (long long)(t - 1) * plane;
            const bool lout = out && lane >= 2 && lane < 30;
#pragma unroll
            for (int r = 2; r <= R + 1; ++r) {
                float ux = f_mul(u1xm[r], dxm);
                if (t - 1 < nx - 1) {
                    ux = face_update(ux, cv, p1[r], p1m[r]);
                    if (GEOM && !(flm[r] & SF_OPX)) ux = 0.0f;
                }
                ux = keep(r, ux);
                const float pk = __shfl_down_sync(kFull, p1m[r], 1);
                float uz = f_mul(u1zm[r], dk);
                if (kface) {
                    uz = face_update(uz, cv, pk, p1m[r]);
                    if (GEOM && !(flm[r] & SF_OPZ)) uz = 0.0f;
                }
                uz = keep(r, uz);
                const float uzl = __shfl_up_sync(kFull, uz, 1);
                const bool air = !GEOM || (flm[r] & SF_AIR);
                float pn = pressure(p1m[r], cp, ux, u2xm[r], u2y[r], u2y[r - 1], uz, uzl, air, dxm,
                                    dj[r], dk);
                if (smask) pn = inject(pn, src, smask, io.val2, t - 1, jw - 2 + r, k, air);
                if (lout && (!EDGE || rin[r])) {
                    const long long c = bo + roff[r];
                    __stcs(io.po + c, pn);
                    __stcs(io.vxo + c, f_mul(ux, dxm));
                    __stcs(io.vyo + c, f_mul(u2y[r], dj[r]));
                    __stcs(io.vzo + c, f_mul(uz, dk));
                }
                u2xm[r] = ux;
            }
        }
        // plane t's level-1 state becomes the previous plane's
#pragma unroll
        for (int r = 1; r <= R + 2; ++r) {
            u1xm[r] = u1x[r];
            p1m[r] = p1[r];
            if (r <= R + 1) {
                u1ym[r] = u1y[r];
                flm[r] = FL[r];
            }
            if (r >= 2 && r <= R + 1) u1zm[r] = u1z[r];
        }
    }
}
