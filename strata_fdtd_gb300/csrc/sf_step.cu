// sf_step.cu -- fused per-step kernels for the strata-fdtd time-step path.
//
// One launch advances one grid by one time step and does, per cell, the
// work of the reference's separate whole-grid passes (paths relative to
// src/strata_fdtd/ of rjwalters/strata-fdtd):
//   update_velocity          _kernels/src/fdtd_step.cpp:15-82
//   apply_rigid_boundaries   _kernels/src/boundaries.cpp:66-89
//   update_pressure          _kernels/src/fdtd_step.cpp:84-212
//   apply_pml_velocity       _kernels/src/pml.cpp:47-98
//   apply_pml_pressure       _kernels/src/pml.cpp:100-149
//   source injection         core/solver.py:2386-2433
//   probe sampling           core/solver.py:2435-2439
// and, with ADE materials, the pole recursions and corrections of
// _kernels/src/ade.cpp:25-580 in the order of core/solver.py:2135-2193.
// NU: a nonuniform grid (update_velocity_nonuniform / update_pressure_
// nonuniform, fdtd_step.cpp:235-456, and for ADE modulus poles
// compute_divergence_nonuniform, ade.cpp:582-694, in the order of
// core/solver.py:2195-2283; the density and pressure corrections keep the
// minimum spacing, as the reference passes them).
//
// The reference updates the fields in place, pass after pass.  A single pass
// cannot: the new pressure of a cell needs the new face velocities of its
// lower neighbours, which another block may be rewriting.  So the state is
// double-buffered (read set A, write set B, swap): the same 32 bytes of
// HBM traffic per cell as an in-place fused pass, and every neighbour value
// a thread reads is the old one.  Lower-neighbour face velocities are
// recomputed from old values, bit-identical to what that neighbour computes.
//
// Arithmetic is FP32 with every rounding where the reference rounds (no
// fused multiply-add): v + cv*(p1-p0); p + cp*((dvx+dvy)+dvz); PML on p as
// ((p*dx)*dy)*dz; the source added in FP64 and rounded once.
#include <cuda_runtime.h>

#include "sf_common.cuh"

namespace {

constexpr int BX = 32;  // threads along k (contiguous)
constexpr int BY = 8;   // threads along j

// Density-pole velocity correction on the face between cells lo and hi
// (ade.cpp:228-401): v += corr*(J[hi]-J[lo]) for each density pole whose
// material holds both cells, Debye poles first then Lorentz.
__device__ __forceinline__ float ade_face(float v, const SfPoles& P, uint8_t m_lo, uint8_t m_hi,
                                          long long lo, long long hi) {
    if (m_lo == 0 || m_lo != m_hi) return v;
#pragma unroll 1
    for (int q = 0; q < P.n; ++q) {
        const sf_pole& pl = P.p[q];
        if (pl.target == 0 && pl.material_id == m_lo)
            v = f_add(v, f_mul(pl.corr, f_sub(pl.J[hi], pl.J[lo])));
    }
    return v;
}

template <bool GEOM, bool ADE, bool NU>
__global__ void __launch_bounds__(BX* BY) k_step(SfStepArgs a, SfSources src, SfPoles poles) {
    const int k = a.reg_lo[2] + blockIdx.x * BX + threadIdx.x;
    const int j = a.reg_lo[1] + blockIdx.y * BY + threadIdx.y;
    const int i = a.reg_lo[0] + blockIdx.z;

    // Probe values of the input state are the previous step's samples.
    if (a.trace_prev != nullptr && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0) {
        for (int t = threadIdx.y * BX + threadIdx.x; t < a.n_probe; t += BX * BY)
            a.trace_prev[t] = a.p[a.probe_cells[t]];
    }
    if (k >= a.reg_hi[2] || j >= a.reg_hi[1]) return;

    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const long long plane = a.plane;
    const long long c = (long long)i * plane + (long long)j * nz + k;
    const float cv = a.cv;
    const float pc = a.p[c];
    const uint8_t fc = GEOM ? a.flags[c] : (uint8_t)SF_ALL;
    uint8_t mc = 0;
    if (ADE) mc = a.mat[c];

    // Faces on the high side of this cell.  The last plane of each axis
    // carries no update (fdtd_step.cpp:34,54,77 loop bounds).
    // face coefficients: cv, or per face float(coeff_v_base * inv_face)
    const float cvx = NU ? a.nu_cv[0][i] : cv, cvy = NU ? a.nu_cv[1][j] : cv,
                cvz = NU ? a.nu_cv[2][k] : cv;
    float vxn = a.vx[c], vyn = a.vy[c], vzn = a.vz[c];
    if (i < nx - 1) {
        vxn = face_update(vxn, cvx, a.p[c + plane], pc);
        if (ADE) vxn = ade_face(vxn, poles, mc, a.mat[c + plane], c, c + plane);
        if (GEOM && !(fc & SF_OPX)) vxn = 0.0f;
    }
    if (j < ny - 1) {
        vyn = face_update(vyn, cvy, a.p[c + nz], pc);
        if (ADE) vyn = ade_face(vyn, poles, mc, a.mat[c + nz], c, c + nz);
        if (GEOM && !(fc & SF_OPY)) vyn = 0.0f;
    }
    if (k < nz - 1) {
        vzn = face_update(vzn, cvz, a.p[c + 1], pc);
        if (ADE) vzn = ade_face(vzn, poles, mc, a.mat[c + 1], c, c + 1);
        if (GEOM && !(fc & SF_OPZ)) vzn = 0.0f;
    }

    // Faces on the low side, recomputed from the old state exactly as the
    // neighbour computes them; the domain's low boundary face is zero.
    float vxm = 0.0f, vym = 0.0f, vzm = 0.0f;
    if (i > 0) {
        const long long m = c - plane;
        float t = face_update(a.vx[m], NU ? a.nu_cv[0][i - 1] : cv, pc, a.p[m]);
        if (ADE) t = ade_face(t, poles, a.mat[m], mc, m, c);
        if (GEOM && !(a.flags[m] & SF_OPX)) t = 0.0f;
        vxm = t;
    }
    if (j > 0) {
        const long long m = c - nz;
        float t = face_update(a.vy[m], NU ? a.nu_cv[1][j - 1] : cv, pc, a.p[m]);
        if (ADE) t = ade_face(t, poles, a.mat[m], mc, m, c);
        if (GEOM && !(a.flags[m] & SF_OPY)) t = 0.0f;
        vym = t;
    }
    if (k > 0) {
        const long long m = c - 1;
        float t = face_update(a.vz[m], NU ? a.nu_cv[2][k - 1] : cv, pc, a.p[m]);
        if (ADE) t = ade_face(t, poles, a.mat[m], mc, m, c);
        if (GEOM && !(a.flags[m] & SF_OPZ)) t = 0.0f;
        vzm = t;
    }

    const bool air = (fc & SF_AIR) != 0;
    const float ddx = f_sub(vxn, vxm), ddy = f_sub(vyn, vym), ddz = f_sub(vzn, vzm);
    // cell scales: 1, or the cell's inverse spacing per axis
    const float sx = NU ? a.nu_inv[0][i] : 1.0f, sy = NU ? a.nu_inv[1][j] : 1.0f,
                sz = NU ? a.nu_inv[2][k] : 1.0f;
    float pn;
    if (NU)  // update_pressure_nonuniform: each term scaled first
        pn = air ? f_add(pc, f_mul(a.cp, f_add(f_add(f_mul(sx, ddx), f_mul(sy, ddy)),
                                                f_mul(sz, ddz))))
                 : 0.0f;
    else
        pn = air ? f_add(pc, f_mul(a.cp, f_add(f_add(ddx, ddy), ddz))) : 0.0f;

    if (ADE && mc != 0 && poles.n_modulus > 0) {
        // compute_divergence (ade.cpp:479-580; nonuniform :582-694): each
        // difference scaled before the add
        const float s0 = NU ? sx : poles.inv_dx, s1 = NU ? sy : poles.inv_dx,
                    s2 = NU ? sz : poles.inv_dx;
        const float div = f_add(f_add(f_mul(ddx, s0), f_mul(ddy, s1)), f_mul(ddz, s2));
#pragma unroll 1
        for (int q = 0; q < poles.n; ++q) {
            const sf_pole& pl = poles.p[q];
            if (pl.target != 1 || pl.material_id != mc) continue;
            const float j0 = pl.J[c];
            float jn;
            if (pl.kind == 0) {  // ade.cpp:70-116
                jn = f_add(f_mul(pl.c0, j0), f_mul(pl.c1, div));
            } else {  // ade.cpp:172-226
                const float jp = pl.J_prev[c];
                jn = f_add(f_add(f_mul(pl.c0, j0), f_mul(pl.c1, jp)), f_mul(pl.c2, div));
                pl.J_prev[c] = j0;
            }
            pl.J[c] = jn;
            pn = f_add(pn, f_mul(pl.corr, jn));  // ade.cpp:403-477
        }
        if (!air) pn = 0.0f;  // core/solver.py:2193
    }

    // PML: velocities decay after the pressure used them (pml.cpp:47-98);
    // pressure decays axis by axis (pml.cpp:100-149).
    const float di = a.dx[i], dj = a.dy[j], dk = a.dz[k];
    a.vxo[c] = f_mul(vxn, di);
    a.vyo[c] = f_mul(vyn, dj);
    a.vzo[c] = f_mul(vzn, dk);
    pn = f_mul(f_mul(f_mul(pn, di), dj), dk);

    // Sources, in order, into air cells: p = float(double(p) + value).
#pragma unroll 1
    for (int q = 0; q < src.n; ++q) {
        const sf_source& S = src.s[q];
        bool hit;
        if (S.kind == 0)
            hit = (i == S.a) && (j == S.b) && (k == S.c);
        else
            hit = (S.a == 0) ? (i == S.b) : ((S.a == 1) ? (j == S.b) : (k == S.b));
        if (hit && air) pn = __double2float_rn(d_add((double)pn, a.src_val[q]));
    }
    a.po[c] = pn;
}

// Density-pole recursions from the old pressure, before the step kernel
// reads the updated J (ade.cpp:25-68 Debye, 118-170 Lorentz).
// Walks only the box that holds every material cell.
__global__ void k_ade_density(SfStepArgs a, SfPoles poles, long long n) {
    const int ey = a.ade_hi[1] - a.ade_lo[1], ez = a.ade_hi[2] - a.ade_lo[2];
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = a.ade_lo[0] + (int)(t / ((long long)ey * ez));
        const int r = (int)(t % ((long long)ey * ez));
        const long long c = (long long)i * a.plane + (long long)(a.ade_lo[1] + r / ez) * a.nz +
                            (a.ade_lo[2] + r % ez);
        const uint8_t mc = a.mat[c];
        if (mc == 0) continue;
        const float pc = a.p[c];
        for (int q = 0; q < poles.n; ++q) {
            const sf_pole& pl = poles.p[q];
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

__global__ void k_probe_gather(const float* __restrict__ p, const long long* __restrict__ cells,
                               int n, float* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = p[cells[t]];
}

// Microphone rows: trilinear sum over 8 corners in float, from 0, of one
// field (field[m]: 0 p, 1 vx, 2 vy, 3 vz; null = all p).  Corner order and
// the float sum are those of record_microphones_batch (microphones.cpp:82-118)
// and of Microphone.record / _interpolate_velocity (core/solver.py:1004-1118),
// whose float32 products and sums are the same operations.
__global__ void k_mic_gather(const float* __restrict__ p, const float* __restrict__ vx,
                             const float* __restrict__ vy, const float* __restrict__ vz,
                             const int* __restrict__ field, const long long* __restrict__ idx,
                             const float* __restrict__ w, int n, float* __restrict__ out) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    const int f = field ? field[m] : 0;
    const float* __restrict__ src = f == 1 ? vx : (f == 2 ? vy : (f == 3 ? vz : p));
    float s = 0.0f;
#pragma unroll
    for (int q = 0; q < 8; ++q) s = f_add(s, f_mul(w[8 * m + q], src[idx[8 * m + q]]));
    out[m] = s;
}

// One pressure-plane boundary operation over the plane perpendicular to
// op.axis; thread t = (u, v), the plane's two in-plane indices in C order.
// Mur (kind 0): low end then high end, each p_b = float(double(prev) +
// coeff * double(p_i - p_b)) and prev = p_i -- NumPy's float64 coefficient
// times the float32 difference, rounded once into p (_boundaries.py:479-513).
// Radiation impedance (kind 1), one end: p_b = float(double(float(R) p_i) +
// (1 - R) (double(prev) + coeff double(p_i - p_b))), prev = p_i
// (_boundaries.py:707-770).
__global__ void k_plane_bc(float* __restrict__ p, float* __restrict__ prev_lo,
                           float* __restrict__ prev_hi, int kind, int axis, int side,
                           double coeff, double R, int nx, int ny, int nz) {
    const int n3[3] = {nx, ny, nz};
    const int nu = axis == 0 ? ny : nx, nv = axis == 2 ? ny : nz;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nu * nv) return;
    const int u = (int)(t / nv), v = (int)(t % nv);
    const int n = n3[axis];
    auto at = [&](int w) -> long long {  // cell at position w along the axis
        if (axis == 0) return ((long long)w * ny + u) * nz + v;
        if (axis == 1) return ((long long)u * ny + w) * nz + v;
        return ((long long)u * ny + v) * nz + w;
    };
    if (kind == 0) {
        const long long b0 = at(0), i0 = at(1);
        p[b0] = __double2float_rn(d_add((double)prev_lo[t], d_mul(coeff, (double)f_sub(p[i0], p[b0]))));
        prev_lo[t] = p[i0];
        const long long b1 = at(n - 1), i1 = at(n - 2);
        p[b1] = __double2float_rn(d_add((double)prev_hi[t], d_mul(coeff, (double)f_sub(p[i1], p[b1]))));
        prev_hi[t] = p[i1];
    } else {
        const long long b = side == 0 ? at(0) : at(n - 1), in = side == 0 ? at(1) : at(n - 2);
        const float pi = p[in], pb = p[b];
        const double abc = d_add((double)prev_lo[t], d_mul(coeff, (double)f_sub(pi, pb)));
        const float rig = f_mul(__double2float_rn(R), pi);
        p[b] = __double2float_rn(d_add((double)rig, d_mul(d_sub(1.0, R), abc)));
        prev_lo[t] = pi;
    }
}

// One source after the plane boundaries (core/solver.py:2386-2433): air
// cells of a point or a plane, p = float(double(p) + value).
__global__ void k_inject(float* __restrict__ p, const uint8_t* __restrict__ flags, int kind,
                         int a, int b, int c, const double* __restrict__ val, int nx, int ny,
                         int nz) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long cell;
    if (kind == 0) {
        if (t > 0) return;
        cell = ((long long)a * ny + b) * nz + c;
    } else {
        const int nu = a == 0 ? ny : nx, nv = a == 2 ? ny : nz;
        if (t >= (long long)nu * nv) return;
        const int u = (int)(t / nv), v = (int)(t % nv);
        if (a == 0) cell = ((long long)b * ny + u) * nz + v;
        else if (a == 1) cell = ((long long)u * ny + b) * nz + v;
        else cell = ((long long)u * ny + v) * nz + b;
    }
    if (flags && !(flags[cell] & SF_AIR)) return;
    p[cell] = __double2float_rn(d_add((double)p[cell], *val));
}

// A weighted (membrane) source: f[cells[t]] = float(double(f) + value * w[t])
// (core/solver.py:2389-2412, NumPy's float64 product and sum, one rounding).
__global__ void k_inject_weighted(float* __restrict__ f, const long long* __restrict__ cells,
                                  const double* __restrict__ w, long long n,
                                  const double* __restrict__ val) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const long long c = cells[t];
    f[c] = __double2float_rn(d_add((double)f[c], d_mul(*val, w[t])));
}

// Face flags from the geometry mask (boundaries.cpp:13-64 rule).
__global__ void k_build_flags(const uint8_t* __restrict__ geom, uint8_t* __restrict__ flags,
                              int nx, int ny, int nz) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= nz || j >= ny) return;
    const long long plane = (long long)ny * nz;
    const long long c = (long long)i * plane + (long long)j * nz + k;
    const bool a = geom[c] != 0;
    uint8_t f = a ? SF_AIR : 0;
    if (a && i < nx - 1 && geom[c + plane]) f |= SF_OPX;
    if (a && j < ny - 1 && geom[c + nz]) f |= SF_OPY;
    if (a && k < nz - 1 && geom[c + 1]) f |= SF_OPZ;
    flags[c] = f;
}

// Energy partial sums in FP64: block b writes (sum p^2, sum |v|^2) over air
// cells to scratch[2b], scratch[2b+1]; a second launch folds them.
constexpr int EN_THREADS = 256;
__global__ void k_energy_partial(const float* __restrict__ p, const float* __restrict__ vx,
                                 const float* __restrict__ vy, const float* __restrict__ vz,
                                 const uint8_t* __restrict__ flags, long long n,
                                 double* __restrict__ scratch) {
    __shared__ double sp[EN_THREADS], sv[EN_THREADS];
    double ap = 0.0, av = 0.0;
    for (long long c = (long long)blockIdx.x * EN_THREADS + threadIdx.x; c < n;
         c += (long long)gridDim.x * EN_THREADS) {
        if (flags != nullptr && !(flags[c] & SF_AIR)) continue;
        const double pp = p[c], x = vx[c], y = vy[c], z = vz[c];
        ap += pp * pp;
        av += x * x + y * y + z * z;
    }
    sp[threadIdx.x] = ap;
    sv[threadIdx.x] = av;
    __syncthreads();
    for (int s = EN_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sp[threadIdx.x] += sp[threadIdx.x + s];
            sv[threadIdx.x] += sv[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        scratch[2 * blockIdx.x] = sp[0];
        scratch[2 * blockIdx.x + 1] = sv[0];
    }
}

__global__ void k_energy_final(double* scratch, int nblocks, double* out) {
    __shared__ double sp[EN_THREADS], sv[EN_THREADS];
    double ap = 0.0, av = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += EN_THREADS) {
        ap += scratch[2 * b];
        av += scratch[2 * b + 1];
    }
    sp[threadIdx.x] = ap;
    sv[threadIdx.x] = av;
    __syncthreads();
    for (int s = EN_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sp[threadIdx.x] += sp[threadIdx.x + s];
            sv[threadIdx.x] += sv[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sp[0];
        out[1] = sv[0];
    }
}

}  // namespace

// ---- launchers used by sf_api.cu -------------------------------------------

int sf_launch_build_flags(const uint8_t* geom, uint8_t* flags, int nx, int ny, int nz,
                          cudaStream_t st) {
    dim3 blk(BX, BY, 1), grd((nz + BX - 1) / BX, (ny + BY - 1) / BY, nx);
    k_build_flags<<<grd, blk, 0, st>>>(geom, flags, nx, ny, nz);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_build_flags launch failed");
}

int sf_launch_step(const SfStepArgs& a, const SfSources& src, const SfPoles& poles, bool geom,
                   cudaStream_t st) {
    // the cells of a.reg_lo .. a.reg_hi (the whole grid unless the plan
    // splits an ADE step between a warp-tile kernel and this one)
    const int ex = a.reg_hi[0] - a.reg_lo[0], ey = a.reg_hi[1] - a.reg_lo[1],
              ez = a.reg_hi[2] - a.reg_lo[2];
    if (ex <= 0 || ey <= 0 || ez <= 0) return 0;
    dim3 blk(BX, BY, 1), grd((ez + BX - 1) / BX, (ey + BY - 1) / BY, ex);
    const bool ade = poles.n > 0;
    if (ade && poles.n_density > 0) {
        const long long n = (long long)(a.ade_hi[0] - a.ade_lo[0]) * (a.ade_hi[1] - a.ade_lo[1]) *
                            (a.ade_hi[2] - a.ade_lo[2]);
        const int blocks = (int)((n + 255) / 256 < 152 * 16 ? (n + 255) / 256 : 152 * 16);
        if (n > 0) k_ade_density<<<blocks, 256, 0, st>>>(a, poles, n);
    }
    const bool nu = a.nu_cv[0] != nullptr;
    if (nu) {
        if (geom)
            ade ? k_step<true, true, true><<<grd, blk, 0, st>>>(a, src, poles)
                : k_step<true, false, true><<<grd, blk, 0, st>>>(a, src, poles);
        else
            ade ? k_step<false, true, true><<<grd, blk, 0, st>>>(a, src, poles)
                : k_step<false, false, true><<<grd, blk, 0, st>>>(a, src, poles);
    } else if (geom) {
        if (ade)
            k_step<true, true, false><<<grd, blk, 0, st>>>(a, src, poles);
        else
            k_step<true, false, false><<<grd, blk, 0, st>>>(a, src, poles);
    } else {
        if (ade)
            k_step<false, true, false><<<grd, blk, 0, st>>>(a, src, poles);
        else
            k_step<false, false, false><<<grd, blk, 0, st>>>(a, src, poles);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_step launch failed");
}

int sf_launch_probe_gather(const float* p, const long long* cells, int n, float* out,
                           cudaStream_t st) {
    if (n <= 0) return 0;
    k_probe_gather<<<(n + 127) / 128, 128, 0, st>>>(p, cells, n, out);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_probe_gather launch failed");
}

int sf_launch_plane_bc(float* p, float* prev_lo, float* prev_hi, const sf_plane_bc& op, int nx,
                       int ny, int nz, cudaStream_t st) {
    const long long n = (long long)(op.axis == 0 ? ny : nx) * (op.axis == 2 ? ny : nz);
    k_plane_bc<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p, prev_lo, prev_hi, op.kind, op.axis,
                                                            op.side, op.coeff, op.reflection, nx,
                                                            ny, nz);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_plane_bc launch failed");
}

int sf_launch_inject(float* p, const uint8_t* flags, const sf_source& s, const double* val, int nx,
                     int ny, int nz, cudaStream_t st) {
    long long n = 1;
    if (s.kind != 0) n = (long long)(s.a == 0 ? ny : nx) * (s.a == 2 ? ny : nz);
    k_inject<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p, flags, s.kind, s.a, s.b, s.c, val, nx,
                                                          ny, nz);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_inject launch failed");
}

int sf_launch_inject_weighted(float* f, const long long* cells, const double* w, long long n,
                              const double* val, cudaStream_t st) {
    if (n <= 0) return 0;
    k_inject_weighted<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(f, cells, w, n, val);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_inject_weighted launch failed");
}

int sf_launch_mic_gather(const float* p, const float* vx, const float* vy, const float* vz,
                         const int* field, const long long* idx, const float* w, int n, float* out,
                         cudaStream_t st) {
    if (n <= 0) return 0;
    k_mic_gather<<<(n + 127) / 128, 128, 0, st>>>(p, vx, vy, vz, field, idx, w, n, out);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_mic_gather launch failed");
}

long long sf_energy_blocks(long long n, int sms) {
    const long long cap = 8LL * (sms > 0 ? sms : 1);
    long long b = (n + EN_THREADS - 1) / EN_THREADS;
    return b < cap ? (b < 1 ? 1 : b) : cap;
}

int sf_launch_energy(const float* p, const float* vx, const float* vy, const float* vz,
                     const uint8_t* flags, long long n, int sms, double* scratch, double* out2,
                     cudaStream_t st) {
    const int nb = (int)sf_energy_blocks(n, sms);
    k_energy_partial<<<nb, EN_THREADS, 0, st>>>(p, vx, vy, vz, flags, n, scratch);
    k_energy_final<<<1, EN_THREADS, 0, st>>>(scratch, nb, out2);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("energy launch failed");
}
