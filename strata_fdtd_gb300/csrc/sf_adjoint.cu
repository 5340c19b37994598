// sf_adjoint.cu -- forward and reverse-time (adjoint) steps of the
// differentiable solve.
//
// Scheme: the reference's staggered update (fdtd_step.cpp:15-212 order) with a
// per-cell density rho = rho0 * (1 + theta) in place of the scalar rho of
// core/solver.py:1584-1586: every face velocity uses its own coefficient
//     cv_face = -(dt/dx) * (1/rho_lo + 1/rho_hi) / 2
// while the pressure coefficient cp = -K dt/dx keeps K = rho0 c^2.  Rigid
// walls (an optional air mask) set cv = 0 on every face that touches a solid
// cell: from rest such a face's velocity and a solid cell's pressure stay
// zero, as the reference's rigid pass and its p = 0 in solids
// (boundaries.cpp:66-89, fdtd_step.cpp:84-212) keep them, and the forward and
// adjoint kernels need no mask of their own.  PML decays and the point source
// as the reference (pml.cpp:47-149, core/solver.py:2413-2421); probe samples
// after each step.  The per-cell density, and the optional occupancy field
// phi that scales each face coefficient by (1 - phi_lo)(1 - phi_hi) (the
// geometry as a design field), are builder-defined: the reference has only
// a scalar rho and binary solids.
//
// One step is linear in the state u = (p, v):
//     v' = v + C G p          (C = diag(cv), G = face differences)
//     p' = p + cp Div v'
//     v'' = Dv v',  p'' = Dp p' + s
// so its adjoint, with mu_p = Dp lambda_p'' and
// mu_v = Dv lambda_v'' + cp Div^T mu_p, is
//     lambda_v = mu_v,  lambda_p = mu_p + G^T C mu_v,
//     dL/dcv_face += mu_v(face) * (G p^n)(face)
// which k_dadj evaluates per cell (one fused stencil pass, reverse time).
// Both directions are templated on the working precision: float, double, or
// dwf (double-word floats, sf_dw.cuh: FP64-class accuracy on the FP32 pipe).
// Values crossing the boundary (design field, source values, traces,
// targets, gradients) are in the "external" type: the working type itself,
// or double for dwf.
#include <cuda_runtime.h>

#include <type_traits>

#include "sf_common.cuh"
#include "sf_dw.cuh"
#include "sf_gb300.h"

namespace {

template <typename T>
struct Ext {
    using E = T;
    static __device__ __forceinline__ T in(E v) { return v; }
    static __device__ __forceinline__ E out(T v) { return v; }
};
template <>
struct Ext<dwf> {
    using E = double;
    static __device__ __forceinline__ dwf in(double v) { return dwf(v); }
    static __device__ __forceinline__ double out(dwf v) { return v.to_double(); }
};

template <typename T>
struct DiffPtrs {
    int nx, ny, nz;
    long long plane;
    T cp;
    const T* cvx;
    const T* cvy;
    const T* cvz;
    const T* dx;
    const T* dy;
    const T* dz;
    int unit_lo[3], unit_hi[3];  // sf_diff_desc: indices whose decays (and neighbours') are 1
};

// Whether every cell of this (32 k x 8 j) block at plane i, and each of its
// six neighbours, has all three decays exactly 1: block-uniform, so the
// kernels branch once into a body without the decay products.
template <typename T>
__device__ __forceinline__ bool block_in_unit_decay(const DiffPtrs<T>& g, int i) {
    const int j0 = blockIdx.y * blockDim.y, k0 = blockIdx.x * blockDim.x;
    const int j1 = min(j0 + (int)blockDim.y, g.ny) - 1, k1 = min(k0 + (int)blockDim.x, g.nz) - 1;
    return i >= g.unit_lo[0] && i < g.unit_hi[0] && j0 >= g.unit_lo[1] && j1 < g.unit_hi[1] &&
           k0 >= g.unit_lo[2] && k1 < g.unit_hi[2];
}

// Kernels with a second body for blocks where every decay is 1: the
// double-word ones, whose decay product is about ten FP32 instructions, and
// the FP64 ones, whose products run on GB300's narrow FP64 pipe (measured at
// 128^3: gradients 3% and 7% faster; the FP32 kernels, one FP32 multiply
// per product, measured slower with the second body).
template <typename T>
constexpr bool kUnitBodies = !std::is_same<T, float>::value;

// d * a, where UNIT says that the decay d is known to be exactly 1
template <bool UNIT, typename T>
__device__ __forceinline__ T decay_mul(T a, const T& d) {
    if constexpr (UNIT) return a;
    else return d * a;
}

// Per-face dL/dcv accumulators, 8 bytes per face.  The FP64 solve keeps a
// double.  The FP32 solve keeps a double-word pair of floats (hi, lo): each
// term a*b is formed exactly as ph + pl (pl = fma(a, b, -ph)) and added with
// the accurate double-word sum (AccurateDWPlusDW of Joldes, Muller and
// Popescu, "Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic", ACM TOMS 44(2), 2017: relative error at most
// 3u^2, u = 2^-24), so that the FP32 adjoint issues no FP64 instruction in
// its per-step kernel (GB300's FP64 pipe bounded it).
template <typename T>
struct GradAcc;

template <>
struct GradAcc<double> {
    template <class I>
    static __device__ __forceinline__ void add(double* g, I c, double a, double b) {
        g[c] += a * b;
    }
    template <class I>
    static __device__ __forceinline__ double load(const double* g, I c) { return g[c]; }
};

template <>
struct GradAcc<float> {
    // s + e = a + b exactly (Knuth's 2Sum)
    static __device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
        s = __fadd_rn(a, b);
        const float bv = __fsub_rn(s, a);
        const float av = __fsub_rn(s, bv);
        e = __fadd_rn(__fsub_rn(a, av), __fsub_rn(b, bv));
    }
    // s + e = a + b exactly when |a| >= |b| (Dekker's Fast2Sum)
    static __device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
        s = __fadd_rn(a, b);
        e = __fsub_rn(b, __fsub_rn(s, a));
    }
    template <class I>
    static __device__ __forceinline__ void add(double* g, I c, float a, float b) {
        float2* q = reinterpret_cast<float2*>(g) + c;
        const float2 x = *q;
        const float ph = __fmul_rn(a, b);
        const float pl = __fmaf_rn(a, b, -ph);
        float sh, sl, th, tl, vh, vl, zh, zl;
        two_sum(x.x, ph, sh, sl);
        two_sum(x.y, pl, th, tl);
        fast_two_sum(sh, __fadd_rn(sl, th), vh, vl);
        fast_two_sum(vh, __fadd_rn(tl, vl), zh, zl);
        *q = make_float2(zh, zl);
    }
    template <class I>
    static __device__ __forceinline__ double load(const double* g, I c) {
        const float2 v = reinterpret_cast<const float2*>(g)[c];
        return double(v.x) + double(v.y);
    }
};

// Double-word solve: double-word products of double-word factors, summed in
// double-word (sf_dw.cuh), the same 8 bytes per face.
template <>
struct GradAcc<dwf> {
    template <class I>
    static __device__ __forceinline__ void add(double* g, I c, dwf a, dwf b) {
        float2* q = reinterpret_cast<float2*>(g) + c;
        const float2 x = *q;
        const dwf z = sf_dw::add(dwf(x.x, x.y), a * b);  // accurate: a long running sum
        *q = make_float2(z.hi, z.lo);
    }
    template <class I>
    static __device__ __forceinline__ double load(const double* g, I c) {
        const float2 v = reinterpret_cast<const float2*>(g)[c];
        return double(v.x) + double(v.y);
    }
};

// Forward launches record up to this many probes themselves (one warp-uniform
// compare per probe and cell) instead of launching k_dprobe after each step.
constexpr int kFusedProbes = 4;

// Coefficients from theta: cv_a(c) for the face between c and c + e_a
// (zero on the last plane of each axis, which carries no face update, and on
// faces that touch a solid cell of the air mask `air`, when given).  With an
// occupancy field phi (solid fraction per cell) the face coefficient is
// scaled by the open fractions of its two cells, (1 - phi_c)(1 - phi_n):
// phi = 1 closes every face of the cell, a rigid wall.
// (formed in the external type: in double for a double-word solve, then
// rounded to the nearest double-word)
template <typename T, typename E = typename Ext<T>::E>
__global__ void k_dcoef(const E* __restrict__ theta, const uint8_t* __restrict__ air,
                        const E* __restrict__ occ, T* __restrict__ cvx, T* __restrict__ cvy,
                        T* __restrict__ cvz, int nx, int ny, int nz, E dt_dx, E rho0) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= nz || j >= ny) return;
    const long long plane = (long long)ny * nz;
    const long long c = (long long)i * plane + (long long)j * nz + k;
    const E b0 = E(1) / (rho0 * (E(1) + theta[c]));
    const bool solid = air && !air[c];
    const E w0 = occ ? E(1) - occ[c] : E(1);
    auto face = [&](long long n) {
        if (solid || (air && !air[n])) return T(0);
        const E b1 = E(1) / (rho0 * (E(1) + theta[n]));
        const E base = -dt_dx * E(0.5) * (b0 + b1);
        return Ext<T>::in(occ ? base * (w0 * (E(1) - occ[n])) : base);
    };
    cvx[c] = (i < nx - 1) ? face(c + plane) : T(0);
    cvy[c] = (j < ny - 1) ? face(c + nz) : T(0);
    cvz[c] = (k < nz - 1) ? face(c + 1) : T(0);
}

// Forward step (per cell, ping-pong): out = step(in); p_store, when given,
// receives the step's input pressure; with n_fused > 0 the cells listed in
// probe_cells write their new pressure into trace_row (else k_dprobe samples
// the output after the step).  I: the cell index type (int when the grid
// has fewer than 2^31 cells: cheaper address arithmetic, same results).
// UNIT: the block lies where every decay is 1, whose products are skipped.
template <bool UNIT, typename T, typename I, typename E>
__device__ __forceinline__ void dfwd_cell(const DiffPtrs<T>& g, int i, int j, int k, const T* __restrict__ p,
                                          const T* __restrict__ vx, const T* __restrict__ vy,
                                          const T* __restrict__ vz, T* __restrict__ po,
                                          T* __restrict__ vxo, T* __restrict__ vyo,
                                          T* __restrict__ vzo, long long src_cell,
                                          const T* __restrict__ src_val, T* __restrict__ p_store,
                                          const int64_t* __restrict__ probe_cells, int n_fused,
                                          E* __restrict__ trace_row) {
    const I plane = (I)g.plane;
    const I nz = g.nz;
    const I c = (I)i * plane + (I)j * nz + k;
    const T pc = p[c];
    if (p_store) p_store[c] = pc;
    T ux = vx[c], uy = vy[c], uz = vz[c];
    if (i < g.nx - 1) ux = ux + g.cvx[c] * (p[c + plane] - pc);
    if (j < g.ny - 1) uy = uy + g.cvy[c] * (p[c + nz] - pc);
    if (k < nz - 1) uz = uz + g.cvz[c] * (p[c + 1] - pc);
    T uxm = T(0), uym = T(0), uzm = T(0);
    if (i > 0) uxm = vx[c - plane] + g.cvx[c - plane] * (pc - p[c - plane]);
    if (j > 0) uym = vy[c - nz] + g.cvy[c - nz] * (pc - p[c - nz]);
    if (k > 0) uzm = vz[c - 1] + g.cvz[c - 1] * (pc - p[c - 1]);
    T pn = pc + g.cp * (((ux - uxm) + (uy - uym)) + (uz - uzm));
    if constexpr (UNIT) {
        vxo[c] = ux;
        vyo[c] = uy;
        vzo[c] = uz;
    } else {
        const T di = g.dx[i], dj = g.dy[j], dk = g.dz[k];
        vxo[c] = ux * di;
        vyo[c] = uy * dj;
        vzo[c] = uz * dk;
        pn = ((pn * di) * dj) * dk;
    }
    if ((long long)c == src_cell && src_val != nullptr) pn = pn + *src_val;
    po[c] = pn;
    for (int q = 0; q < n_fused; ++q)
        if ((long long)c == probe_cells[q]) trace_row[q] = Ext<T>::out(pn);
}

// Blocks of 256 threads per SM the forward asks for: with 32-bit cell
// indices 8 (32 registers), 6 in FP64 (40: its two bodies spill at 32); 4
// (64) with 64-bit ones.
template <typename T, typename I>
constexpr int kFwdMinBlocks = sizeof(I) == 8 ? 4 : (std::is_same<T, double>::value ? 6 : 8);

template <typename T, typename I, typename E = typename Ext<T>::E>
__global__ void __launch_bounds__(256, (kFwdMinBlocks<T, I>)) k_dfwd(DiffPtrs<T> g, const T* __restrict__ p, const T* __restrict__ vx,
                       const T* __restrict__ vy, const T* __restrict__ vz, T* __restrict__ po,
                       T* __restrict__ vxo, T* __restrict__ vyo, T* __restrict__ vzo,
                       long long src_cell, const T* __restrict__ src_val, T* __restrict__ p_store,
                       const int64_t* __restrict__ probe_cells, int n_fused, E* __restrict__ trace_row) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    const bool unit = kUnitBodies<T> && block_in_unit_decay(g, i);
    if (k >= g.nz || j >= g.ny) return;
    if (unit)
        dfwd_cell<kUnitBodies<T>, T, I, E>(g, i, j, k, p, vx, vy, vz, po, vxo, vyo, vzo, src_cell,
                                           src_val, p_store, probe_cells, n_fused, trace_row);
    else
        dfwd_cell<false, T, I, E>(g, i, j, k, p, vx, vy, vz, po, vxo, vyo, vzo, src_cell, src_val,
                                  p_store, probe_cells, n_fused, trace_row);
}

template <typename T, typename E = typename Ext<T>::E>
__global__ void k_dprobe(const T* __restrict__ p, const int64_t* __restrict__ cells, int n,
                         E* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = Ext<T>::out(p[cells[t]]);
}

// lambda_p(probe) += w * 2 (trace - target): the loss gradient at step n.
// (A double-word solve has no atomic add: one thread adds the probes in
// order, which also handles probes that share a cell.)
template <typename T, typename E = typename Ext<T>::E>
__global__ void k_dinject(T* __restrict__ lp, const int64_t* __restrict__ cells, int n,
                          const E* __restrict__ trace, const E* __restrict__ target, E w) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (std::is_same<T, dwf>::value) {
        if (t == 0)
            for (int q = 0; q < n; ++q)
                lp[cells[q]] = sf_dw::add(lp[cells[q]], dwf(w * 2.0 * (trace[q] - target[q])));
    } else {
        if (t < n) atomicAdd(&lp[cells[t]], w * T(2) * (trace[t] - target[t]));
    }
}

// Adjoint of one step.  in: lambda after the step; out: lambda before it;
// pst: p^n (the step's input pressure); g*: accumulated dL/dcv per face,
// 8 bytes per face as GradAcc<T> keeps them (the sum runs over every step
// and cancels, so it keeps about twice T's precision for T = float).
// UNIT: the block and its neighbours lie where every decay is 1, whose
// products are skipped.
template <bool UNIT, typename T, typename I>
__device__ __forceinline__ void dadj_cell(const DiffPtrs<T>& g, int i, int j, int k,
                                          const T* __restrict__ lp, const T* __restrict__ lx,
                                          const T* __restrict__ ly, const T* __restrict__ lz,
                                          T* __restrict__ lpo, T* __restrict__ lxo,
                                          T* __restrict__ lyo, T* __restrict__ lzo,
                                          const T* __restrict__ pst, double* __restrict__ gx,
                                          double* __restrict__ gy, double* __restrict__ gz) {
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const I plane = (I)g.plane;
    const I c = (I)i * plane + (I)j * nz + k;
    // mu_p = Dp lambda_p at this cell and its six neighbours
    auto mup = [&](int ii, int jj, int kk, I q) -> T {
        if constexpr (UNIT) return lp[q];
        else return g.dx[ii] * g.dy[jj] * g.dz[kk] * lp[q];
    };
    const T m0 = mup(i, j, k, c);
    const T mxp = (i < nx - 1) ? mup(i + 1, j, k, c + plane) : T(0);
    const T myp = (j < ny - 1) ? mup(i, j + 1, k, c + nz) : T(0);
    const T mzp = (k < nz - 1) ? mup(i, j, k + 1, c + 1) : T(0);
    // mu_v on the cell's high faces (the last plane's face has no +1 cell)
    const T vx_hi = decay_mul<UNIT>(lx[c], g.dx[i]) + g.cp * (m0 - mxp);
    const T vy_hi = decay_mul<UNIT>(ly[c], g.dy[j]) + g.cp * (m0 - myp);
    const T vz_hi = decay_mul<UNIT>(lz[c], g.dz[k]) + g.cp * (m0 - mzp);
    // mu_v on the low faces (owned by the lower neighbour)
    T vx_lo = T(0), vy_lo = T(0), vz_lo = T(0);
    if (i > 0)
        vx_lo = decay_mul<UNIT>(lx[c - plane], g.dx[i - 1]) + g.cp * (mup(i - 1, j, k, c - plane) - m0);
    if (j > 0)
        vy_lo = decay_mul<UNIT>(ly[c - nz], g.dy[j - 1]) + g.cp * (mup(i, j - 1, k, c - nz) - m0);
    if (k > 0)
        vz_lo = decay_mul<UNIT>(lz[c - 1], g.dz[k - 1]) + g.cp * (mup(i, j, k - 1, c - 1) - m0);
    lxo[c] = vx_hi;
    lyo[c] = vy_hi;
    lzo[c] = vz_hi;
    // lambda_p = mu_p + G^T C mu_v
    T acc = m0;
    if (i > 0) acc += g.cvx[c - plane] * vx_lo;
    if (j > 0) acc += g.cvy[c - nz] * vy_lo;
    if (k > 0) acc += g.cvz[c - 1] * vz_lo;
    acc -= g.cvx[c] * vx_hi + g.cvy[c] * vy_hi + g.cvz[c] * vz_hi;
    lpo[c] = acc;
    // dL/dcv on the high faces: mu_v * (p^n[hi] - p^n[lo])
    const T p0 = pst[c];
    if (i < nx - 1) GradAcc<T>::add(gx, c, vx_hi, pst[c + plane] - p0);
    if (j < ny - 1) GradAcc<T>::add(gy, c, vy_hi, pst[c + nz] - p0);
    if (k < nz - 1) GradAcc<T>::add(gz, c, vz_hi, pst[c + 1] - p0);
}

template <typename T, typename I>
__global__ void k_dadj(DiffPtrs<T> g, const T* __restrict__ lp, const T* __restrict__ lx,
                       const T* __restrict__ ly, const T* __restrict__ lz, T* __restrict__ lpo,
                       T* __restrict__ lxo, T* __restrict__ lyo, T* __restrict__ lzo,
                       const T* __restrict__ pst, double* __restrict__ gx,
                       double* __restrict__ gy, double* __restrict__ gz) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    const bool unit = kUnitBodies<T> && block_in_unit_decay(g, i);
    if (k >= g.nz || j >= g.ny) return;
    if (unit)
        dadj_cell<kUnitBodies<T>, T, I>(g, i, j, k, lp, lx, ly, lz, lpo, lxo, lyo, lzo, pst, gx, gy,
                                        gz);
    else
        dadj_cell<false, T, I>(g, i, j, k, lp, lx, ly, lz, lpo, lxo, lyo, lzo, pst, gx, gy, gz);
}

// dL/dtheta(c) = (dt/dx) rho0 / (2 rho(c)^2) * sum of dL/dcv over its faces;
// a wall face's cv is zero whatever theta is, so it contributes nothing, and a
// solid cell's gradient is zero.  With an occupancy field phi each face's
// term carries its open-fraction factor (1 - phi_c)(1 - phi_n), and, when
// out_occ is given, dL/dphi(c) = sum over the faces of dL/dcv * (-base)
// * (1 - phi_n), base = -(dt/dx)(1/rho_c + 1/rho_n)/2.
template <typename T, typename E = typename Ext<T>::E>
__global__ void k_dgrad(const E* __restrict__ theta, const uint8_t* __restrict__ air,
                        const E* __restrict__ occ, const double* __restrict__ gx,
                        const double* __restrict__ gy, const double* __restrict__ gz,
                        E* __restrict__ out, E* __restrict__ out_occ, int nx, int ny, int nz,
                        double dt_dx, double rho0) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= nz || j >= ny) return;
    const long long plane = (long long)ny * nz;
    const long long c = (long long)i * plane + (long long)j * nz + k;
    using A = GradAcc<T>;
    if (air && !air[c]) {
        out[c] = E(0);
        if (out_occ) out_occ[c] = E(0);
        return;
    }
    auto open = [&](long long n) { return !air || air[n]; };
    const double rho = rho0 * (1.0 + double(theta[c]));
    if (!occ) {
        // high faces (zero on the last plane), then the low ones
        double s = 0.0;
        if (i < nx - 1 && open(c + plane)) s += A::load(gx, c);
        if (j < ny - 1 && open(c + nz)) s += A::load(gy, c);
        if (k < nz - 1 && open(c + 1)) s += A::load(gz, c);
        if (i > 0 && open(c - plane)) s += A::load(gx, c - plane);
        if (j > 0 && open(c - nz)) s += A::load(gy, c - nz);
        if (k > 0 && open(c - 1)) s += A::load(gz, c - 1);
        out[c] = E(s * dt_dx * rho0 / (2.0 * rho * rho));
        return;
    }
    const double b0 = 1.0 / rho, w0 = 1.0 - double(occ[c]);
    double st = 0.0, so = 0.0;  // sum of dL/dcv * w_n; sum of dL/dcv * (-base) * w_n
    auto face = [&](const double* gf, long long q, long long n) {
        const double g = A::load(gf, q);
        const double wn = 1.0 - double(occ[n]);
        const double b1 = 1.0 / (rho0 * (1.0 + double(theta[n])));
        st += g * wn;
        so += g * (dt_dx * 0.5 * (b0 + b1)) * wn;
    };
    if (i < nx - 1 && open(c + plane)) face(gx, c, c + plane);
    if (j < ny - 1 && open(c + nz)) face(gy, c, c + nz);
    if (k < nz - 1 && open(c + 1)) face(gz, c, c + 1);
    if (i > 0 && open(c - plane)) face(gx, c - plane, c - plane);
    if (j > 0 && open(c - nz)) face(gy, c - nz, c - nz);
    if (k > 0 && open(c - 1)) face(gz, c - 1, c - 1);
    out[c] = E(st * w0 * dt_dx * rho0 / (2.0 * rho * rho));
    if (out_occ) out_occ[c] = E(so);
}

template <typename T>
DiffPtrs<T> ptrs(const sf_diff_desc* d, const void* const* cv) {
    DiffPtrs<T> g;
    g.nx = d->nx;
    g.ny = d->ny;
    g.nz = d->nz;
    g.plane = (long long)d->ny * d->nz;
    g.cp = (T)d->cp;
    g.cvx = static_cast<const T*>(cv[0]);
    g.cvy = static_cast<const T*>(cv[1]);
    g.cvz = static_cast<const T*>(cv[2]);
    g.dx = static_cast<const T*>(d->decay[0]);
    g.dy = static_cast<const T*>(d->decay[1]);
    g.dz = static_cast<const T*>(d->decay[2]);
    for (int a = 0; a < 3; ++a) {
        g.unit_lo[a] = d->unit_lo[a];
        g.unit_hi[a] = d->unit_hi[a];
    }
    return g;
}

dim3 grid_of(const sf_diff_desc* d) { return dim3((d->nz + 31) / 32, (d->ny + 7) / 8, d->nx); }

template <typename T>
int forward(const sf_diff_desc* d, const void* const* cv, void* const* set0, void* const* set1,
            int cur, int64_t n, const void* src_vals, void* trace, void* p_store, cudaStream_t st) {
    using E = typename Ext<T>::E;
    const DiffPtrs<T> g = ptrs<T>(d, cv);
    const long long N = (long long)d->nx * d->ny * d->nz;
    const T* sv = static_cast<const T*>(src_vals);  // already in the working type
    E* tr = static_cast<E*>(trace);
    T* ps = static_cast<T*>(p_store);
    const bool fuse = tr && d->n_probe > 0 && d->n_probe <= kFusedProbes;
    const bool narrow = N < (1LL << 31);
    for (int64_t s = 0; s < n; ++s) {
        void* const* in = cur ? set1 : set0;
        void* const* out = cur ? set0 : set1;
        auto kernel = narrow ? k_dfwd<T, int> : k_dfwd<T, long long>;
        kernel<<<grid_of(d), dim3(32, 8), 0, st>>>(
            g, (const T*)in[0], (const T*)in[1], (const T*)in[2], (const T*)in[3], (T*)out[0],
            (T*)out[1], (T*)out[2], (T*)out[3], d->src_cell, sv ? sv + s : nullptr,
            ps ? ps + s * N : nullptr, d->probe_cells, fuse ? d->n_probe : 0,
            fuse ? tr + s * d->n_probe : nullptr);
        if (tr && d->n_probe > 0 && !fuse)
            k_dprobe<T><<<(d->n_probe + 127) / 128, 128, 0, st>>>((const T*)out[0], d->probe_cells,
                                                                  d->n_probe, tr + s * d->n_probe);
        cur = 1 - cur;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("sf_diff_forward: launch failed");
}

template <typename T>
int adjoint(const sf_diff_desc* d, const void* const* cv, void* const* lam0, void* const* lam1,
            int cur, int64_t n, const void* p_store, const void* trace, const void* target,
            double weight, void* const* grad_cv, cudaStream_t st) {
    using E = typename Ext<T>::E;
    const DiffPtrs<T> g = ptrs<T>(d, cv);
    const long long N = (long long)d->nx * d->ny * d->nz;
    const T* ps = static_cast<const T*>(p_store);
    const E* tr = static_cast<const E*>(trace);
    const E* tg = static_cast<const E*>(target);
    const bool narrow = N < (1LL << 31);
    for (int64_t s = n - 1; s >= 0; --s) {
        void* const* in = cur ? lam1 : lam0;  // lambda after step s
        void* const* out = cur ? lam0 : lam1;
        if (tr && tg && d->n_probe > 0)
            k_dinject<T><<<(d->n_probe + 127) / 128, 128, 0, st>>>(
                (T*)in[0], d->probe_cells, d->n_probe, tr + s * d->n_probe, tg + s * d->n_probe,
                (E)weight);
        auto kernel = narrow ? k_dadj<T, int> : k_dadj<T, long long>;
        kernel<<<grid_of(d), dim3(32, 8), 0, st>>>(
            g, (const T*)in[0], (const T*)in[1], (const T*)in[2], (const T*)in[3], (T*)out[0],
            (T*)out[1], (T*)out[2], (T*)out[3], ps + s * N, (double*)grad_cv[0],
            (double*)grad_cv[1], (double*)grad_cv[2]);
        cur = 1 - cur;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("sf_diff_adjoint: launch failed");
}

int check_desc(const sf_diff_desc* d) {
    if (!d) return sf_fail("sf_diff: NULL descriptor");
    if (d->nx < 1 || d->ny < 1 || d->nz < 1 || d->nx > 65535)
        return sf_fail("sf_diff: bad grid dimensions");
    if (d->dtype < 0 || d->dtype > 2)
        return sf_fail("sf_diff: dtype must be 0 (f32), 1 (f64) or 2 (double-word f32)");
    if (!d->decay[0] || !d->decay[1] || !d->decay[2]) return sf_fail("sf_diff: decay arrays required");
    if (d->src_cell >= (long long)d->nx * d->ny * d->nz) return sf_fail("sf_diff: source outside");
    if (d->n_probe < 0 || (d->n_probe > 0 && !d->probe_cells)) return sf_fail("sf_diff: bad probes");
    return 0;
}

}  // namespace

extern "C" {

int sf_diff_coefficients(const sf_diff_desc* d, const void* theta, void* cvx, void* cvy, void* cvz,
                         void* stream) {
    if (int rc = check_desc(d)) return rc;
    if (!theta || !cvx || !cvy || !cvz) return sf_fail("sf_diff_coefficients: NULL buffer");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const dim3 grd = grid_of(d), blk(32, 8);
    if (d->dtype == 1)
        k_dcoef<double><<<grd, blk, 0, st>>>(
            (const double*)theta, d->geometry, (const double*)d->occupancy, (double*)cvx,
            (double*)cvy, (double*)cvz, d->nx, d->ny, d->nz, d->dt_over_dx, d->rho0);
    else if (d->dtype == 2)
        k_dcoef<dwf><<<grd, blk, 0, st>>>(
            (const double*)theta, d->geometry, (const double*)d->occupancy, (dwf*)cvx, (dwf*)cvy,
            (dwf*)cvz, d->nx, d->ny, d->nz, d->dt_over_dx, d->rho0);
    else
        k_dcoef<float><<<grd, blk, 0, st>>>(
            (const float*)theta, d->geometry, (const float*)d->occupancy, (float*)cvx, (float*)cvy,
            (float*)cvz, d->nx, d->ny, d->nz, (float)d->dt_over_dx, (float)d->rho0);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("sf_diff_coefficients: launch failed");
}

int sf_diff_forward(const sf_diff_desc* d, void* const* cv, void* const* set0, void* const* set1,
                    int cur, int64_t n_steps, const void* src_vals, void* trace, void* p_store,
                    void* stream) {
    if (int rc = check_desc(d)) return rc;
    if (!cv || !set0 || !set1 || (cur != 0 && cur != 1) || n_steps < 0)
        return sf_fail("sf_diff_forward: bad arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (d->dtype == 2)
        return forward<dwf>(d, cv, set0, set1, cur, n_steps, src_vals, trace, p_store, st);
    return d->dtype == 1
               ? forward<double>(d, cv, set0, set1, cur, n_steps, src_vals, trace, p_store, st)
               : forward<float>(d, cv, set0, set1, cur, n_steps, src_vals, trace, p_store, st);
}

int sf_diff_adjoint(const sf_diff_desc* d, void* const* cv, void* const* lam0, void* const* lam1,
                    int cur, int64_t n_steps, const void* p_store, const void* trace,
                    const void* target, double weight, void* const* grad_cv, void* stream) {
    if (int rc = check_desc(d)) return rc;
    if (!cv || !lam0 || !lam1 || !p_store || !grad_cv || (cur != 0 && cur != 1) || n_steps < 0)
        return sf_fail("sf_diff_adjoint: bad arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (d->dtype == 2)
        return adjoint<dwf>(d, cv, lam0, lam1, cur, n_steps, p_store, trace, target, weight,
                            grad_cv, st);
    return d->dtype == 1 ? adjoint<double>(d, cv, lam0, lam1, cur, n_steps, p_store, trace, target,
                                           weight, grad_cv, st)
                         : adjoint<float>(d, cv, lam0, lam1, cur, n_steps, p_store, trace, target,
                                          weight, grad_cv, st);
}

int sf_diff_grad_fields(const sf_diff_desc* d, const void* theta, void* const* grad_cv,
                        void* out_theta, void* out_occupancy, void* stream) {
    if (int rc = check_desc(d)) return rc;
    if (!theta || !grad_cv || !out_theta) return sf_fail("sf_diff_grad_fields: NULL buffer");
    if (out_occupancy && !d->occupancy)
        return sf_fail("sf_diff_grad_fields: an occupancy gradient needs the occupancy field");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const double* g0 = (const double*)grad_cv[0];
    const double* g1 = (const double*)grad_cv[1];
    const double* g2 = (const double*)grad_cv[2];
    if (d->dtype == 1)
        k_dgrad<double><<<grid_of(d), dim3(32, 8), 0, st>>>(
            (const double*)theta, d->geometry, (const double*)d->occupancy, g0, g1, g2,
            (double*)out_theta, (double*)out_occupancy, d->nx, d->ny, d->nz, d->dt_over_dx,
            d->rho0);
    else if (d->dtype == 2)
        k_dgrad<dwf><<<grid_of(d), dim3(32, 8), 0, st>>>(
            (const double*)theta, d->geometry, (const double*)d->occupancy, g0, g1, g2,
            (double*)out_theta, (double*)out_occupancy, d->nx, d->ny, d->nz, d->dt_over_dx,
            d->rho0);
    else
        k_dgrad<float><<<grid_of(d), dim3(32, 8), 0, st>>>(
            (const float*)theta, d->geometry, (const float*)d->occupancy, g0, g1, g2,
            (float*)out_theta, (float*)out_occupancy, d->nx, d->ny, d->nz, d->dt_over_dx,
            d->rho0);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("sf_diff_grad_fields: launch failed");
}

int sf_diff_grad_theta(const sf_diff_desc* d, const void* theta, void* const* grad_cv, void* out,
                       void* stream) {
    return sf_diff_grad_fields(d, theta, grad_cv, out, nullptr, stream);
}

}  // extern "C"
