/*
 * sf_oracle.c -- CPU restatement of the strata-fdtd native time-step path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the GB300
 * kernels and the CPU baseline that bench.py times beside them.  Only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs load
 * it.  The product (strata_fdtd_gb300) never links, imports or calls it.
 *
 * The file is compiled twice from the same text:
 *   -DORC_REAL=float  -DORC_SUFFIX=f32   bit-exact restatement of the reference
 *                                        native (C++/OpenMP) kernels
 *   -DORC_REAL=double -DORC_SUFFIX=f64   the same arithmetic in FP64, used to
 *                                        state the error of every FP32 result
 * Compile with -ffp-contract=off: the reference x86 build has no FMA, and the
 * float results are only bit-exact without contraction.
 *
 * Every function cites the reference function it restates (paths relative to
 * src/strata_fdtd/ of rjwalters/strata-fdtd).  Layout everywhere is C order,
 * idx = (i*ny + j)*nz + k, as _kernels/include/fdtd_types.hpp:36-42.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#ifndef ORC_REAL
#define ORC_REAL float
#define ORC_SUFFIX f32
#endif

typedef ORC_REAL real;
#define ORC_CAT2(a, b) a##_##b
#define ORC_CAT(a, b) ORC_CAT2(a, b)
#define FN(name) ORC_CAT(orc_##name, ORC_SUFFIX)

#define IDX(i, j, k) ((((int64_t)(i)) * ny + (j)) * (int64_t)nz + (k))

#if defined(_OPENMP)
#include <omp.h>
#define OMP_FOR _Pragma("omp parallel for schedule(static)")
#else
#define OMP_FOR
#endif

/* _kernels/src/fdtd_step.cpp:15-82 (update_velocity).
 * v_a += cv * (p[a+1] - p[a]) for a < n_a - 1; the last plane is untouched. */
void FN(update_velocity)(const real* p, real* vx, real* vy, real* vz,
                         int nx, int ny, int nz, real cv) {
    OMP_FOR
    for (int i = 0; i < nx; i++) {
        for (int j = 0; j < ny; j++) {
            for (int k = 0; k < nz; k++) {
                const int64_t c = IDX(i, j, k);
                if (i < nx - 1) vx[c] += cv * (p[IDX(i + 1, j, k)] - p[c]);
                if (j < ny - 1) vy[c] += cv * (p[IDX(i, j + 1, k)] - p[c]);
                if (k < nz - 1) vz[c] += cv * (p[c + 1] - p[c]);
            }
        }
    }
}

/* _kernels/src/fdtd_step.cpp:84-212 (update_pressure).
 * p += cp * ((dvx + dvy) + dvz) with v[-1] = 0 on the low faces; p = 0 where
 * the geometry cell is solid (geom == NULL means all air). */
void FN(update_pressure)(real* p, const real* vx, const real* vy, const real* vz,
                         const uint8_t* geom, int nx, int ny, int nz, real cp) {
    OMP_FOR
    for (int i = 0; i < nx; i++) {
        for (int j = 0; j < ny; j++) {
            for (int k = 0; k < nz; k++) {
                const int64_t c = IDX(i, j, k);
                if (geom && !geom[c]) {
                    p[c] = (real)0;
                    continue;
                }
                const real dx = (i > 0) ? (vx[c] - vx[IDX(i - 1, j, k)]) : vx[c];
                const real dy = (j > 0) ? (vy[c] - vy[IDX(i, j - 1, k)]) : vy[c];
                const real dz = (k > 0) ? (vz[c] - vz[c - 1]) : vz[c];
                p[c] += cp * (dx + dy + dz);
            }
        }
    }
}

/* _kernels/src/fdtd_step.cpp:235-305 (update_velocity_nonuniform): the face
 * coefficient is formed per face as coeff_v_base * inv_face[i] (a rounded
 * product), then v += coeff * (p[a+1] - p[a]) for a < n_a - 1. */
void FN(update_velocity_nu)(const real* p, real* vx, real* vy, real* vz, int nx, int ny, int nz,
                            real cvb, const real* ifx, const real* ify, const real* ifz) {
    OMP_FOR
    for (int i = 0; i < nx; i++) {
        for (int j = 0; j < ny; j++) {
            for (int k = 0; k < nz; k++) {
                const int64_t c = IDX(i, j, k);
                if (i < nx - 1) {
                    const real cf = cvb * ifx[i];
                    vx[c] += cf * (p[IDX(i + 1, j, k)] - p[c]);
                }
                if (j < ny - 1) {
                    const real cf = cvb * ify[j];
                    vy[c] += cf * (p[IDX(i, j + 1, k)] - p[c]);
                }
                if (k < nz - 1) {
                    const real cf = cvb * ifz[k];
                    vz[c] += cf * (p[c + 1] - p[c]);
                }
            }
        }
    }
}

/* _kernels/src/fdtd_step.cpp:307-439 (update_pressure_nonuniform): each
 * difference scaled by the cell's inverse spacing before the sum, v[-1] = 0
 * on the low faces, p = 0 in solids:
 * p += cpb * ((icx (dvx) + icy (dvy)) + icz (dvz)). */
void FN(update_pressure_nu)(real* p, const real* vx, const real* vy, const real* vz,
                            const uint8_t* geom, int nx, int ny, int nz, real cpb,
                            const real* icx, const real* icy, const real* icz) {
    OMP_FOR
    for (int i = 0; i < nx; i++) {
        for (int j = 0; j < ny; j++) {
            for (int k = 0; k < nz; k++) {
                const int64_t c = IDX(i, j, k);
                if (geom && !geom[c]) {
                    p[c] = (real)0;
                    continue;
                }
                const real dx = icx[i] * ((i > 0) ? (vx[c] - vx[IDX(i - 1, j, k)]) : vx[c]);
                const real dy = icy[j] * ((j > 0) ? (vy[c] - vy[IDX(i, j - 1, k)]) : vy[c]);
                const real dz = icz[k] * ((k > 0) ? (vz[c] - vz[c - 1]) : vz[c]);
                p[c] += cpb * (dx + dy + dz);
            }
        }
    }
}

/* _kernels/src/boundaries.cpp:13-64 + 66-89 (precompute_boundary_cells and
 * apply_rigid_boundaries): a face velocity is zeroed when either cell that it
 * separates is solid.  The last plane along each axis carries no face. */
void FN(apply_rigid)(real* vx, real* vy, real* vz, const uint8_t* geom,
                     int nx, int ny, int nz) {
    OMP_FOR
    for (int i = 0; i < nx; i++) {
        for (int j = 0; j < ny; j++) {
            for (int k = 0; k < nz; k++) {
                const int64_t c = IDX(i, j, k);
                if (i < nx - 1 && (!geom[c] || !geom[IDX(i + 1, j, k)])) vx[c] = (real)0;
                if (j < ny - 1 && (!geom[c] || !geom[IDX(i, j + 1, k)])) vy[c] = (real)0;
                if (k < nz - 1 && (!geom[c] || !geom[c + 1])) vz[c] = (real)0;
            }
        }
    }
}

/* Face lists exactly as precompute_boundary_cells (boundaries.cpp:13-64):
 * ascending flat index, one list per axis.  Returns the number of entries
 * written (or needed, when out == NULL). */
int64_t FN(boundary_faces)(const uint8_t* geom, int nx, int ny, int nz, int axis,
                           int32_t* out) {
    int64_t n = 0;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                const int64_t c = IDX(i, j, k);
                int blocked = 0;
                if (axis == 0 && i < nx - 1) blocked = !geom[c] || !geom[IDX(i + 1, j, k)];
                if (axis == 1 && j < ny - 1) blocked = !geom[c] || !geom[IDX(i, j + 1, k)];
                if (axis == 2 && k < nz - 1) blocked = !geom[c] || !geom[c + 1];
                if (blocked) {
                    if (out) out[n] = (int32_t)c;
                    n++;
                }
            }
    return n;
}

/* _kernels/src/pml.cpp:13-45 (initialize_pml): decay = exp(-sigma * dt),
 * evaluated in the working precision (std::exp(float) in the reference). */
void FN(pml_decay)(const real* sigma, int n, real dt, real* out) {
    for (int i = 0; i < n; i++) {
#if defined(ORC_IS_DOUBLE)
        out[i] = exp(-sigma[i] * dt);
#else
        out[i] = expf(-sigma[i] * dt);
#endif
    }
}

/* _kernels/src/pml.cpp:47-98 (apply_pml_velocity): vx *= dx[i], vy *= dy[j],
 * vz *= dz[k] over every cell; a NULL decay array means that axis is off. */
void FN(pml_velocity)(real* vx, real* vy, real* vz, const real* dx, const real* dy,
                      const real* dz, int nx, int ny, int nz) {
    OMP_FOR
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                const int64_t c = IDX(i, j, k);
                if (dx) vx[c] *= dx[i];
                if (dy) vy[c] *= dy[j];
                if (dz) vz[c] *= dz[k];
            }
}

/* _kernels/src/pml.cpp:100-149 (apply_pml_pressure): three separate passes,
 * so p is rounded after each axis: ((p*dx[i])*dy[j])*dz[k]. */
void FN(pml_pressure)(real* p, const real* dx, const real* dy, const real* dz,
                      int nx, int ny, int nz) {
    OMP_FOR
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                const int64_t c = IDX(i, j, k);
                real v = p[c];
                if (dx) v = v * dx[i];
                if (dy) v = v * dy[j];
                if (dz) v = v * dz[k];
                p[c] = v;
            }
}

/* core/solver.py:2386-2421 (_inject_sources, point and plane): the waveform
 * value is an FP64 scalar, so NumPy evaluates p + val in double and rounds
 * once on the store.  kind 0 = point (a,b,c = i,j,k), kind 1 = plane
 * (a = axis, b = index).  Only air cells receive the source. */
void FN(inject)(real* p, const uint8_t* geom, int nx, int ny, int nz, int kind, int a,
                int b, int c, double val) {
    if (kind == 0) {
        const int64_t q = IDX(a, b, c);
        if (!geom || geom[q]) p[q] = (real)((double)p[q] + val);
        return;
    }
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                const int on = (a == 0 && i == b) || (a == 1 && j == b) || (a == 2 && k == b);
                if (!on) continue;
                const int64_t q = IDX(i, j, k);
                if (!geom || geom[q]) p[q] = (real)((double)p[q] + val);
            }
}

/* _kernels/src/ade.cpp:25-68 / 70-116 (update_ade_{density,modulus}_debye):
 * J = alpha*J + beta*src where material_id == mat. */
void FN(ade_debye)(real* J, const real* src, const uint8_t* mat, int mat_id, real alpha,
                   real beta, int64_t n) {
    OMP_FOR
    for (int64_t q = 0; q < n; q++)
        if (mat[q] == mat_id) J[q] = alpha * J[q] + beta * src[q];
}

/* _kernels/src/ade.cpp:118-170 / 172-226 (update_ade_*_lorentz):
 * J' = (a*J + b*Jprev) + d*src; Jprev' = J. */
void FN(ade_lorentz)(real* J, real* Jp, const real* src, const uint8_t* mat, int mat_id,
                     real a, real b, real d, int64_t n) {
    OMP_FOR
    for (int64_t q = 0; q < n; q++)
        if (mat[q] == mat_id) {
            const real j0 = J[q], jp = Jp[q];
            const real jn = a * j0 + b * jp + d * src[q];
            Jp[q] = j0;
            J[q] = jn;
        }
}

/* _kernels/src/ade.cpp:228-401 (apply_ade_velocity_correction), one density
 * pole: v_a += coeff * (J[a+1] - J[a]) on faces whose two cells are both in
 * material mat; coeff = (-dt / rho_inf) * inv_dx computed by the caller. */
void FN(ade_velocity_correction)(real* vx, real* vy, real* vz, const real* J,
                                 const uint8_t* mat, int mat_id, real coeff, int nx,
                                 int ny, int nz) {
    OMP_FOR
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                const int64_t c = IDX(i, j, k);
                if (mat[c] != mat_id) continue;
                if (i < nx - 1 && mat[IDX(i + 1, j, k)] == mat_id)
                    vx[c] += coeff * (J[IDX(i + 1, j, k)] - J[c]);
                if (j < ny - 1 && mat[IDX(i, j + 1, k)] == mat_id)
                    vy[c] += coeff * (J[IDX(i, j + 1, k)] - J[c]);
                if (k < nz - 1 && mat[c + 1] == mat_id) vz[c] += coeff * (J[c + 1] - J[c]);
            }
}

/* _kernels/src/ade.cpp:403-477 (apply_ade_pressure_correction), one modulus
 * pole: p += coeff * J where material_id == mat; coeff = -K_inf * dt. */
void FN(ade_pressure_correction)(real* p, const real* J, const uint8_t* mat, int mat_id,
                                 real coeff, int64_t n) {
    OMP_FOR
    for (int64_t q = 0; q < n; q++)
        if (mat[q] == mat_id) p[q] += coeff * J[q];
}

/* _kernels/src/ade.cpp:479-580 (compute_divergence): the x term is stored
 * first, then the y and z terms are added, each scaled by inv_dx before the
 * add: ((dvx*s) + (dvy*s)) + (dvz*s). */
void FN(divergence)(real* div, const real* vx, const real* vy, const real* vz, int nx,
                    int ny, int nz, real inv_dx) {
    OMP_FOR
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                const int64_t c = IDX(i, j, k);
                real d = ((i > 0) ? (vx[c] - vx[IDX(i - 1, j, k)]) : vx[c]) * inv_dx;
                d += ((j > 0) ? (vy[c] - vy[IDX(i, j - 1, k)]) : vy[c]) * inv_dx;
                d += ((k > 0) ? (vz[c] - vz[c - 1]) : vz[c]) * inv_dx;
                div[c] = d;
            }
}

/* _kernels/src/ade.cpp:582-694 (compute_divergence_nonuniform): the same
 * three passes with each cell's inverse spacing per axis, inv_d*_cell. */
void FN(divergence_nu)(real* div, const real* vx, const real* vy, const real* vz, int nx,
                       int ny, int nz, const real* sx, const real* sy, const real* sz) {
    OMP_FOR
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                const int64_t c = IDX(i, j, k);
                real d = ((i > 0) ? (vx[c] - vx[IDX(i - 1, j, k)]) : vx[c]) * sx[i];
                d += ((j > 0) ? (vy[c] - vy[IDX(i, j - 1, k)]) : vy[c]) * sy[j];
                d += ((k > 0) ? (vz[c] - vz[c - 1]) : vz[c]) * sz[k];
                div[c] = d;
            }
}

/* ------------------------------------------------------------------------ */
/* Whole-step driver for the plain path (no ADE), so that tests and the CPU
 * baseline can run many steps without a Python call per kernel.  Order is
 * FDTDSolver.step with backend="native" (core/solver.py:2003-2077):
 *   update_velocity -> apply_rigid_boundaries (if a geometry was set) ->
 *   update_pressure -> PML velocity -> PML pressure -> sources -> probes.
 * For speed the per-step work is fused into two OpenMP sweeps that keep each
 * cell's arithmetic identical to the separate reference passes.            */

typedef struct {
    int nx, ny, nz;
    real cv, cp;
    const uint8_t* geom; /* NULL: no geometry set (all air, no rigid pass) */
    const real *dx, *dy, *dz; /* PML decays, NULL = axis off */
    int n_src;
    const int32_t* src; /* n_src x 4: kind, a, b, c */
    int n_probe;
    const int64_t* probe_cell; /* flat indices */
} FN(plan);

void FN(run_plain)(const FN(plan) * P, real* p, real* vx, real* vy, real* vz,
                   int64_t n_steps, const double* src_vals /* n_steps x n_src */,
                   real* trace /* n_steps x n_probe */) {
    const int nx = P->nx, ny = P->ny, nz = P->nz;
    const real cv = P->cv, cp = P->cp;
    const uint8_t* g = P->geom;
    for (int64_t s = 0; s < n_steps; s++) {
        /* sweep 1: velocity update + rigid zero (per face, same arithmetic
         * as update_velocity followed by apply_rigid_boundaries) */
        OMP_FOR
        for (int i = 0; i < nx; i++)
            for (int j = 0; j < ny; j++)
                for (int k = 0; k < nz; k++) {
                    const int64_t c = IDX(i, j, k);
                    if (i < nx - 1) {
                        const int64_t n1 = IDX(i + 1, j, k);
                        vx[c] += cv * (p[n1] - p[c]);
                        if (g && (!g[c] || !g[n1])) vx[c] = (real)0;
                    }
                    if (j < ny - 1) {
                        const int64_t n1 = IDX(i, j + 1, k);
                        vy[c] += cv * (p[n1] - p[c]);
                        if (g && (!g[c] || !g[n1])) vy[c] = (real)0;
                    }
                    if (k < nz - 1) {
                        vz[c] += cv * (p[c + 1] - p[c]);
                        if (g && (!g[c] || !g[c + 1])) vz[c] = (real)0;
                    }
                }
        /* sweep 2: pressure update (reads the undecayed velocities), then
         * the PML velocity decay of the faces whose pressure readers are
         * all done -- each cell decays its own three faces after computing
         * its pressure; neighbours read the faces of lower cells, which is
         * why the decay is deferred to a third sweep. */
        OMP_FOR
        for (int i = 0; i < nx; i++)
            for (int j = 0; j < ny; j++)
                for (int k = 0; k < nz; k++) {
                    const int64_t c = IDX(i, j, k);
                    real pc;
                    if (g && !g[c]) {
                        pc = (real)0;
                    } else {
                        const real ddx = (i > 0) ? (vx[c] - vx[IDX(i - 1, j, k)]) : vx[c];
                        const real ddy = (j > 0) ? (vy[c] - vy[IDX(i, j - 1, k)]) : vy[c];
                        const real ddz = (k > 0) ? (vz[c] - vz[c - 1]) : vz[c];
                        pc = p[c] + cp * (ddx + ddy + ddz);
                    }
                    if (P->dx) pc = pc * P->dx[i];
                    if (P->dy) pc = pc * P->dy[j];
                    if (P->dz) pc = pc * P->dz[k];
                    p[c] = pc;
                }
        FN(pml_velocity)(vx, vy, vz, P->dx, P->dy, P->dz, nx, ny, nz);
        for (int q = 0; q < P->n_src; q++) {
            const int32_t* d = P->src + 4 * q;
            FN(inject)(p, g, nx, ny, nz, d[0], d[1], d[2], d[3], src_vals[s * P->n_src + q]);
        }
        for (int q = 0; q < P->n_probe; q++) trace[s * P->n_probe + q] = p[P->probe_cell[q]];
    }
}

int FN(omp_threads)(void) {
#if defined(_OPENMP)
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void FN(set_threads)(int n) {
#if defined(_OPENMP)
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
