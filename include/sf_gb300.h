/*
 * sf_gb300.h -- C ABI of the GB300 (sm_103a) time-step path for the
 * strata-fdtd acoustic FDTD solver.
 *
 * This library replaces the reference's pybind11 module `_kernels`
 * (src/strata_fdtd/_kernels/kernels.cpp:74-924 of rjwalters/strata-fdtd),
 * which the solver calls once per kernel per step with host NumPy arrays.
 * Here the boundary sits one level higher: a *plan* holds one grid's
 * device-resident state description, and one call advances it by many steps.
 *
 * Conventions
 *  - Every function returns int status: 0 = ok, nonzero = error; the message
 *    is in sf_last_error() (thread-local).  No C++ exception crosses the ABI.
 *  - Field buffers are caller-owned device memory (the Python layer uses
 *    PyTorch tensors), float32, C order: idx = (i*ny + j)*nz + k.
 *  - Work is enqueued on the caller's stream (cudaStream_t passed as void*,
 *    NULL = legacy default stream) and is asynchronous unless stated.
 *  - A plan is used by one host thread at a time.
 *  - Arithmetic reproduces the reference native path bit for bit (FP32, no
 *    fused multiply-add, reference operation order).
 */
#ifndef SF_GB300_H
#define SF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SF_ABI_VERSION 1
#define SF_MAX_SOURCES 16
#define SF_MAX_POLES 16
#define SF_MAX_PLANE_OPS 8

typedef struct sf_plan sf_plan;

/* Grid description.  coeff_v / coeff_p are the FP32-rounded scalars that the
 * reference passes as `float` through pybind11 (core/solver.py:1584-1586 ->
 * kernels.cpp:113,146). */
typedef struct {
    int32_t nx, ny, nz;
    float coeff_v; /* -dt / (rho*dx) */
    float coeff_p; /* -rho*c^2*dt / dx */
    uint32_t flags; /* reserved, 0 */
} sf_grid_desc;

/* Source descriptor (core/solver.py:2413-2433): kind 0 = point at (a,b,c);
 * kind 1 = plane with axis a (0,1,2) at index b; kind 2 = weighted cell
 * list a (sf_plan_set_weighted_source) added to field b (0 p, 1 vx, 2 vy,
 * 3 vz), a membrane source.  Sources inject into air
 * cells only, in the order given. */
typedef struct {
    int32_t kind, a, b, c;
} sf_source;

/* ADE pole (materials/base.py:157-188, ade.hpp:44-109).  kind 0 = Debye
 * (c0 = alpha, c1 = beta), kind 1 = Lorentz (c0 = a, c1 = b, c2 = d).
 * target 0 = density, 1 = modulus.  corr is the FP32 correction coefficient
 * as ade.cpp forms it: density (-dt / rho_inf) * inv_dx (ade.cpp:263);
 * modulus -K_inf * dt (ade.cpp:420).  J / J_prev are caller-owned device
 * arrays of nx*ny*nz floats (J_prev only for Lorentz). */
typedef struct {
    int32_t material_id, kind, target, reserved;
    float c0, c1, c2, corr;
    float* J;
    float* J_prev;
} sf_pole;

/* SDF program node for sf_voxelize (geometry/sdf.py).  Nodes run in order
 * on a distance stack and a point stack:
 *   op 1 BOX      a = centre, b = size
 *   op 2 SPHERE   a = centre, s0 = radius
 *   op 3 CYLINDER a = p1, b = unit axis, s0 = length, s1 = radius
 *   op 10 UNION n          pop n, push min (child order)
 *   op 11 INTERSECTION n   pop n, push max
 *   op 12 DIFFERENCE n     pop n (base first), push max(base, -s1, -s2 ...)
 *   op 20 PUSH_TRANSLATE a push point - a
 *   op 21 PUSH_SCALE a     push point / a
 *   op 22 POP_POINT
 *   op 23 SCALE_DIST s0    top distance *= s0
 *   op 24 NEGATE           top distance = -top
 *   op 25 PUSH_ROTATE a, b push the point times rows a, b (and the next
 *                          node's a, op 26 ROTATE_ROW2) of a 3x3 matrix
 *   op 4 CONE     a = p1, b = unit axis, s0 = length, s1 = r1; the next
 *                 node (op 27 DATA) a[0] = r2 - r1
 *   op 5 HORN     a = throat, b = unit axis, s0 = length, s1 = throat
 *                 radius, n = flare (0 conical, 1 exponential, 2 hyperbolic,
 *                 3 tractrix); the next DATA node a[0] = its constant (m,
 *                 alpha, alpha, R)
 *   op 6 TUBE n   a tube along the 3-D path of the next n DATA nodes (a =
 *                 vertex, s0 = radius there, b = segment to the next vertex,
 *                 s1 = its squared length)
 *   op 7 SPIRAL n the same in the xy plane, extruded over 0 <= z <= s0
 *   op 13 SMOOTH_UNION, 14 SMOOTH_INTERSECTION, 15 SMOOTH_DIFFERENCE
 *                 pop b, a (pushed in that order), push the polynomial blend
 *                 of a and b (negated b for 15) with radius s0  */
typedef struct {
    int32_t op, n;
    double a[3], b[3];
    double s0, s1;
} sf_sdf_node;

/* Pressure-plane boundary operation, applied after the PML in list order
 * (the reference's boundary loop, core/solver.py:2040-2047).  kind 0 = Mur
 * first-order ABC on both ends of `axis` (_boundaries.py:420-527): p_b =
 * float(double(prev) + coeff * double(p_i - p_b)), prev = p_i, low end then
 * high end; kind 1 = radiation impedance on one end (side 0 low, 1 high;
 * _boundaries.py:529-793): p_b = float(double(float(R) * p_i) + (1 - R) *
 * (double(prev) + coeff * double(p_i - p_b))), prev = p_i.  coeff is the
 * Mur coefficient (c dt - dx)/(c dt + dx) in FP64, R the reflection. */
typedef struct {
    int32_t kind, axis, side, reserved;
    double coeff, reflection;
} sf_plane_bc;

typedef struct {
    int32_t device, sm_count, cc_major, cc_minor;
    int64_t total_mem;
    int32_t l2_bytes, max_smem_per_block;
    char name[96];
} sf_device_info_t;

/* --- library ------------------------------------------------------------ */
/* Replaces _kernels.__version__ / has_openmp (kernels.cpp:76-84). */
const char* sf_version(void);
const char* sf_last_error(void);
int sf_device_info(int device, sf_device_info_t* out);

/* --- plans --------------------------------------------------------------- */
/* Replaces the per-call shape checks of kernels.cpp:21-65 and the
 * coefficient hand-off of core/solver.py:1584-1586. */
int sf_plan_create(const sf_grid_desc* desc, sf_plan** out);
/* The plan's own device tables (face flags, decays, probe cells ...) are
 * queued for release rather than freed at once: cudaFree waits for every
 * kernel on the device, which would stall a host that retires one solve
 * while others run.  The queue is released when 1 GiB or 4096 buffers have
 * accumulated, or by sf_release_deferred(); batches (sf_batch_destroy) do
 * the same with their tables and graphs. */
int sf_plan_destroy(sf_plan* plan);
/* Free every queued buffer and graph now (waits for the device).  No
 * counterpart in the reference. */
int sf_release_deferred(void);

/* Bind the two ping-pong copies of p, vx, vy, vz (8 device buffers of
 * nx*ny*nz floats).  Set 0 holds the current state.  The plan never frees
 * them.  Replaces the NumPy arrays passed to update_velocity /
 * update_pressure (kernels.cpp:108-176). */
int sf_plan_bind_fields(sf_plan* plan, float* p0, float* vx0, float* vy0, float* vz0,
                        float* p1, float* vx1, float* vy1, float* vz1);
/* Which set (0 or 1) holds the current state after the steps so far. */
int sf_plan_current(const sf_plan* plan);
/* Choose which set holds the current state (after a host upload). */
int sf_plan_set_current(sf_plan* plan, int which);

/* Geometry mask (device, nx*ny*nz bytes, nonzero = air) or NULL for all
 * air.  Builds the plan's per-cell face flags on the stream.  Replaces
 * precompute_boundary_cells + apply_rigid_boundaries (kernels.cpp:226-273,
 * boundaries.cpp:13-89) and the geometry argument of update_pressure. */
int sf_plan_set_geometry(sf_plan* plan, const uint8_t* geometry_dev, void* stream);

/* PML sigma profiles (host float arrays of nx, ny, nz, or NULL = axis off)
 * and dt as the float the reference passes; decays exp(-sigma*dt) are formed
 * on the host in float exactly as initialize_pml (pml.cpp:13-45,
 * kernels.cpp:286-329) and applied as apply_pml_velocity / apply_pml_pressure
 * (pml.cpp:47-149). */
int sf_plan_set_pml(sf_plan* plan, const float* sigma_x, const float* sigma_y,
                    const float* sigma_z, float dt);
/* Same, with decay factors supplied directly (host float arrays or NULL). */
int sf_plan_set_pml_decay(sf_plan* plan, const float* decay_x, const float* decay_y,
                          const float* decay_z);

/* Sources (at most SF_MAX_SOURCES) -- replaces _inject_sources
 * (core/solver.py:2386-2433). */
int sf_plan_set_sources(sf_plan* plan, int n, const sf_source* sources);
/* Probe cells (flat indices, host array) -- replaces _record_probes
 * (core/solver.py:2435-2439). */
int sf_plan_set_probes(sf_plan* plan, int n, const int64_t* cells);

/* Omni microphones: per microphone 8 corner cells (flat indices) and 8
 * float weights, host arrays of 8*n, in the corner order and float
 * arithmetic of precompute_microphone_data (microphones.cpp:16-80);
 * recorded after each step by sf_plan_step_ex as the float sum from 0 of
 * weight * p (record_microphones_batch, microphones.cpp:82-118). */
int sf_plan_set_microphones(sf_plan* plan, int n, const int64_t* idx8, const float* w8);
/* Microphone rows of any field: field[n] selects what row q interpolates
 * (0 p, 1 vx, 2 vy, 3 vz; NULL = all p).  A directional microphone of the
 * reference (Microphone.record with velocities, core/solver.py:1004-1118)
 * is four rows -- p at its grid position, vx/vy/vz at the staggered,
 * clamped positions of _interpolate_velocity -- with float32 weights, the
 * same float products and float sum from 0; the polar-pattern combination
 * of the four samples (core/solver.py:1120-1179) runs on the host. */
int sf_plan_set_microphones_ex(sf_plan* plan, int n, const int32_t* field, const int64_t* idx8,
                               const float* w8);

/* ADE materials: material_id (device, nx*ny*nz bytes) and the pole table
 * (at most SF_MAX_POLES; Debye poles first, then Lorentz, each in field
 * order, as ADEMaterialData holds them).  inv_dx = float(1/dx).  Replaces
 * update_ade_* / apply_ade_*_correction / compute_divergence
 * (kernels.cpp:670-886, ade.cpp:25-580) in the order of
 * core/solver.py:2135-2193; on a nonuniform grid (sf_plan_set_nonuniform)
 * compute_divergence_nonuniform (ade.cpp:582-694) in the order of
 * core/solver.py:2195-2283, the corrections still with inv_dx (the
 * reference passes 1/min spacing).  n = 0 turns ADE off. */
int sf_plan_set_ade(sf_plan* plan, const uint8_t* material_id_dev, int n, const sf_pole* poles,
                    float inv_dx);

/* Nonuniform grid (core/grid.py:148-532; replaces create_nonuniform_grid_data
 * and update_velocity/pressure_nonuniform, fdtd_step.cpp:235-456).
 * cv_face[a]: n_a floats, cv_face[a][i] = float(coeff_v_base) *
 * inv_face[a][i] formed in float by the caller (the last entry is unused);
 * inv_cell[a]: n_a cell inverse spacings.  The grid descriptor's coeff_p is
 * then coeff_p_base = -rho c^2 dt and coeff_v is unused: the velocity update
 * is v += cv_face[i] * (p[i+1] - p[i]) and the pressure update p +=
 * coeff_p_base * ((inv_x (dvx) + inv_y (dvy)) + inv_z (dvz)), each term
 * scaled before the sum.  Steps run the warp-tile kernels (and, with ADE
 * materials, the per-cell kernel inside the material box).  Both NULL
 * returns the plan to a uniform grid. */
int sf_plan_set_nonuniform(sf_plan* plan, const float* const* cv_face, const float* const* inv_cell);

/* Weighted cell list `slot` (0 .. SF_MAX_SOURCES-1) of a kind-2 source:
 * after each step field[cells[q]] = float(double(field[cells[q]]) + value *
 * weights[q]) for the air cells listed (the caller lists only air cells), as
 * NumPy's p[mask] += value * weights[mask] (core/solver.py:2389-2412).  Host
 * arrays of n; n = 0 clears the slot.  Kind-2 sources are injected after the
 * step and its plane boundaries, with the other sources, in order. */
int sf_plan_set_weighted_source(sf_plan* plan, int slot, int64_t n, const int64_t* cells,
                                const double* weights);

/* Plane boundary operations (at most SF_MAX_PLANE_OPS; n = 0 removes them)
 * and their stored planes, zeroed.  With any of them a step runs: the fused
 * update with the PML, the operations in order, then the sources, as the
 * reference's step does (core/solver.py:2040-2052).  Each axis an
 * operation touches needs at least 2 cells.  Replaces ABCFirstOrder /
 * RadiationImpedance.apply_pressure. */
int sf_plan_set_plane_boundaries(sf_plan* plan, int n, const sf_plane_bc* ops);

/* Box [lo, hi) holding every cell with a nonzero material id; the
 * density-pole pass walks only this box, and an ADE step on a warp-tile
 * configuration gives the box (grown by one cell, rounded out to whole
 * tiles) to the per-cell ADE kernel and the rest of the grid to the
 * warp-tile kernel.  No counterpart in the reference (its ADE kernels sweep
 * the whole grid). */
int sf_plan_set_ade_box(sf_plan* plan, const int32_t* lo, const int32_t* hi);

/* Step-kernel configuration.  config 0 = automatic (the autotuned
 * configuration if sf_plan_autotune ran, else the default warp tiles), 1 =
 * one thread per cell, 2 = slab march along i with shared-memory halos,
 * then thread columns along i ("col*": vector width, block rows, register
 * cap, streaming stores) and warp tiles with lane-shuffled neighbours
 * ("tile_*": float4 lanes, needs nz % 4 == 0 and 16-byte aligned fields;
 * "tile1_*": one cell per lane; "*_wb": ordinary write-back stores of the
 * new state instead of evict-first ones), then multi-step pipelines
 * ("tile_pipe*", "tile_stream*": 2 or 3 steps per launch, the intermediate
 * states in rings of planes held in L2; used for whole groups of steps when
 * the plan has float4 tiles, no ADE poles, no microphones, plane boundaries
 * or weighted sources, and the streaming form's warps all fit on the device
 * at once; other steps run the default warp tiles), as named by
 * sf_kernel_config_name.  A
 * configuration the grid cannot take falls back to scalar columns.  i_chunk
 * = planes per block (0 = automatic; pipelines: planes per chunk / between
 * progress updates).  With ADE poles the warp-tile
 * configurations split each step with the per-cell kernel (see
 * sf_plan_set_ade_box); any other configuration runs the per-cell kernel.
 * Every configuration gives identical results.  No counterpart in the
 * reference (its kernels are CPU loops). */
int sf_plan_set_kernel(sf_plan* plan, int config, int i_chunk);
int sf_kernel_config_count(void);
const char* sf_kernel_config_name(int config);

/* Bound of every cross-warp wait inside the multi-step pipeline kernels:
 * `spins` sleeps of 64-256 ns before a wait gives up (0 = the default 2^22,
 * about 1 s).  On expiry the kernel sets an error flag, its other waits and
 * claims return at once, and sf_plan_step returns nonzero with "a
 * dependency wait expired" in sf_last_error(); the state of that call is
 * void and the next call starts clean.  hold_first_item != 0 is a test hook:
 * the first work item also waits on a device flag that nothing sets, so the
 * expiry path runs without any fault.  No counterpart in the reference. */
int sf_plan_set_wait_limit(sf_plan* plan, int64_t spins, int hold_first_item);

/* Autotuner: times every single-step configuration (the multi-step
 * pipelines only run when chosen with sf_plan_set_kernel) that fits the
 * grid for `launches`
 * step launches each (reading the current state and writing the other set
 * without swapping, no sources, no probes -- the state is unchanged) and
 * makes the fastest the plan's automatic choice, then times that one with
 * 8-48 planes per block (pipelines: 1-8 planes per chunk) unless
 * sf_plan_set_kernel fixed i_chunk, and keeps the fastest; with ADE poles
 * only the warp-tile configurations, timed outside their ADE region.  ms_out
 * (host, may be NULL) receives sf_kernel_config_count() times per step (-1 =
 * not run);
 * best_out (may be NULL) the chosen configuration.  Synchronises the stream.
 * No counterpart in the reference. */
int sf_plan_autotune(sf_plan* plan, int launches, void* stream, float* ms_out, int* best_out);

/* Advance n_steps.  src_values_dev: device doubles [n_steps][n_sources]
 * (the waveform at each step's time; may be NULL when there are no
 * sources).  trace_dev: device floats [n_steps][n_probes] receiving p at
 * each probe after each step (may be NULL when there are no probes).  A
 * call that ran a multi-step pipeline synchronises the stream at its end to
 * read the pipeline's wait-expiry flag (outside stream capture), and fails
 * if a bounded wait expired.
 * Replaces FDTDSolver.step's native dispatch (core/solver.py:2003-2102). */
int sf_plan_step(sf_plan* plan, int64_t n_steps, const double* src_values_dev,
                 float* trace_dev, void* stream);
/* Same, also writing microphone samples to mic_trace_dev [n_steps][n_mics]
 * (may be NULL). */
int sf_plan_step_ex(sf_plan* plan, int64_t n_steps, const double* src_values_dev,
                    float* trace_dev, float* mic_trace_dev, void* stream);

/* Acoustic energy of the current state, (1/2) sum(p^2/(rho c^2) + rho v^2)
 * dV over air cells, as compute_energy (core/solver.py:2689-2705); result
 * written to a host double after a stream sync.  scratch_dev: device
 * doubles, at least sf_energy_scratch_doubles() of them. */
int64_t sf_energy_scratch_doubles(const sf_plan* plan);
int sf_plan_energy(sf_plan* plan, double rho, double c, double dx, double* scratch_dev,
                   double* out_host, void* stream);

/* The same energy for callers that cannot allocate device memory when they
 * need the number (a process whose HBM another caching allocator holds, or
 * a real-time loop that must not call cudaMalloc / cudaFree).  No
 * counterpart in the reference.  It allocates nothing: its scratch is a
 * fixed 4096-double (32 KiB) array in the library's device image, present
 * on every GPU that loads the library until exit.  The array's device
 * address is looked up (cudaGetSymbolAddress) once per device, with that
 * device current, by the first sf_plan_create on it, so this call neither
 * loads the module nor looks anything up; plans and this entry point are not
 * usable across a cudaDeviceReset.  Calls share the array: two calls whose
 * work overlaps on the GPU race.  Refuses (nonzero status) a reduction that
 * would need more than the 4096 doubles (a device with more than 255 SMs).
 * Synchronises the stream. */
int sf_plan_energy_noalloc(sf_plan* plan, double rho, double c, double dx, double* out_host,
                           void* stream);

/* --- batches of independent grids ---------------------------------------- */
/* A batch advances many plans (grids of any sizes, with or without
 * geometry, PML, sources, probes, ADE) together: per time step one
 * persistent launch whose warps take (grid, i-chunk, row block, column
 * block) work items from a device work queue, plus the ADE density pass,
 * the probe gather and a step-counter advance.  Results are identical to
 * stepping each plan alone.  No counterpart in the reference (it steps one
 * solver at a time on the CPU). */
typedef struct sf_batch sf_batch;
int sf_batch_create(sf_batch** out);
int sf_batch_destroy(sf_batch* batch);
/* Add a plan that will run n_steps (its own count; shorter members drop out
 * of the queue).  src_values_dev: [n_steps][n_sources] doubles; trace_dev:
 * [n_steps][n_probes] floats or NULL.  Pointers advance with each run. */
int sf_batch_add(sf_batch* batch, sf_plan* plan, int64_t n_steps, const double* src_values_dev,
                 float* trace_dev);
/* Same, with mic_trace_dev [n_steps][microphone rows] floats receiving the
 * plan's microphone rows after each step (required when it has any).
 * Nonuniform grids join the batch (warp-tile items) unless they also carry
 * ADE materials; plans with plane boundaries or weighted (membrane) sources
 * are refused: they step alone.  No counterpart in the reference. */
int sf_batch_add_ex(sf_batch* batch, sf_plan* plan, int64_t n_steps,
                    const double* src_values_dev, float* trace_dev, float* mic_trace_dev);
int sf_batch_clear(sf_batch* batch);
/* Work-item shape: rows of 32 columns (4, 8 or 16; the thread-column path
 * only -- warp tiles take 4 rows with float4 lanes, else 2) and i planes per
 * item (0 = 16).  sf_batch_tiles: the number of items of the last build. */
int sf_batch_set_tiles(sf_batch* batch, int rows, int i_chunk);
int sf_batch_tiles(const sf_batch* batch);
/* Path of the items away from every material box: 0 thread columns, 1
 * warp tiles (lane-shuffled neighbours; float4 lanes where nz % 4 == 0 and
 * the fields are 16-byte aligned), 2 (default) the same with the next plane
 * loaded ahead, 3 as 2 with a 64-register cap (more resident warps).  Items that meet a material box always run the ADE column
 * path. */
int sf_batch_set_kernel(sf_batch* batch, int kind);
/* Time the 9 item shapes (rows 4/8/16 x i_chunk 8/16/32) of the current
 * path on the members' current state without changing it and keep the
 * fastest; ms_out[9] may be NULL. */
int sf_batch_autotune(sf_batch* batch, int launches, void* stream, float* ms_out, int* best_rows,
                      int* best_chunk);
/* Advance every member by min(its remaining steps, n_steps).  graph_steps >
 * 0 captures that many steps as one CUDA graph and replays it. */
int sf_batch_run(sf_batch* batch, int64_t n_steps, int graph_steps, void* stream);

/* --- differentiable solve (reverse-time adjoint) ------------------------- */
/* A builder-defined extension with no counterpart in the reference (whose
 * density is a scalar, core/solver.py:1584-1586): per-cell density
 * rho = rho0 (1 + theta) with face coefficients
 * cv = -(dt/dx) (1/rho_lo + 1/rho_hi) / 2, K = rho0 c^2 fixed, PML decays and
 * a point source as the reference.  Rigid walls come from an optional air
 * mask (geometry: device, nx*ny*nz bytes, nonzero = air, as the reference's
 * set_geometry, core/solver.py:1682): a face that touches a solid cell has
 * cv = 0, so its velocity stays zero and a solid cell's pressure stays zero,
 * which is the reference's rigid pass (boundaries.cpp:66-89, p = 0 in
 * solids, fdtd_step.cpp:84-212) for a solve started from rest; such faces
 * carry no gradient.  The caller passes src_cell < 0 when the source cell is
 * solid (the reference injects into air cells only).  dtype 0 = float32,
 * 1 = float64, 2 = double-word float32 for every array below.  decay[3]:
 * device arrays of nx, ny, nz (1 where an axis has no PML).  src_cell < 0:
 * no source. */
typedef struct {
    int32_t nx, ny, nz, dtype;
    double cp;         /* -K dt / dx */
    double dt_over_dx; /* dt / dx */
    double rho0;
    const void* decay[3];
    int64_t src_cell;
    int32_t n_probe, reserved;
    const int64_t* probe_cells; /* device */
    const uint8_t* geometry;    /* device air mask, or NULL: no solids */
    /* device occupancy field phi (N values of the external type: float for
     * dtype 0, double otherwise), or NULL.  Each face coefficient is scaled
     * by the open fractions of its two cells, (1 - phi_lo)(1 - phi_hi): phi
     * = 1 closes every face of a cell (a rigid wall), phi in (0, 1) a
     * partly open one, so the solve is differentiable in the geometry. */
    const void* occupancy;
    /* Per axis a, the indices [unit_lo[a], unit_hi[a]) whose decay[a] is
     * exactly 1 together with both neighbours' (an index past either end
     * counts as 1); empty when unit_hi <= unit_lo, as a zero-filled
     * descriptor leaves it.  Blocks of cells inside all three ranges skip
     * their products with the decays, which changes no value (x * 1 == x
     * in every working type). */
    int32_t unit_lo[3], unit_hi[3];
} sf_diff_desc;
/* cv arrays (3 x N) from theta (N). */
int sf_diff_coefficients(const sf_diff_desc* d, const void* theta, void* cvx, void* cvy, void* cvz,
                         void* stream);
/* n_steps forward steps between two state sets (4 pointers each: p, vx,
 * vy, vz), starting from set `cur`; src_vals [n] (device, may be NULL; in
 * the working type: for dtype 2 each value as its nearest (hi, lo) float
 * pair, as the state arrays);
 * trace [n][n_probe] (may be NULL); p_store [n][N] receives each step's input
 * pressure (may be NULL). */
int sf_diff_forward(const sf_diff_desc* d, void* const* cv, void* const* set0, void* const* set1,
                    int cur, int64_t n_steps, const void* src_vals, void* trace, void* p_store,
                    void* stream);
/* Reverse-time adjoint of the same n_steps: lambda sets (4 pointers each),
 * starting from set `cur` holding lambda after the last step; p_store as
 * written by the forward; the probe-loss gradient weight*2*(trace-target)
 * is injected before each step's adjoint; dL/dcv accumulates into
 * grad_cv[3], three arrays of N 8-byte words, zero-filled by the caller (the
 * per-face sum runs over every step and cancels, so it keeps more precision
 * than the fields): doubles for dtype 1; for dtype 0 a pair of floats
 * (hi, lo) per face whose exact sum is the value, updated in double-word
 * arithmetic so that the FP32 adjoint needs no FP64 instruction. */
int sf_diff_adjoint(const sf_diff_desc* d, void* const* cv, void* const* lam0, void* const* lam1,
                    int cur, int64_t n_steps, const void* p_store, const void* trace,
                    const void* target, double weight, void* const* grad_cv, void* stream);
/* dL/dtheta (dtype) from dL/dcv (grad_cv as sf_diff_adjoint left it). */
int sf_diff_grad_theta(const sf_diff_desc* d, const void* theta, void* const* grad_cv, void* out,
                       void* stream);
/* dL/dtheta and, when out_occupancy is not NULL (it needs d->occupancy),
 * dL/dphi, both in the external type, from the same grad_cv. */
int sf_diff_grad_fields(const sf_diff_desc* d, const void* theta, void* const* grad_cv,
                        void* out_theta, void* out_occupancy, void* stream);

/* --- voxelisation -------------------------------------------------------- */
/* mask[i,j,k] = sdf(cell centre) <= 0, cell centre = (i + 0.5)*res, as
 * SDFPrimitive.voxelize (geometry/sdf.py:99-125) with grid coordinates
 * np.arange(n)*res + res/2 (core/grid.py:86-88).  invert != 0 stores the
 * complement (air = outside a solid).  out_dev: nx*ny*nz bytes. */
int sf_voxelize(const sf_sdf_node* nodes, int n_nodes, int nx, int ny, int nz, double res,
                int invert, uint8_t* out_dev, void* stream);
/* Same at the cell centres of a nonuniform grid: coords[3] host arrays of
 * nx, ny, nz doubles (NonuniformGrid.x/y/z_coords, core/grid.py:148-532). */
int sf_voxelize_coords(const sf_sdf_node* nodes, int n_nodes, int nx, int ny, int nz,
                       const double* const* coords, int invert, uint8_t* out_dev, void* stream);

/* Geometry and material ids voxelised in one pass, replacing
 * MaterializedGeometry.voxelize_with_materials
 * (geometry/material_assignment.py:133-171): program 0 (nodes[prog_off[0]
 * .. prog_off[1]-1]) is the geometry, whose inside is air (geom_dev = 1);
 * programs 1..n_regions are the material regions in assignment order, with
 * ids[0..n_regions-1].  mat_dev receives the id of the last region that
 * contains the cell centre, in air cells only, else 0.  coords: NULL for a
 * uniform grid of spacing res, else three host arrays of cell centres.
 * Both outputs are nx*ny*nz device bytes.  Synchronous. */
int sf_voxelize_materials(const sf_sdf_node* nodes, const int32_t* prog_off, int n_regions,
                          const uint8_t* ids, int nx, int ny, int nz, double res,
                          const double* const* coords, uint8_t* geom_dev, uint8_t* mat_dev,
                          void* stream);

/* Signed distance of the same program at n points (device doubles, n x 3,
 * row major) into out_dev[n]; replaces SDFPrimitive.sdf
 * (geometry/sdf.py:67-80).  Synchronous. */
int sf_sdf_eval(const sf_sdf_node* nodes, int n_nodes, const double* points_dev, int64_t n,
                double* out_dev, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SF_GB300_H */
