// sf_common.cuh -- shared device helpers and plan layout for the GB300 path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "sf_gb300.h"

// Rounded FP32 / FP64 operations.  The intrinsics are never contracted into
// a fused multiply-add, which bit-exact parity with the reference (built
// without FMA) requires.  The build also passes -fmad=false.
__device__ __forceinline__ float f_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float f_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float f_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double d_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double d_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double d_mul(double a, double b) { return __dmul_rn(a, b); }

// One face velocity: v + cv*(p_hi - p_lo) (fdtd_step.cpp:44,61,78).
__device__ __forceinline__ float face_update(float v, float cv, float p_hi, float p_lo) {
    return f_add(v, f_mul(cv, f_sub(p_hi, p_lo)));
}

// Per-cell flag byte built from the geometry mask by sf_plan_set_geometry.
//   bit 0: cell is air
//   bit 1/2/3: the +x/+y/+z face of the cell joins two air cells (open)
// A face whose bit is clear is held at zero velocity (rigid wall), the rule
// of precompute_boundary_cells (boundaries.cpp:13-64).
enum : uint8_t { SF_AIR = 1, SF_OPX = 2, SF_OPY = 4, SF_OPZ = 8, SF_ALL = 15 };

struct SfSources {
    int n;
    sf_source s[SF_MAX_SOURCES];
};

struct SfPoles {
    int n;            // poles, Debye first then Lorentz (reference field order)
    int n_density;    // how many have target == density
    int n_modulus;
    float inv_dx;
    sf_pole p[SF_MAX_POLES];
};

// Everything one launch of the step kernel needs for one grid.
struct SfStepArgs {
    int nx, ny, nz;
    long long plane;  // ny*nz
    float cv, cp;
    const float* __restrict__ p;
    const float* __restrict__ vx;
    const float* __restrict__ vy;
    const float* __restrict__ vz;
    float* __restrict__ po;
    float* __restrict__ vxo;
    float* __restrict__ vyo;
    float* __restrict__ vzo;
    const uint8_t* __restrict__ flags;  // null: every cell air, every face open
    const float* __restrict__ dx;       // PML decays, 1.0f where an axis is off
    const float* __restrict__ dy;
    const float* __restrict__ dz;
    const double* __restrict__ src_val;  // this step's waveform values [n_src]
    int n_probe;
    const long long* __restrict__ probe_cells;
    float* __restrict__ trace_prev;  // probe values of the input state, or null
    const uint8_t* __restrict__ mat;  // ADE material ids (ADE kernels only)
    int reverse;                      // column kernels: dispatch i-chunks high to low
    int ade_lo[3], ade_hi[3];         // box holding every material cell
    int reg_lo[3], reg_hi[3];         // per-cell kernel: the cells it updates
    int skip_lo[3], skip_hi[3];       // warp-tile kernels: tile-aligned cells they leave out
    const float* nu_cv[3];            // nonuniform grid: face coefficients per axis, or null
    const float* nu_inv[3];           // nonuniform grid: cell inverse spacings per axis
};

#define SF_CUDA_OK(expr)                                                   \
    do {                                                                   \
        cudaError_t e_ = (expr);                                           \
        if (e_ != cudaSuccess) return sf_fail_cuda(e_, #expr, __FILE__, __LINE__); \
    } while (0)

int sf_fail(const char* msg);
int sf_fail_cuda(cudaError_t e, const char* what, const char* file, int line);
