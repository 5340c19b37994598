// ref_harness.cpp -- extern "C" entry points over the reference's own native
// kernels (rjwalters/strata-fdtd, src/strata_fdtd/_kernels/src/*.cpp), so the
// oracle restatement can be checked against the reference bit for bit.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile from the reference
// sources where they lie (nothing of the reference is copied into this
// repository); the output goes to oracle/_ref/, which is not committed.
// Only tests/ and tests/golden/make_golden.py load the result.
#include <cstdint>
#include <cstring>
#include <vector>

#include "ade.hpp"
#include "boundaries.hpp"
#include "fdtd_step.hpp"
#include "fdtd_types.hpp"
#include "pml.hpp"

using namespace fdtd;

extern "C" {

// fdtd_step.cpp:15 update_velocity
void ref_update_velocity(const float* p, float* vx, float* vy, float* vz, int nx, int ny,
                         int nz, float cv) {
    update_velocity(p, vx, vy, vz, GridShape{nx, ny, nz}, cv);
}

// fdtd_step.cpp:84 update_pressure (geometry is a C++ bool array, 1 byte)
void ref_update_pressure(float* p, const float* vx, const float* vy, const float* vz,
                         const uint8_t* geom, int nx, int ny, int nz, float cp) {
    update_pressure(p, vx, vy, vz, reinterpret_cast<const bool*>(geom),
                    GridShape{nx, ny, nz}, cp);
}

// boundaries.cpp:13 precompute_boundary_cells, held as an opaque handle
void* ref_bc_create(const uint8_t* geom, int nx, int ny, int nz) {
    return new BoundaryCells(
        precompute_boundary_cells(reinterpret_cast<const bool*>(geom), GridShape{nx, ny, nz}));
}
int64_t ref_bc_list(void* h, int axis, int32_t* out) {
    auto* bc = static_cast<BoundaryCells*>(h);
    const std::vector<int>& v =
        axis == 0 ? bc->vx_indices : (axis == 1 ? bc->vy_indices : bc->vz_indices);
    if (out) std::memcpy(out, v.data(), v.size() * sizeof(int));
    return static_cast<int64_t>(v.size());
}
// boundaries.cpp:66 apply_rigid_boundaries
void ref_bc_apply(void* h, float* vx, float* vy, float* vz) {
    apply_rigid_boundaries(vx, vy, vz, *static_cast<BoundaryCells*>(h));
}
void ref_bc_destroy(void* h) { delete static_cast<BoundaryCells*>(h); }

// pml.cpp:13 initialize_pml (dt arrives as float, as through pybind)
void* ref_pml_create(const float* sx, const float* sy, const float* sz, int nx, int ny,
                     int nz, float dt) {
    return new PMLData(initialize_pml(sx, sy, sz, GridShape{nx, ny, nz}, dt));
}
int ref_pml_decay(void* h, int axis, float* out) {
    auto* pml = static_cast<PMLData*>(h);
    const std::vector<float>& v =
        axis == 0 ? pml->decay_x : (axis == 1 ? pml->decay_y : pml->decay_z);
    if (out) std::memcpy(out, v.data(), v.size() * sizeof(float));
    return static_cast<int>(v.size());
}
// pml.cpp:47 / :100
void ref_pml_velocity(void* h, float* vx, float* vy, float* vz, int nx, int ny, int nz) {
    apply_pml_velocity(vx, vy, vz, *static_cast<PMLData*>(h), GridShape{nx, ny, nz});
}
void ref_pml_pressure(void* h, float* p, int nx, int ny, int nz) {
    apply_pml_pressure(p, *static_cast<PMLData*>(h), GridShape{nx, ny, nz});
}
void ref_pml_destroy(void* h) { delete static_cast<PMLData*>(h); }

// ade.hpp:44 ADEMaterialData, filled the way solver.py:2996-3083 fills it
void* ref_ade_create(int n_materials_plus_one) {
    auto* d = new ADEMaterialData();
    d->rho_inf.assign(n_materials_plus_one, 0.0f);
    d->K_inf.assign(n_materials_plus_one, 0.0f);
    return d;
}
void ref_ade_set_material(void* h, int mat, float rho_inf, float K_inf) {
    auto* d = static_cast<ADEMaterialData*>(h);
    d->rho_inf[mat] = rho_inf;
    d->K_inf[mat] = K_inf;
}
void ref_ade_add_debye(void* h, int mat, int target, int field, float alpha, float beta) {
    auto* d = static_cast<ADEMaterialData*>(h);
    ADEMaterialData::DebyePole p;
    p.material_id = mat;
    p.target = target;
    p.field_index = field;
    p.coeffs.alpha = alpha;
    p.coeffs.beta = beta;
    d->debye_poles.push_back(p);
    d->n_debye_fields = field + 1 > d->n_debye_fields ? field + 1 : d->n_debye_fields;
}
void ref_ade_add_lorentz(void* h, int mat, int target, int field, float a, float b,
                         float dd) {
    auto* d = static_cast<ADEMaterialData*>(h);
    ADEMaterialData::LorentzPole p;
    p.material_id = mat;
    p.target = target;
    p.field_index = field;
    p.coeffs.a = a;
    p.coeffs.b = b;
    p.coeffs.d = dd;
    d->lorentz_poles.push_back(p);
    d->n_lorentz_fields = field + 1 > d->n_lorentz_fields ? field + 1 : d->n_lorentz_fields;
}
void ref_ade_destroy(void* h) { delete static_cast<ADEMaterialData*>(h); }

// ade.cpp:25 / :70 / :118 / :172
void ref_ade_density_debye(float* J, const float* p, const uint8_t* mat, void* h, int nx,
                           int ny, int nz) {
    update_ade_density_debye(J, p, mat, *static_cast<ADEMaterialData*>(h),
                             GridShape{nx, ny, nz});
}
void ref_ade_modulus_debye(float* J, const float* div, const uint8_t* mat, void* h, int nx,
                           int ny, int nz) {
    update_ade_modulus_debye(J, div, mat, *static_cast<ADEMaterialData*>(h),
                             GridShape{nx, ny, nz});
}
void ref_ade_density_lorentz(float* J, float* Jp, const float* p, const uint8_t* mat,
                             void* h, int nx, int ny, int nz) {
    update_ade_density_lorentz(J, Jp, p, mat, *static_cast<ADEMaterialData*>(h),
                               GridShape{nx, ny, nz});
}
void ref_ade_modulus_lorentz(float* J, float* Jp, const float* div, const uint8_t* mat,
                             void* h, int nx, int ny, int nz) {
    update_ade_modulus_lorentz(J, Jp, div, mat, *static_cast<ADEMaterialData*>(h),
                               GridShape{nx, ny, nz});
}
// ade.cpp:228 / :403 / :479
void ref_ade_velocity_correction(float* vx, float* vy, float* vz, const float* Jd,
                                 const float* Jl, const uint8_t* mat, void* h, int nx,
                                 int ny, int nz, float dt, float inv_dx) {
    apply_ade_velocity_correction(vx, vy, vz, Jd, Jl, mat, *static_cast<ADEMaterialData*>(h),
                                  GridShape{nx, ny, nz}, dt, inv_dx);
}
void ref_ade_pressure_correction(float* p, const float* Jd, const float* Jl,
                                 const uint8_t* mat, void* h, int nx, int ny, int nz,
                                 float dt) {
    apply_ade_pressure_correction(p, Jd, Jl, mat, *static_cast<ADEMaterialData*>(h),
                                  GridShape{nx, ny, nz}, dt);
}
void ref_compute_divergence(float* div, const float* vx, const float* vy, const float* vz,
                            int nx, int ny, int nz, float inv_dx) {
    compute_divergence(div, vx, vy, vz, GridShape{nx, ny, nz}, inv_dx);
}

}  // extern "C"
