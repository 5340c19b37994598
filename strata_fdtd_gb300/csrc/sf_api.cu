// sf_api.cu -- the extern "C" boundary declared in include/sf_gb300.h.
//
// Host-side plan management.  A plan describes one grid: its coefficients,
// the caller's two ping-pong field sets, and the small device tables it owns
// (face flags, PML decays, probe cells).  sf_plan_step enqueues one fused
// kernel per time step on the caller's stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "sf_common.cuh"

#ifndef SF_VERSION_STRING
#define SF_VERSION_STRING "0.1.0"
#endif

#include "sf_kernels.h"

// Step-kernel configuration used when the plan has not been autotuned.
#ifndef SF_CFG_DEFAULT
#define SF_CFG_DEFAULT (SF_CFG_COL_FIRST + 0)
#define SF_CFG_TILE_FIRST (SF_CFG_COL_FIRST + kSfColConfigCount)
#define SF_CFG_TILE_DEFAULT (SF_CFG_TILE_FIRST + 2)
#define SF_CFG_TILE1_DEFAULT (SF_CFG_TILE_FIRST + 11)
#define SF_CFG_PIPE_FIRST (SF_CFG_TILE_FIRST + kSfTileConfigCount)
#define SF_CFG_TB_FIRST (SF_CFG_PIPE_FIRST + kSfPipeConfigCount)
#endif

namespace {
thread_local std::string g_err;
}

int sf_fail(const char* msg) {
    g_err = msg;
    return 1;
}

int sf_fail_cuda(cudaError_t e, const char* what, const char* file, int line) {
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file,
                  line);
    g_err = buf;
    return 2;
}

#include "sf_plan_internal.h"

int sf_noalloc_setup(int dev);  // defined with the no-alloc energy array below

// Deferred device frees.  cudaFree waits for all work on the device, so a
// plan or a batch released while other solves' kernels run would stall the
// host until they finish (a served stream retires and builds solves while
// the next group runs).  The buffers of destroyed plans and batches and the
// batches' graphs are queued here instead and released together once 1 GiB
// or 4096 entries have accumulated, or by sf_release_deferred().
namespace {
struct SfDeferred {
    int device;
    void* ptr;
    cudaGraphExec_t exec;
    cudaGraph_t graph;
};
std::mutex g_def_mu;
std::vector<SfDeferred> g_def;
size_t g_def_bytes = 0;
constexpr size_t kDeferredBytes = size_t(1) << 30, kDeferredCount = 4096;

void release_deferred_locked() {
    for (const SfDeferred& d : g_def) {
        DeviceGuard g(d.device);
        if (d.exec) cudaGraphExecDestroy(d.exec);
        if (d.graph) cudaGraphDestroy(d.graph);
        if (d.ptr) cudaFree(d.ptr);
    }
    g_def.clear();
    g_def_bytes = 0;
}

void defer_push(const SfDeferred& d, size_t bytes) {
    std::lock_guard<std::mutex> lock(g_def_mu);
    g_def.push_back(d);
    g_def_bytes += bytes;
    if (g_def_bytes >= kDeferredBytes || g_def.size() >= kDeferredCount) release_deferred_locked();
}
}  // namespace

void sf_defer_free(void* p, size_t bytes) {
    if (!p) return;
    int dev = 0;
    cudaGetDevice(&dev);
    defer_push({dev, p, nullptr, nullptr}, bytes);
}

void sf_defer_graph(cudaGraphExec_t exec, cudaGraph_t graph) {
    if (!exec && !graph) return;
    int dev = 0;
    cudaGetDevice(&dev);
    defer_push({dev, nullptr, exec, graph}, 0);
}

extern "C" int sf_release_deferred(void) {
    std::lock_guard<std::mutex> lock(g_def_mu);
    release_deferred_locked();
    return 0;
}

namespace {

int set_decays(sf_plan* P, const float* host[3]) {
    const int n[3] = {P->d.nx, P->d.ny, P->d.nz};
    for (int a = 0; a < 3; ++a) {
        std::vector<float> h(n[a], 1.0f);
        if (host[a]) std::memcpy(h.data(), host[a], sizeof(float) * n[a]);
        SF_CUDA_OK(cudaMemcpy(P->decay[a], h.data(), sizeof(float) * n[a], cudaMemcpyHostToDevice));
    }
    return 0;
}



}  // namespace

extern "C" {

const char* sf_version(void) {
    return "strata_fdtd_gb300 " SF_VERSION_STRING " (sm_103a, abi " "1" ")";
}

const char* sf_last_error(void) { return g_err.c_str(); }

int sf_device_info(int device, sf_device_info_t* out) {
    if (!out) return sf_fail("sf_device_info: out is NULL");
    cudaDeviceProp pr;
    SF_CUDA_OK(cudaGetDeviceProperties(&pr, device));
    std::memset(out, 0, sizeof(*out));
    out->device = device;
    out->sm_count = pr.multiProcessorCount;
    out->cc_major = pr.major;
    out->cc_minor = pr.minor;
    out->total_mem = (int64_t)pr.totalGlobalMem;
    out->l2_bytes = pr.l2CacheSize;
    out->max_smem_per_block = (int32_t)pr.sharedMemPerBlockOptin;
    std::strncpy(out->name, pr.name, sizeof(out->name) - 1);
    return 0;
}

int sf_plan_create(const sf_grid_desc* desc, sf_plan** out) {
    if (!desc || !out) return sf_fail("sf_plan_create: NULL argument");
    if (desc->nx < 1 || desc->ny < 1 || desc->nz < 1)
        return sf_fail("sf_plan_create: grid dimensions must be >= 1");
    if (desc->nx > 65535) return sf_fail("sf_plan_create: nx > 65535 is not supported");
    auto* P = new sf_plan();
    P->d = *desc;
    P->n = (long long)desc->nx * desc->ny * desc->nz;
    P->ade_hi[0] = desc->nx;
    P->ade_hi[1] = desc->ny;
    P->ade_hi[2] = desc->nz;
    cudaGetDevice(&P->device);
    if (cudaDeviceGetAttribute(&P->sms, cudaDevAttrMultiProcessorCount, P->device) != cudaSuccess ||
        P->sms < 1) {
        delete P;
        return sf_fail("sf_plan_create: cannot query the device's SM count");
    }
    if (int rc = sf_noalloc_setup(P->device)) {
        delete P;
        return rc;
    }
    const int n[3] = {desc->nx, desc->ny, desc->nz};
    for (int a = 0; a < 3; ++a) {
        if (cudaMalloc(&P->decay[a], sizeof(float) * n[a]) != cudaSuccess) {
            sf_plan_destroy(P);
            return sf_fail("sf_plan_create: cudaMalloc of PML tables failed");
        }
    }
    const float* none[3] = {nullptr, nullptr, nullptr};
    if (int rc = set_decays(P, none)) {
        sf_plan_destroy(P);
        return rc;
    }
    *out = P;
    return 0;
}

int sf_plan_destroy(sf_plan* P) {
    if (!P) return 0;
    DeviceGuard g(P->device);
    for (auto& d : P->decay) sf_defer_free(d, 0);
    sf_defer_free(P->flags, (size_t)P->n);
    sf_defer_free(P->probe_cells, 0);
    sf_defer_free(P->mic_idx, 0);
    sf_defer_free(P->mic_w, 0);
    sf_defer_free(P->mic_field, 0);
    sf_defer_free(P->nu, 0);
    sf_defer_free(P->plane_prev, 0);
    for (int q = 0; q < SF_MAX_SOURCES; ++q) {
        sf_defer_free(P->wsrc_cells[q], 0);
        sf_defer_free(P->wsrc_w[q], 0);
    }
    sf_defer_free(P->pipe_ring, P->pipe_ring_floats * sizeof(float));
    sf_defer_free(P->pipe_ctrl, 0);
    sf_defer_free(P->pipe_err, 0);
    sf_defer_free(P->pipe_order, 0);
    delete P;
    return 0;
}

int sf_plan_bind_fields(sf_plan* P, float* p0, float* vx0, float* vy0, float* vz0, float* p1,
                        float* vx1, float* vy1, float* vz1) {
    if (!P) return sf_fail("sf_plan_bind_fields: NULL plan");
    float* all[8] = {p0, vx0, vy0, vz0, p1, vx1, vy1, vz1};
    for (int q = 0; q < 8; ++q) {
        if (!all[q]) return sf_fail("sf_plan_bind_fields: NULL field buffer");
        if (reinterpret_cast<uintptr_t>(all[q]) % 16 != 0)
            return sf_fail("sf_plan_bind_fields: field buffers must be 16-byte aligned");
        P->f[q / 4][q % 4] = all[q];
    }
    P->bound = true;
    P->cur = 0;
    return 0;
}

int sf_plan_current(const sf_plan* P) { return P ? P->cur : -1; }

int sf_plan_set_current(sf_plan* P, int which) {
    if (!P || (which != 0 && which != 1)) return sf_fail("sf_plan_set_current: bad argument");
    P->cur = which;
    return 0;
}

int sf_plan_set_geometry(sf_plan* P, const uint8_t* geom, void* stream) {
    if (!P) return sf_fail("sf_plan_set_geometry: NULL plan");
    DeviceGuard g(P->device);
    if (!geom) {
        cudaFree(P->flags);
        P->flags = nullptr;
        return 0;
    }
    if (!P->flags) SF_CUDA_OK(cudaMalloc(&P->flags, (size_t)P->n));
    return sf_launch_build_flags(geom, P->flags, P->d.nx, P->d.ny, P->d.nz,
                                 static_cast<cudaStream_t>(stream));
}

int sf_plan_set_pml(sf_plan* P, const float* sx, const float* sy, const float* sz, float dt) {
    if (!P) return sf_fail("sf_plan_set_pml: NULL plan");
    DeviceGuard g(P->device);
    const int n[3] = {P->d.nx, P->d.ny, P->d.nz};
    const float* sig[3] = {sx, sy, sz};
    std::vector<float> dec[3];
    const float* host[3] = {nullptr, nullptr, nullptr};
    for (int a = 0; a < 3; ++a) {
        if (!sig[a]) continue;
        dec[a].resize(n[a]);
        // pml.cpp:13-45: std::exp on float arguments, dt already a float
        for (int q = 0; q < n[a]; ++q) dec[a][q] = std::exp(-sig[a][q] * dt);
        host[a] = dec[a].data();
    }
    return set_decays(P, host);
}

int sf_plan_set_nonuniform(sf_plan* P, const float* const* cv_face, const float* const* inv_cell) {
    if (!P) return sf_fail("sf_plan_set_nonuniform: NULL plan");
    DeviceGuard g(P->device);
    cudaFree(P->nu);
    P->nu = nullptr;
    if (!cv_face && !inv_cell) return 0;  // back to a uniform grid
    if (!cv_face || !inv_cell) return sf_fail("sf_plan_set_nonuniform: need both tables");
    for (int a = 0; a < 3; ++a)
        if (!cv_face[a] || !inv_cell[a]) return sf_fail("sf_plan_set_nonuniform: NULL axis table");
    const int n[3] = {P->d.nx, P->d.ny, P->d.nz};
    const long long total = 2LL * (n[0] + n[1] + n[2]);
    SF_CUDA_OK(cudaMalloc(&P->nu, sizeof(float) * total));
    const float* const* tables[2] = {cv_face, inv_cell};
    long long off = 0;
    for (int t = 0; t < 2; ++t)
        for (int a = 0; a < 3; ++a) {
            SF_CUDA_OK(cudaMemcpy(P->nu + off, tables[t][a], sizeof(float) * n[a],
                                  cudaMemcpyHostToDevice));
            off += n[a];
        }
    P->tuned = 0;  // the autotuner's choice was made for the other arithmetic
    P->tuned_ich = 0;
    return 0;
}

int sf_plan_set_weighted_source(sf_plan* P, int slot, int64_t n, const int64_t* cells,
                                const double* weights) {
    if (!P) return sf_fail("sf_plan_set_weighted_source: NULL plan");
    if (slot < 0 || slot >= SF_MAX_SOURCES || n < 0 || (n > 0 && (!cells || !weights)))
        return sf_fail("sf_plan_set_weighted_source: bad slot or table");
    for (int64_t q = 0; q < n; ++q)
        if (cells[q] < 0 || cells[q] >= P->n)
            return sf_fail("sf_plan_set_weighted_source: cell outside the grid");
    DeviceGuard g(P->device);
    cudaFree(P->wsrc_cells[slot]);
    cudaFree(P->wsrc_w[slot]);
    P->wsrc_cells[slot] = nullptr;
    P->wsrc_w[slot] = nullptr;
    P->wsrc_n[slot] = 0;
    if (n == 0) return 0;
    SF_CUDA_OK(cudaMalloc(&P->wsrc_cells[slot], sizeof(long long) * n));
    SF_CUDA_OK(cudaMalloc(&P->wsrc_w[slot], sizeof(double) * n));
    SF_CUDA_OK(cudaMemcpy(P->wsrc_cells[slot], cells, sizeof(long long) * n, cudaMemcpyHostToDevice));
    SF_CUDA_OK(cudaMemcpy(P->wsrc_w[slot], weights, sizeof(double) * n, cudaMemcpyHostToDevice));
    P->wsrc_n[slot] = n;
    return 0;
}

int sf_plan_set_plane_boundaries(sf_plan* P, int n, const sf_plane_bc* ops) {
    if (!P) return sf_fail("sf_plan_set_plane_boundaries: NULL plan");
    if (n < 0 || n > SF_MAX_PLANE_OPS || (n > 0 && !ops))
        return sf_fail("sf_plan_set_plane_boundaries: at most 8 operations");
    const int dims[3] = {P->d.nx, P->d.ny, P->d.nz};
    long long total = 0;
    long long off[SF_MAX_PLANE_OPS][2];
    for (int q = 0; q < n; ++q) {
        const sf_plane_bc& o = ops[q];
        if ((o.kind != 0 && o.kind != 1) || o.axis < 0 || o.axis > 2 ||
            (o.kind == 1 && o.side != 0 && o.side != 1))
            return sf_fail("sf_plan_set_plane_boundaries: bad operation");
        if (dims[o.axis] < 2)
            return sf_fail("sf_plan_set_plane_boundaries: the axis needs at least 2 cells");
        const long long plane = (long long)(o.axis == 0 ? dims[1] : dims[0]) *
                                (o.axis == 2 ? dims[1] : dims[2]);
        off[q][0] = total;
        total += plane;
        off[q][1] = total;
        if (o.kind == 0) total += plane;  // Mur keeps both ends
    }
    DeviceGuard g(P->device);
    cudaFree(P->plane_prev);
    P->plane_prev = nullptr;
    P->n_plane = 0;
    if (n == 0) return 0;
    SF_CUDA_OK(cudaMalloc(&P->plane_prev, sizeof(float) * total));
    SF_CUDA_OK(cudaMemset(P->plane_prev, 0, sizeof(float) * total));
    for (int q = 0; q < n; ++q) {
        P->plane_ops[q] = ops[q];
        P->plane_off[q][0] = off[q][0];
        P->plane_off[q][1] = off[q][1];
    }
    P->n_plane = n;
    return 0;
}

int sf_plan_set_pml_decay(sf_plan* P, const float* dx, const float* dy, const float* dz) {
    if (!P) return sf_fail("sf_plan_set_pml_decay: NULL plan");
    DeviceGuard g(P->device);
    const float* host[3] = {dx, dy, dz};
    return set_decays(P, host);
}

int sf_plan_set_sources(sf_plan* P, int n, const sf_source* s) {
    if (!P) return sf_fail("sf_plan_set_sources: NULL plan");
    if (n < 0 || n > SF_MAX_SOURCES) return sf_fail("sf_plan_set_sources: at most 16 sources");
    if (n > 0 && !s) return sf_fail("sf_plan_set_sources: NULL source table");
    const int dims[3] = {P->d.nx, P->d.ny, P->d.nz};
    for (int q = 0; q < n; ++q) {
        if (s[q].kind == 0) {
            if (s[q].a < 0 || s[q].a >= dims[0] || s[q].b < 0 || s[q].b >= dims[1] ||
                s[q].c < 0 || s[q].c >= dims[2])
                return sf_fail("sf_plan_set_sources: point source outside the grid");
        } else if (s[q].kind == 1) {
            if (s[q].a < 0 || s[q].a > 2 || s[q].b < 0 || s[q].b >= dims[s[q].a])
                return sf_fail("sf_plan_set_sources: plane source outside the grid");
        } else if (s[q].kind == 2) {
            if (s[q].a < 0 || s[q].a >= SF_MAX_SOURCES || s[q].b < 0 || s[q].b > 3)
                return sf_fail("sf_plan_set_sources: weighted source needs a slot and a field");
        } else {
            return sf_fail("sf_plan_set_sources: kind must be 0 (point), 1 (plane) or 2 (weighted)");
        }
    }
    P->src.n = n;
    for (int q = 0; q < n; ++q) P->src.s[q] = s[q];
    return 0;
}

int sf_plan_set_probes(sf_plan* P, int n, const int64_t* cells) {
    if (!P) return sf_fail("sf_plan_set_probes: NULL plan");
    if (n < 0 || (n > 0 && !cells)) return sf_fail("sf_plan_set_probes: bad probe table");
    for (int q = 0; q < n; ++q)
        if (cells[q] < 0 || cells[q] >= P->n) return sf_fail("sf_plan_set_probes: cell outside the grid");
    DeviceGuard g(P->device);
    cudaFree(P->probe_cells);
    P->probe_cells = nullptr;
    P->n_probe = n;
    P->probe_tile_max = 0;
    if (n == 0) return 0;
    {  // probes per 32 k x 4 row tile column (the streaming pipeline holds at most 32)
        const long long plane = (long long)P->d.ny * P->d.nz;
        std::vector<long long> key(n);
        for (int q = 0; q < n; ++q) {
            const long long rem = cells[q] % plane;
            key[q] = (rem / P->d.nz) / 4 * ((P->d.nz + 31) / 32) + (rem % P->d.nz) / 32;
        }
        std::sort(key.begin(), key.end());
        for (int q = 0, run = 0; q < n; ++q) {
            run = (q > 0 && key[q] == key[q - 1]) ? run + 1 : 1;
            if (run > P->probe_tile_max) P->probe_tile_max = run;
        }
    }
    SF_CUDA_OK(cudaMalloc(&P->probe_cells, sizeof(long long) * n));
    SF_CUDA_OK(cudaMemcpy(P->probe_cells, cells, sizeof(long long) * n, cudaMemcpyHostToDevice));
    return 0;
}

int sf_plan_set_ade(sf_plan* P, const uint8_t* mat, int n, const sf_pole* poles, float inv_dx) {
    if (!P) return sf_fail("sf_plan_set_ade: NULL plan");
    if (n < 0 || n > SF_MAX_POLES) return sf_fail("sf_plan_set_ade: at most 16 poles");
    if (n > 0 && (!mat || !poles)) return sf_fail("sf_plan_set_ade: NULL material ids or poles");
    SfPoles T{};
    T.inv_dx = inv_dx;
    for (int q = 0; q < n; ++q) {
        const sf_pole& pl = poles[q];
        if (pl.kind != 0 && pl.kind != 1) return sf_fail("sf_plan_set_ade: bad pole kind");
        if (pl.target != 0 && pl.target != 1) return sf_fail("sf_plan_set_ade: bad pole target");
        if (pl.material_id < 1 || pl.material_id > 255)
            return sf_fail("sf_plan_set_ade: material id must be 1..255");
        if (!pl.J || (pl.kind == 1 && !pl.J_prev))
            return sf_fail("sf_plan_set_ade: missing auxiliary field buffer");
        if (q > 0 && poles[q - 1].kind == 1 && pl.kind == 0)
            return sf_fail("sf_plan_set_ade: Debye poles must precede Lorentz poles");
        T.p[q] = pl;
        if (pl.target == 0) ++T.n_density; else ++T.n_modulus;
    }
    T.n = n;
    P->poles = T;
    P->mat = n > 0 ? mat : nullptr;
    return 0;
}

int sf_plan_set_ade_box(sf_plan* P, const int32_t* lo, const int32_t* hi) {
    if (!P || !lo || !hi) return sf_fail("sf_plan_set_ade_box: NULL argument");
    const int n[3] = {P->d.nx, P->d.ny, P->d.nz};
    for (int a = 0; a < 3; ++a)
        if (lo[a] < 0 || hi[a] > n[a] || lo[a] > hi[a])
            return sf_fail("sf_plan_set_ade_box: box outside the grid");
    for (int a = 0; a < 3; ++a) {
        P->ade_lo[a] = lo[a];
        P->ade_hi[a] = hi[a];
    }
    return 0;
}

int sf_plan_set_kernel(sf_plan* P, int config, int i_chunk) {
    if (!P) return sf_fail("sf_plan_set_kernel: NULL plan");
    if (config < 0 || config >= sf_kernel_config_count())
        return sf_fail("sf_plan_set_kernel: unknown kernel configuration");
    if (i_chunk < 0) return sf_fail("sf_plan_set_kernel: negative i_chunk");
    P->variant = config;
    P->i_chunk = i_chunk;
    return 0;
}

int sf_plan_set_wait_limit(sf_plan* P, int64_t spins, int hold_first_item) {
    if (!P) return sf_fail("sf_plan_set_wait_limit: NULL plan");
    if (spins < 0) return sf_fail("sf_plan_set_wait_limit: negative limit");
    P->pipe_spin_limit = spins;
    P->pipe_hold = hold_first_item != 0;
    return 0;
}

int sf_kernel_config_count(void) {
    return SF_CFG_COL_FIRST + kSfColConfigCount + kSfTileConfigCount + kSfPipeConfigCount +
           kSfTbConfigCount;
}

const char* sf_kernel_config_name(int config) {
    if (config == SF_CFG_AUTO) return "auto";
    if (config == SF_CFG_CELL) return "cell";
    if (config == SF_CFG_MARCH) return "march";
    if (config >= SF_CFG_COL_FIRST && config < SF_CFG_COL_FIRST + kSfColConfigCount)
        return kSfColConfigs[config - SF_CFG_COL_FIRST].name;
    if (config >= SF_CFG_TILE_FIRST && config < SF_CFG_PIPE_FIRST)
        return kSfTileConfigs[config - SF_CFG_TILE_FIRST].name;
    if (config >= SF_CFG_PIPE_FIRST && config < SF_CFG_TB_FIRST)
        return kSfPipeConfigs[config - SF_CFG_PIPE_FIRST].name;
    if (config >= SF_CFG_TB_FIRST && config < sf_kernel_config_count())
        return kSfTbConfigs[config - SF_CFG_TB_FIRST].name;
    return nullptr;
}

}  // extern "C"

namespace {

void fill_args(const sf_plan* P, SfStepArgs& a, bool with_trace) {
    a = SfStepArgs{};
    a.nx = P->d.nx;
    a.ny = P->d.ny;
    a.nz = P->d.nz;
    a.plane = (long long)P->d.ny * P->d.nz;
    a.cv = P->d.coeff_v;
    a.cp = P->d.coeff_p;
    a.flags = P->flags;
    a.dx = P->decay[0];
    a.dy = P->decay[1];
    a.dz = P->decay[2];
    a.n_probe = with_trace ? P->n_probe : 0;
    a.probe_cells = P->probe_cells;
    a.mat = P->mat;
    const int n3[3] = {P->d.nx, P->d.ny, P->d.nz};
    for (int q = 0; q < 3; ++q) {
        a.ade_lo[q] = P->ade_lo[q];
        a.ade_hi[q] = P->ade_hi[q];
        a.reg_lo[q] = 0;  // the per-cell kernel covers the grid
        a.reg_hi[q] = n3[q];
        a.skip_lo[q] = a.skip_hi[q] = 0;  // the warp-tile kernels skip nothing
        a.nu_cv[q] = a.nu_inv[q] = nullptr;
    }
    if (P->nu) {
        long long off = 0;
        for (int q = 0; q < 3; off += n3[q], ++q) a.nu_cv[q] = P->nu + off;
        for (int q = 0; q < 3; off += n3[q], ++q) a.nu_inv[q] = P->nu + off;
    }
}

void set_io(const sf_plan* P, SfStepArgs& a, int in) {
    const int out = 1 - in;
    a.p = P->f[in][0];
    a.vx = P->f[in][1];
    a.vy = P->f[in][2];
    a.vz = P->f[in][3];
    a.po = P->f[out][0];
    a.vxo = P->f[out][1];
    a.vyo = P->f[out][2];
    a.vzo = P->f[out][3];
}

// The configuration a step of this plan runs: the explicit choice, else the
// autotuned one, else the default warp-tile configuration where the grid
// allows it (nz % 4 == 0, aligned fields, 32-bit offsets), else the first
// column configuration.  With ADE poles only the warp-tile configurations
// (which then leave the material box to the per-cell kernel, see
// ade_region) and the per-cell kernel itself are used.
bool is_pipe(int cfg) { return cfg >= SF_CFG_PIPE_FIRST && cfg < SF_CFG_TB_FIRST; }
bool is_tb(int cfg) { return cfg >= SF_CFG_TB_FIRST; }
// The two-step kernels take uniform grids without ADE poles.
bool tb_fits(const sf_plan* P, const SfStepArgs& a) {
    return P->poles.n == 0 && P->nu == nullptr && sf_tb_supported(a);
}
int default_single(const SfStepArgs& a) {
    return sf_tile_supported(a, 4) ? SF_CFG_TILE_DEFAULT
                                   : (sf_tile_supported(a, 1) ? SF_CFG_TILE1_DEFAULT : SF_CFG_DEFAULT);
}
bool pipe_fits(sf_plan* P, int cfg, const SfStepArgs& a);
int chunk_for(const sf_plan* P, int cfg);

int effective_config(const sf_plan* P, const SfStepArgs& a) {
    int cfg;
    if (P->variant != SF_CFG_AUTO) cfg = P->variant;
    else if (P->tuned > 0) cfg = P->tuned;
    else if (sf_tile_supported(a, 4)) cfg = SF_CFG_TILE_DEFAULT;
    else cfg = sf_tile_supported(a, 1) ? SF_CFG_TILE1_DEFAULT : SF_CFG_DEFAULT;
    if (is_pipe(cfg)) {  // when the pipeline fits the plan; else the default choice
        if (pipe_fits(const_cast<sf_plan*>(P), cfg, a)) return cfg;
        cfg = default_single(a);
    }
    if (is_tb(cfg)) {  // likewise for the two-step kernels
        if (tb_fits(P, a)) return cfg;
        cfg = default_single(a);
    }
    const bool tile_ok =
        cfg >= SF_CFG_TILE_FIRST && sf_tile_supported(a, kSfTileConfigs[cfg - SF_CFG_TILE_FIRST].vec);
    if (P->nu && !tile_ok && cfg != SF_CFG_CELL)  // nonuniform: warp tiles or per-cell only
        cfg = sf_tile_supported(a, 4) ? SF_CFG_TILE_DEFAULT : SF_CFG_TILE1_DEFAULT;
    else if (P->poles.n > 0 && !tile_ok)
        cfg = SF_CFG_CELL;
    return cfg;
}

// The cells an ADE step gives to the per-cell kernel when warp-tile
// configuration cfg (i-chunk ich) runs the rest: the material box grown by
// one cell (the faces the ADE terms touch) and rounded out to whole tiles of
// that configuration.  Outside it no cell and no face carries an ADE term
// (both cells of a corrected face lie in one material), so the warp-tile
// kernel's plain arithmetic is the reference's there.  Empty when the plan
// has no material cells.
void ade_region(const sf_plan* P, int cfg, int ich, int lo[3], int hi[3]) {
    const SfTileConfig& t = kSfTileConfigs[cfg - SF_CFG_TILE_FIRST];
    const int n3[3] = {P->d.nx, P->d.ny, P->d.nz};
    const int span[3] = {ich, t.vec == 4 ? 4 * t.rows * t.warps : t.rows * t.warps, 32};
    bool empty = false;
    for (int q = 0; q < 3; ++q) empty = empty || P->ade_hi[q] <= P->ade_lo[q];
    for (int q = 0; q < 3; ++q) {
        if (empty) {
            lo[q] = hi[q] = 0;
            continue;
        }
        const int l = P->ade_lo[q] > 0 ? P->ade_lo[q] - 1 : 0;
        const int h = P->ade_hi[q] < n3[q] ? P->ade_hi[q] + 1 : n3[q];
        lo[q] = l / span[q] * span[q];
        hi[q] = (h + span[q] - 1) / span[q] * span[q];
        if (hi[q] > n3[q]) hi[q] = n3[q];
    }
}


int chunk_for(const sf_plan* P, int cfg) {
    if (P->i_chunk > 0) return P->i_chunk;
    if (cfg == P->tuned && P->tuned_ich > 0) return P->tuned_ich;
    if (is_pipe(cfg))  // planes per chunk / between progress updates
        return kSfPipeConfigs[cfg - SF_CFG_PIPE_FIRST].stream ? 4 : 2;
    if (is_tb(cfg)) {  // about four waves of blocks, chunks of at least 4 planes
        const SfTbConfig& c = kSfTbConfigs[cfg - SF_CFG_TB_FIRST];
        int sms = 152;
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess)
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const long long tiles = (long long)((P->d.nz + 27) / 28) *
                                ((P->d.ny + c.rows * c.warps - 1) / (c.rows * c.warps));
        long long chunks = (4LL * c.minb * sms + tiles - 1) / tiles;
        if (chunks < 1) chunks = 1;
        long long ich = (P->d.nx + chunks - 1) / chunks;
        if (ich < 4) ich = 4;
        if (ich > P->d.nx) ich = P->d.nx;
        return (int)ich;
    }
    if (cfg >= SF_CFG_TILE_FIRST) {
        const SfTileConfig& t = kSfTileConfigs[cfg - SF_CFG_TILE_FIRST];
        if (t.vec == 1) return auto_chunk(P, 32, t.rows * t.warps);
        if (P->d.nz % 4 == 0) return auto_chunk(P, 32, 4 * t.rows * t.warps);
        return auto_chunk(P, 32);
    }
    int kspan = 32;
    if (cfg >= SF_CFG_COL_FIRST) {
        const int vec = kSfColConfigs[cfg - SF_CFG_COL_FIRST].vec;
        if (P->d.nz % vec == 0) kspan = 32 * vec;
    }
    return auto_chunk(P, kspan);
}

// Whether configuration cfg runs as itself on this plan's grid (otherwise
// its launcher substitutes the first column configuration).
bool config_native(const sf_plan* P, int cfg, const SfStepArgs& a) {
    if (is_pipe(cfg)) return pipe_fits(const_cast<sf_plan*>(P), cfg, a);
    if (is_tb(cfg)) return tb_fits(P, a);
    if (cfg >= SF_CFG_TILE_FIRST)
        return sf_tile_supported(a, kSfTileConfigs[cfg - SF_CFG_TILE_FIRST].vec);
    if (cfg >= SF_CFG_COL_FIRST) return P->d.nz % kSfColConfigs[cfg - SF_CFG_COL_FIRST].vec == 0;
    return true;
}

int launch_config(const sf_plan* P, int cfg, int ich, const SfStepArgs& a, const SfSources& src,
                  cudaStream_t st) {
    const bool g = P->flags != nullptr;
    if (cfg == SF_CFG_MARCH) return sf_launch_step_march(a, src, g, ich, st);
    if (cfg >= SF_CFG_TILE_FIRST)
        return sf_launch_step_tile_cfg(a, src, g, cfg - SF_CFG_TILE_FIRST, ich, st);
    if (cfg >= SF_CFG_COL_FIRST)
        return sf_launch_step_col_cfg(a, src, g, cfg - SF_CFG_COL_FIRST, ich, st);
    return sf_launch_step(a, src, P->poles, g, st);
}

// One step of configuration cfg: a single launch, or for an ADE plan on a
// warp-tile configuration the warp-tile kernel outside the ADE region and
// the per-cell kernel (with the density pre-pass) inside it.  Both read
// only the input set and write disjoint cells of the output set.
int launch_step_split(const sf_plan* P, int cfg, int ich, SfStepArgs& a, const SfSources& src,
                      cudaStream_t st) {
    if (P->poles.n == 0 || cfg < SF_CFG_TILE_FIRST) return launch_config(P, cfg, ich, a, src, st);
    int lo[3], hi[3];
    ade_region(P, cfg, ich, lo, hi);
    SfStepArgs t = a;
    for (int q = 0; q < 3; ++q) {
        t.skip_lo[q] = lo[q];
        t.skip_hi[q] = hi[q];
    }
    if (int rc = launch_config(P, cfg, ich, t, src, st)) return rc;
    if (hi[0] <= lo[0]) return 0;
    SfStepArgs c = a;
    c.trace_prev = nullptr;  // sampled by the warp-tile kernel
    for (int q = 0; q < 3; ++q) {
        c.reg_lo[q] = lo[q];
        c.reg_hi[q] = hi[q];
    }
    return sf_launch_step(c, src, P->poles, P->flags != nullptr, st);
}

bool stream_capturing(cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
}

// Rings, counters and claim order of pipeline configuration cfg with S
// planes per chunk; allocated (outside stream capture) when missing or too
// small.  Fails when they would have to be made during a capture.
int pipe_buffers(sf_plan* P, int cfg, int S, cudaStream_t st) {
    const SfPipeConfig& pc = kSfPipeConfigs[cfg - SF_CFG_PIPE_FIRST];
    const int T = pc.levels, L = pc.lag, M = pc.ring_chunks;
    const int nchunks = (P->d.nx + S - 1) / S;
    const long long ntiles = (long long)((P->d.nz + 31) / 32) * ((P->d.ny + 3) / 4);
    // streaming: rings of M planes, a progress count per (level, tile)
    const size_t ring = (size_t)(T - 1) * 4 * M * (pc.stream ? 1 : S) * (size_t)P->d.ny * P->d.nz;
    const long long items = pc.stream ? T * ntiles : 1 + T * nchunks * ntiles;
    if (items >= INT_MAX) return sf_fail("pipeline: too many work items");
    const int ctrl_n = (int)items;
    const bool order_ok = pc.stream || (P->pipe_order && P->pipe_key[0] == T && P->pipe_key[1] == S &&
                                        P->pipe_key[2] == L && P->pipe_key[3] == M);
    const bool ready = P->pipe_ring_floats >= ring && P->pipe_ctrl_n >= ctrl_n && P->pipe_err &&
                       order_ok && P->pipe_grid[0] == cfg + 1;
    if (ready) return 0;
    if (stream_capturing(st)) return sf_fail("pipeline buffers must be made before a stream capture");
    if (P->pipe_ring_floats < ring) {
        cudaFree(P->pipe_ring);
        P->pipe_ring = nullptr;
        P->pipe_ring_floats = 0;
        SF_CUDA_OK(cudaMalloc(&P->pipe_ring, ring * sizeof(float)));
        P->pipe_ring_floats = ring;
    }
    if (P->pipe_ctrl_n < ctrl_n) {
        cudaFree(P->pipe_ctrl);
        P->pipe_ctrl = nullptr;
        P->pipe_ctrl_n = 0;
        SF_CUDA_OK(cudaMalloc(&P->pipe_ctrl, sizeof(int) * ctrl_n));
        P->pipe_ctrl_n = ctrl_n;
    }
    if (!P->pipe_err) {
        SF_CUDA_OK(cudaMalloc(&P->pipe_err, 2 * sizeof(int)));
        SF_CUDA_OK(cudaMemset(P->pipe_err, 0, 2 * sizeof(int)));
    }
    if (!order_ok) {
        // waves w: level s takes chunk w - (s-1)*lag, lower levels first
        std::vector<int> order;
        for (int w = 0; w < nchunks + (T - 1) * L; ++w)
            for (int lv = 1; lv <= T; ++lv) {
                const int c = w - (lv - 1) * L;
                if (c >= 0 && c < nchunks) order.push_back((lv << 24) | c);
            }
        if ((int)order.size() > P->pipe_order_n) {
            cudaFree(P->pipe_order);
            P->pipe_order = nullptr;
            P->pipe_order_n = 0;
            SF_CUDA_OK(cudaMalloc(&P->pipe_order, sizeof(int) * order.size()));
            P->pipe_order_n = (int)order.size();
        }
        SF_CUDA_OK(cudaMemcpy(P->pipe_order, order.data(), sizeof(int) * order.size(),
                              cudaMemcpyHostToDevice));
        P->pipe_key[0] = T;
        P->pipe_key[1] = S;
        P->pipe_key[2] = L;
        P->pipe_key[3] = M;
    }
    if (P->pipe_grid[0] != cfg + 1) {
        P->pipe_grid[1] = sf_pipe_grid(cfg - SF_CFG_PIPE_FIRST, P->flags != nullptr, P->nu != nullptr);
        P->pipe_grid[0] = cfg + 1;
    }
    return 0;
}

// Whether pipeline configuration cfg can run this plan's steps: float4 warp
// tiles, no ADE poles, and for a streaming configuration every warp resident
// at once, at most 32 probes per tile column and a ring of at least S + 3
// planes (S = planes between progress updates).
bool pipe_fits(sf_plan* P, int cfg, const SfStepArgs& a) {
    if (!sf_tile_supported(a, 4) || P->poles.n > 0) return false;
    const SfPipeConfig& pc = kSfPipeConfigs[cfg - SF_CFG_PIPE_FIRST];
    if (!pc.stream) return true;
    if (P->probe_tile_max > 32) return false;
    int S = chunk_for(P, cfg);
    if (S + 3 > pc.ring_chunks) return false;
    if (P->pipe_grid[0] != cfg + 1) {
        P->pipe_grid[1] = sf_pipe_grid(cfg - SF_CFG_PIPE_FIRST, P->flags != nullptr, P->nu != nullptr);
        P->pipe_grid[0] = cfg + 1;
    }
    const long long ntiles = (long long)((P->d.nz + 31) / 32) * ((P->d.ny + 3) / 4);
    return (pc.levels * ntiles + 3) / 4 <= P->pipe_grid[1];
}

// One launch of pipeline configuration cfg: levels steps from set a.p.. to
// set a.po.. (a.src_val: the first step's waveform row; trace_lvl[l]: probe
// row of the state after level l+1, or null).
int launch_pipe(sf_plan* P, int cfg, int S, const SfStepArgs& a, const SfSources& src,
                float* const* trace_lvl, cudaStream_t st) {
    const SfPipeConfig& pc = kSfPipeConfigs[cfg - SF_CFG_PIPE_FIRST];
    if (S < 1) S = 1;
    if (S > P->d.nx) S = P->d.nx;
    if (int rc = pipe_buffers(P, cfg, S, st)) return rc;
    if (pc.stream) {
        SfPipeArgs A{};
        A.a = a;
        A.levels = pc.levels;
        A.S = S;
        A.M = pc.ring_chunks;
        A.ntk = (P->d.nz + 31) / 32;
        A.ntiles = A.ntk * ((P->d.ny + 3) / 4);
        A.ring = P->pipe_ring;
        A.ctrl = P->pipe_ctrl;
        A.err = P->pipe_err;
        A.spin_limit = P->pipe_spin_limit > 0 ? P->pipe_spin_limit : SF_PIPE_SPIN_DEFAULT;
        A.hold = P->pipe_hold ? P->pipe_err + 1 : nullptr;
        for (int l = 0; l < SF_PIPE_MAX_LEVELS; ++l)
            A.trace_lvl[l] = (trace_lvl && l < A.levels - 1) ? trace_lvl[l] : nullptr;
        SF_CUDA_OK(cudaMemsetAsync(P->pipe_ctrl, 0, sizeof(int) * (size_t)A.levels * A.ntiles, st));
        const int rc = sf_launch_step_stream(A, src, P->flags != nullptr, cfg - SF_CFG_PIPE_FIRST, st);
        return rc == SF_PIPE_NOFIT ? sf_fail("k_step_stream: its warps do not fit on the device") : rc;
    }
    SfPipeArgs A{};
    A.a = a;
    A.levels = pc.levels;
    A.S = S;
    A.M = pc.ring_chunks;
    A.nchunks = (P->d.nx + S - 1) / S;
    A.ntk = (P->d.nz + 31) / 32;
    A.ntiles = A.ntk * ((P->d.ny + 3) / 4);  // one warp: 32 k x 4 rows
    A.ngroups = 0;
    for (int w = 0; w < A.nchunks + (A.levels - 1) * pc.lag; ++w)
        for (int lv = 1; lv <= A.levels; ++lv) {
            const int c = w - (lv - 1) * pc.lag;
            A.ngroups += (c >= 0 && c < A.nchunks) ? 1 : 0;
        }
    A.ring = P->pipe_ring;
    A.order = P->pipe_order;
    A.ctrl = P->pipe_ctrl;
    A.err = P->pipe_err;
    A.spin_limit = P->pipe_spin_limit > 0 ? P->pipe_spin_limit : SF_PIPE_SPIN_DEFAULT;
    A.hold = P->pipe_hold ? P->pipe_err + 1 : nullptr;
    for (int l = 0; l < SF_PIPE_MAX_LEVELS; ++l)
        A.trace_lvl[l] = (trace_lvl && l < A.levels - 1) ? trace_lvl[l] : nullptr;
    SF_CUDA_OK(cudaMemsetAsync(P->pipe_ctrl, 0,
                               sizeof(int) * (1 + (size_t)A.levels * A.nchunks * A.ntiles), st));
    const long long items = (long long)A.ngroups * A.ntiles;
    const int grid = (int)(items < P->pipe_grid[1] ? items : P->pipe_grid[1]);
    return sf_launch_step_pipe(A, src, P->flags != nullptr, cfg - SF_CFG_PIPE_FIRST, grid, st);
}

// Reads and clears the pipeline's wait-expiry flag (synchronises the stream).
int pipe_check(sf_plan* P, cudaStream_t st) {
    if (!P->pipe_err || stream_capturing(st)) return 0;
    int e = 0;
    SF_CUDA_OK(cudaMemcpyAsync(&e, P->pipe_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    SF_CUDA_OK(cudaStreamSynchronize(st));
    if (e == 0) return 0;
    cudaMemsetAsync(P->pipe_err, 0, sizeof(int), st);
    return sf_fail("k_step_pipe: a dependency wait expired (results of this call are invalid)");
}

}  // namespace

extern "C" {

int sf_plan_step(sf_plan* P, int64_t n_steps, const double* src_values, float* trace,
                 void* stream) {
    return sf_plan_step_ex(P, n_steps, src_values, trace, nullptr, stream);
}

int sf_plan_step_ex(sf_plan* P, int64_t n_steps, const double* src_values, float* trace,
                    float* mic_trace, void* stream) {
    if (!P) return sf_fail("sf_plan_step: NULL plan");
    if (!P->bound) return sf_fail("sf_plan_step: fields not bound");
    if (n_steps < 0) return sf_fail("sf_plan_step: negative step count");
    if (P->src.n > 0 && !src_values) return sf_fail("sf_plan_step: sources need src_values");
    if (n_steps == 0) return 0;
    DeviceGuard g(P->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    SfStepArgs a;
    fill_args(P, a, trace != nullptr);
    set_io(P, a, P->cur);  // both sets: the alignment check covers every field
    const int cfg0 = effective_config(P, a);
    const bool mics = mic_trace != nullptr && P->n_mic > 0;
    // plane boundaries or weighted sources: sources move after the fused kernel
    bool deferred = P->n_plane > 0;
    for (int q = 0; q < P->src.n; ++q) deferred = deferred || P->src.s[q].kind == 2;
    // A pipeline configuration runs whole groups of its steps per launch when
    // nothing has to happen between steps; remaining steps (and plans with
    // microphones, plane boundaries or weighted sources) run single steps
    // of the default warp-tile configuration.
    const bool pipe = is_pipe(cfg0) && !deferred && !mics;
    const int levels = pipe ? kSfPipeConfigs[cfg0 - SF_CFG_PIPE_FIRST].levels : 1;
    const int pipe_S = pipe ? chunk_for(P, cfg0) : 0;
    // a two-step configuration runs pairs of steps under the same conditions
    const bool tb = is_tb(cfg0) && !deferred && !mics;
    const int tb_ich = tb ? chunk_for(P, cfg0) : 0;
    const int cfg = (is_pipe(cfg0) || is_tb(cfg0)) ? SF_CFG_TILE_DEFAULT : cfg0;
    const int ich = chunk_for(P, cfg);
    bool piped = false;
    for (int64_t s = 0; s < n_steps;) {
        if (pipe && n_steps - s >= levels) {
            set_io(P, a, P->cur);
            a.src_val = P->src.n > 0 ? src_values + s * P->src.n : nullptr;
            a.trace_prev = (a.n_probe > 0 && s > 0) ? trace + (s - 1) * P->n_probe : nullptr;
            float* tl[SF_PIPE_MAX_LEVELS] = {nullptr, nullptr, nullptr, nullptr};
            if (a.n_probe > 0)
                for (int l = 0; l + 1 < levels; ++l) tl[l] = trace + (s + l) * P->n_probe;
            if (int rc = launch_pipe(P, cfg0, pipe_S, a, P->src, tl, st)) return rc;
            piped = true;
            P->cur = 1 - P->cur;
            P->steps_done += levels;
            s += levels;
            continue;
        }
        if (tb && n_steps - s >= 2) {
            set_io(P, a, P->cur);
            a.src_val = P->src.n > 0 ? src_values + s * P->src.n : nullptr;
            a.trace_prev = (a.n_probe > 0 && s > 0) ? trace + (s - 1) * P->n_probe : nullptr;
            a.reverse = (int)((P->steps_done >> 1) & 1);
            float* t1 = a.n_probe > 0 ? trace + s * P->n_probe : nullptr;
            if (int rc = sf_launch_step_tb(a, P->src, P->flags != nullptr, cfg0 - SF_CFG_TB_FIRST,
                                           tb_ich, t1, st))
                return rc;
            P->cur = 1 - P->cur;
            P->steps_done += 2;
            s += 2;
            continue;
        }
        set_io(P, a, P->cur);
        a.src_val = P->src.n > 0 ? src_values + s * P->src.n : nullptr;
        a.trace_prev = (a.n_probe > 0 && s > 0) ? trace + (s - 1) * P->n_probe : nullptr;
        a.reverse = (int)(P->steps_done & 1);
        if (!deferred) {
            if (int rc = launch_step_split(P, cfg, ich, a, P->src, st)) return rc;
        } else {  // step, plane boundaries in order, then the sources in order
            const SfSources none{};
            if (int rc = launch_step_split(P, cfg, ich, a, none, st)) return rc;
            float* const* out = P->f[1 - P->cur];
            for (int q = 0; q < P->n_plane; ++q)
                if (int rc = sf_launch_plane_bc(out[0], P->plane_prev + P->plane_off[q][0],
                                                P->plane_prev + P->plane_off[q][1],
                                                P->plane_ops[q], P->d.nx, P->d.ny, P->d.nz, st))
                    return rc;
            for (int q = 0; q < P->src.n; ++q) {
                const sf_source& S = P->src.s[q];
                int rc;
                if (S.kind == 2)
                    rc = sf_launch_inject_weighted(out[S.b], P->wsrc_cells[S.a], P->wsrc_w[S.a],
                                                   P->wsrc_n[S.a], a.src_val + q, st);
                else
                    rc = sf_launch_inject(out[0], P->flags, S, a.src_val + q, P->d.nx, P->d.ny,
                                          P->d.nz, st);
                if (rc) return rc;
            }
        }
        P->cur = 1 - P->cur;
        ++P->steps_done;
        ++s;
        if (mics)
            if (int rc = sf_launch_mic_gather(P->f[P->cur][0], P->f[P->cur][1], P->f[P->cur][2],
                                              P->f[P->cur][3], P->mic_field, P->mic_idx,
                                              P->mic_w, P->n_mic, mic_trace + (s - 1) * P->n_mic,
                                              st))
                return rc;
    }
    if (trace && P->n_probe > 0)
        if (int rc = sf_launch_probe_gather(P->f[P->cur][0], P->probe_cells, P->n_probe,
                                            trace + (n_steps - 1) * P->n_probe, st))
            return rc;
    return piped ? pipe_check(P, st) : 0;
}

int sf_plan_set_microphones(sf_plan* P, int n, const int64_t* idx8, const float* w8) {
    return sf_plan_set_microphones_ex(P, n, nullptr, idx8, w8);
}

int sf_plan_set_microphones_ex(sf_plan* P, int n, const int32_t* field, const int64_t* idx8,
                               const float* w8) {
    if (!P) return sf_fail("sf_plan_set_microphones: NULL plan");
    if (n < 0 || (n > 0 && (!idx8 || !w8))) return sf_fail("sf_plan_set_microphones: bad table");
    if (field)
        for (int q = 0; q < n; ++q)
            if (field[q] < 0 || field[q] > 3)
                return sf_fail("sf_plan_set_microphones: field must be 0 (p) .. 3 (vz)");
    for (long long q = 0; q < 8LL * n; ++q)
        if (idx8[q] < 0 || idx8[q] >= P->n)
            return sf_fail("sf_plan_set_microphones: corner cell outside the grid");
    DeviceGuard g(P->device);
    cudaFree(P->mic_idx);
    cudaFree(P->mic_w);
    cudaFree(P->mic_field);
    P->mic_idx = nullptr;
    P->mic_w = nullptr;
    P->mic_field = nullptr;
    P->n_mic = n;
    if (n == 0) return 0;
    SF_CUDA_OK(cudaMalloc(&P->mic_idx, sizeof(long long) * 8 * n));
    SF_CUDA_OK(cudaMalloc(&P->mic_w, sizeof(float) * 8 * n));
    SF_CUDA_OK(cudaMemcpy(P->mic_idx, idx8, sizeof(long long) * 8 * n, cudaMemcpyHostToDevice));
    SF_CUDA_OK(cudaMemcpy(P->mic_w, w8, sizeof(float) * 8 * n, cudaMemcpyHostToDevice));
    if (field) {
        SF_CUDA_OK(cudaMalloc(&P->mic_field, sizeof(int) * n));
        SF_CUDA_OK(cudaMemcpy(P->mic_field, field, sizeof(int) * n, cudaMemcpyHostToDevice));
    }
    return 0;
}

int sf_plan_autotune(sf_plan* P, int launches, void* stream, float* ms_out, int* best_out) {
    if (!P) return sf_fail("sf_plan_autotune: NULL plan");
    if (!P->bound) return sf_fail("sf_plan_autotune: fields not bound");
    if (launches < 1) launches = 1;
    DeviceGuard g(P->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int count = sf_kernel_config_count();
    if (ms_out)
        for (int q = 0; q < count; ++q) ms_out[q] = -1.0f;
    // With ADE poles only the warp-tile configurations are candidates; each
    // is timed on the cells outside its ADE region (the per-cell kernel's
    // share inside it is the same for all of them).
    const bool ade = P->poles.n > 0;
    P->tuned_ich = 0;
    // Every trial reads the current set and writes the other one without
    // swapping, with no sources and no probes: the state is untouched, and the
    // next real step overwrites the other set entirely.
    SfStepArgs a;
    fill_args(P, a, false);
    set_io(P, a, P->cur);
    const SfSources none{};
    cudaEvent_t e0, e1;
    SF_CUDA_OK(cudaEventCreate(&e0));
    SF_CUDA_OK(cudaEventCreate(&e1));
    int rc = 0;
    // ms per step of configuration cfg with planes per block ich (a warm-up
    // launch, then `launches` timed ones; a pipeline launch is `levels` steps)
    auto trial = [&](int cfg, int ich, float* ms_step) -> int {
        SfStepArgs t = a;
        if (ade && !is_pipe(cfg)) ade_region(P, cfg, ich, t.skip_lo, t.skip_hi);
        auto one = [&]() -> int {
            if (is_tb(cfg))
                return sf_launch_step_tb(t, none, P->flags != nullptr, cfg - SF_CFG_TB_FIRST, ich,
                                         nullptr, st);
            return is_pipe(cfg) ? launch_pipe(P, cfg, ich, t, none, nullptr, st)
                                : launch_config(P, cfg, ich, t, none, st);
        };
        if (int r = one()) return r;
        if (cudaEventRecord(e0, st) != cudaSuccess) return sf_fail("event record failed");
        for (int q = 0; q < launches; ++q)
            if (int r = one()) return r;
        if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
            return sf_fail("sf_plan_autotune: timing failed");
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        const int steps = is_pipe(cfg) ? kSfPipeConfigs[cfg - SF_CFG_PIPE_FIRST].levels
                                        : (is_tb(cfg) ? 2 : 1);
        *ms_step = ms / (launches * steps);
        return 0;
    };
    int best = 0;
    float best_ms = 0.0f;
    for (int cfg = SF_CFG_CELL; cfg < count && !rc; ++cfg) {
        if (!config_native(P, cfg, a) || ((ade || P->nu) && cfg < SF_CFG_TILE_FIRST)) continue;
        // multi-step pipelines only by explicit choice: on GB300 they are
        // slower than single steps, and their fewer launches per step would
        // win a trial timed under a profiler that serialises launches
        if (is_pipe(cfg)) continue;
        float ms = 0.0f;
        if ((rc = trial(cfg, chunk_for(P, cfg), &ms))) break;
        if (ms_out) ms_out[cfg] = ms;
        if (best == 0 || ms < best_ms) {
            best = cfg;
            best_ms = ms;
        }
    }
    if (!rc) rc = pipe_check(P, st);
    // then the planes per block of the winner (unless the caller fixed them)
    if (!rc && best >= SF_CFG_COL_FIRST && P->i_chunk == 0) {
        const int auto_ich = chunk_for(P, best);
        int best_ich = auto_ich;
        static const int cand_step[] = {8, 12, 16, 20, 24, 32, 48};
        static const int cand_pipe[] = {1, 2, 3, 4, 6, 8};
        static const int cand_tb[] = {4, 8, 12, 16, 25, 32, 50, 64};
        const int* cand = is_pipe(best) ? cand_pipe : (is_tb(best) ? cand_tb : cand_step);
        const int ncand = is_pipe(best) ? 6 : (is_tb(best) ? 8 : 7);
        for (int q = 0; q < ncand && !rc; ++q) {
            const int ich = cand[q];
            if (ich == auto_ich || ich > P->d.nx) continue;
            float ms = 0.0f;
            if ((rc = trial(best, ich, &ms))) break;
            if (ms < best_ms) {
                best_ms = ms;
                best_ich = ich;
            }
        }
        if (!rc && is_pipe(best)) rc = pipe_check(P, st);
        if (!rc && best_ich != auto_ich) P->tuned_ich = best_ich;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (best == 0) best = SF_CFG_CELL;  // ADE on a grid no warp-tile kernel takes
    P->tuned = best;
    if (best_out) *best_out = best;
    return 0;
}

int64_t sf_energy_scratch_doubles(const sf_plan* P) {
    return P ? 2 * sf_energy_blocks(P->n, P->sms) + 2 : 0;
}

int sf_plan_energy(sf_plan* P, double rho, double c, double dx, double* scratch,
                   double* out_host, void* stream) {
    if (!P || !scratch || !out_host) return sf_fail("sf_plan_energy: NULL argument");
    if (!P->bound) return sf_fail("sf_plan_energy: fields not bound");
    DeviceGuard g(P->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const long long nb = sf_energy_blocks(P->n, P->sms);
    float* const* f = P->f[P->cur];
    if (int rc = sf_launch_energy(f[0], f[1], f[2], f[3], P->flags, P->n, P->sms, scratch,
                                  scratch + 2 * nb, st))
        return rc;
    double sums[2];
    SF_CUDA_OK(cudaMemcpyAsync(sums, scratch + 2 * nb, sizeof(sums), cudaMemcpyDeviceToHost, st));
    SF_CUDA_OK(cudaStreamSynchronize(st));
    const double dV = dx * dx * dx;
    *out_host = 0.5 * sums[0] / (rho * c * c) * dV + 0.5 * rho * sums[1] * dV;
    return 0;
}

}  // extern "C"

namespace {

// Upload the program (and the cell centres of a nonuniform grid), voxelise,
// and report a malformed program.
int voxelize_impl(const sf_sdf_node* nodes, int n_nodes, int nx, int ny, int nz,
                  double res, const double* const* coords, int invert, uint8_t* out_dev,
                  cudaStream_t st) {
    if (!nodes || n_nodes < 1 || !out_dev) return sf_fail("sf_voxelize: bad program or output");
    if (nx < 1 || ny < 1 || nz < 1 || nx > 65535) return sf_fail("sf_voxelize: bad grid");
    const size_t prog_bytes = (sizeof(sf_sdf_node) * n_nodes + 15) / 16 * 16;
    const size_t coord_bytes = coords ? sizeof(double) * ((size_t)nx + ny + nz) : 0;
    char* buf = nullptr;  // stream-ordered: no device-wide wait on release
    SF_CUDA_OK(cudaMallocAsync(reinterpret_cast<void**>(&buf), prog_bytes + 16 + coord_bytes, st));
    sf_sdf_node* prog = reinterpret_cast<sf_sdf_node*>(buf);
    int* err = reinterpret_cast<int*>(buf + prog_bytes);
    double* cdev = coords ? reinterpret_cast<double*>(buf + prog_bytes + 16) : nullptr;
    int rc = 0;
    int herr = 0;
    if (cudaMemcpyAsync(prog, nodes, sizeof(sf_sdf_node) * n_nodes, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess) {
        rc = sf_fail("sf_voxelize: upload failed");
    }
    if (!rc && coords) {
        const int n3[3] = {nx, ny, nz};
        size_t off = 0;
        for (int a = 0; a < 3 && !rc; ++a) {
            if (cudaMemcpyAsync(cdev + off, coords[a], sizeof(double) * n3[a],
                                cudaMemcpyHostToDevice, st) != cudaSuccess)
                rc = sf_fail("sf_voxelize: coordinate upload failed");
            off += n3[a];
        }
    }
    if (!rc) rc = sf_launch_voxelize(prog, n_nodes, nx, ny, nz, res, cdev, invert, out_dev, err, st);
    if (!rc && (cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess))
        rc = sf_fail("sf_voxelize: kernel failed");
    cudaFreeAsync(buf, st);
    if (!rc && herr) rc = sf_fail("sf_voxelize: malformed SDF program (stack error)");
    return rc;
}

}  // namespace

namespace {

// Geometry and material ids in one pass (k_voxelize_materials): program p
// is nodes[prog_off[p] .. prog_off[p+1]-1], program 0 the geometry, 1..n the
// regions with ids[0..n-1].
int voxelize_materials_impl(const sf_sdf_node* nodes, const int32_t* prog_off, int n_regions,
                            const uint8_t* ids, int nx, int ny, int nz, double res,
                            const double* const* coords, uint8_t* geom_dev, uint8_t* mat_dev,
                            cudaStream_t st) {
    if (!nodes || !prog_off || n_regions < 0 || n_regions > 255 || (n_regions > 0 && !ids) ||
        !geom_dev || !mat_dev)
        return sf_fail("sf_voxelize_materials: bad programs, ids or outputs");
    if (nx < 1 || ny < 1 || nz < 1 || nx > 65535) return sf_fail("sf_voxelize_materials: bad grid");
    for (int p = 0; p <= n_regions; ++p)
        if (prog_off[p] < 0 || prog_off[p + 1] <= prog_off[p])
            return sf_fail("sf_voxelize_materials: every program needs at least one node");
    const int n_nodes = prog_off[n_regions + 1];
    const size_t prog_bytes = (sizeof(sf_sdf_node) * n_nodes + 15) / 16 * 16;
    const size_t off_bytes = (sizeof(int) * (n_regions + 2) + 15) / 16 * 16;
    const size_t ids_bytes = (size_t)(n_regions + 16) / 16 * 16;
    const size_t coord_bytes = coords ? sizeof(double) * ((size_t)nx + ny + nz) : 0;
    char* buf = nullptr;  // stream-ordered: no device-wide wait on release
    SF_CUDA_OK(cudaMallocAsync(reinterpret_cast<void**>(&buf),
                               prog_bytes + off_bytes + ids_bytes + 16 + coord_bytes, st));
    sf_sdf_node* prog = reinterpret_cast<sf_sdf_node*>(buf);
    int* off = reinterpret_cast<int*>(buf + prog_bytes);
    uint8_t* idd = reinterpret_cast<uint8_t*>(buf + prog_bytes + off_bytes);
    int* err = reinterpret_cast<int*>(buf + prog_bytes + off_bytes + ids_bytes);
    double* cdev = coords ? reinterpret_cast<double*>(buf + prog_bytes + off_bytes + ids_bytes + 16)
                          : nullptr;
    int rc = 0, herr = 0;
    if (cudaMemcpyAsync(prog, nodes, sizeof(sf_sdf_node) * n_nodes, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(off, prog_off, sizeof(int) * (n_regions + 2), cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        (n_regions > 0 &&
         cudaMemcpyAsync(idd, ids, n_regions, cudaMemcpyHostToDevice, st) != cudaSuccess) ||
        cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess)
        rc = sf_fail("sf_voxelize_materials: upload failed");
    if (!rc && coords) {
        const int n3[3] = {nx, ny, nz};
        size_t o = 0;
        for (int a = 0; a < 3 && !rc; ++a) {
            if (!coords[a] || cudaMemcpyAsync(cdev + o, coords[a], sizeof(double) * n3[a],
                                              cudaMemcpyHostToDevice, st) != cudaSuccess)
                rc = sf_fail("sf_voxelize_materials: coordinate upload failed");
            o += n3[a];
        }
    }
    if (!rc)
        rc = sf_launch_voxelize_materials(prog, off, idd, n_regions, nx, ny, nz, res, cdev,
                                          geom_dev, mat_dev, err, st);
    if (!rc && (cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess))
        rc = sf_fail("sf_voxelize_materials: kernel failed");
    cudaFreeAsync(buf, st);
    if (!rc && herr) rc = sf_fail("sf_voxelize_materials: malformed SDF program (stack error)");
    return rc;
}

}  // namespace

extern "C" {

int sf_voxelize_materials(const sf_sdf_node* nodes, const int32_t* prog_off, int n_regions,
                          const uint8_t* ids, int nx, int ny, int nz, double res,
                          const double* const* coords, uint8_t* geom_dev, uint8_t* mat_dev,
                          void* stream) {
    return voxelize_materials_impl(nodes, prog_off, n_regions, ids, nx, ny, nz, res, coords,
                                   geom_dev, mat_dev, static_cast<cudaStream_t>(stream));
}

int sf_voxelize(const sf_sdf_node* nodes, int n_nodes, int nx, int ny, int nz, double res,
                int invert, uint8_t* out_dev, void* stream) {
    return voxelize_impl(nodes, n_nodes, nx, ny, nz, res, nullptr, invert, out_dev,
                         static_cast<cudaStream_t>(stream));
}

int sf_voxelize_coords(const sf_sdf_node* nodes, int n_nodes, int nx, int ny, int nz,
                       const double* const* coords, int invert, uint8_t* out_dev, void* stream) {
    if (!coords || !coords[0] || !coords[1] || !coords[2])
        return sf_fail("sf_voxelize_coords: NULL coordinate array");
    return voxelize_impl(nodes, n_nodes, nx, ny, nz, 0.0, coords, invert, out_dev,
                         static_cast<cudaStream_t>(stream));
}

int sf_sdf_eval(const sf_sdf_node* nodes, int n_nodes, const double* points_dev, int64_t n,
                double* out_dev, void* stream) {
    if (!nodes || n_nodes < 1 || (n > 0 && (!points_dev || !out_dev)))
        return sf_fail("sf_sdf_eval: bad program, points or output");
    if (n == 0) return 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    sf_sdf_node* prog = nullptr;
    SF_CUDA_OK(cudaMallocAsync(reinterpret_cast<void**>(&prog), sizeof(sf_sdf_node) * n_nodes + 16, st));
    int* err = reinterpret_cast<int*>(reinterpret_cast<char*>(prog) + sizeof(sf_sdf_node) * n_nodes);
    int rc = 0, herr = 0;
    if (cudaMemcpyAsync(prog, nodes, sizeof(sf_sdf_node) * n_nodes, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess)
        rc = sf_fail("sf_sdf_eval: upload failed");
    if (!rc) rc = sf_launch_sdf_points(prog, n_nodes, points_dev, n, out_dev, err, st);
    if (!rc && (cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess))
        rc = sf_fail("sf_sdf_eval: kernel failed");
    cudaFreeAsync(prog, st);
    if (!rc && herr) rc = sf_fail("sf_sdf_eval: malformed SDF program (stack error)");
    return rc;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Energy without any device allocation.
//
// Some callers cannot allocate device memory at the moment they want an
// energy reading: a host whose HBM is already reserved by another caching
// allocator (a PyTorch process, say), where a fresh cudaMalloc can fail or
// force that allocator to release its cache; or a real-time loop (an audio
// or auralisation callback) that must not take cudaMalloc / cudaFree, which
// can synchronise the whole device and stall for milliseconds.  For them the
// energy reduction runs with its scratch in a fixed array that lives in the
// library's device image: SF_NOALLOC_ENERGY_DOUBLES doubles (32 KiB), held by
// every GPU that loads the library until the process exits.
//
// The reduction needs 2 partial sums per block plus 2 totals; its block
// count is capped at 8 per SM of the plan's device (1216 on a 152-SM GB300,
// 2434 doubles), so a device with more than 255 SMs is refused with an error.
// Every partial-sum slot is written before it is read, so nothing has to be
// cleared between calls.  All calls share the one array per device: calls
// whose kernels overlap on the GPU (two streams at once) race and must not be
// issued.
#define SF_NOALLOC_ENERGY_DOUBLES 4096
#define SF_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double g_sf_noalloc_energy[SF_NOALLOC_ENERGY_DOUBLES];

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_addr[SF_NOALLOC_MAX_DEVICES] = {nullptr};
}  // namespace

// Looks the array's device address up on device `dev` (which must be
// current), once per device.  Called by sf_plan_create, so the module load
// and the lookup happen when a plan is made and no energy call does them.
// In host code the array's name is only a host-side stand-in; kernels must be
// given this address.  A cudaDeviceReset invalidates it together with every
// plan made before the reset; the library does not support using plans or
// this entry point across a reset.
int sf_noalloc_setup(int dev) {
    if (dev < 0 || dev >= SF_NOALLOC_MAX_DEVICES)
        return sf_fail("sf_plan_create: device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_sf_noalloc_energy);
        if (e != cudaSuccess) return sf_fail_cuda(e, "cudaGetSymbolAddress", __FILE__, __LINE__);
        g_noalloc_addr[dev] = static_cast<double*>(p);
    }
    return 0;
}

extern "C" int sf_plan_energy_noalloc(sf_plan* P, double rho, double c, double dx,
                                      double* out_host, void* stream) {
    if (!P || !out_host) return sf_fail("sf_plan_energy_noalloc: NULL argument");
    if (!P->bound) return sf_fail("sf_plan_energy_noalloc: fields not bound");
    if (P->device < 0 || P->device >= SF_NOALLOC_MAX_DEVICES)
        return sf_fail("sf_plan_energy_noalloc: device ordinal out of range");
    DeviceGuard g(P->device);
    const long long nb = sf_energy_blocks(P->n, P->sms);
    if (2 * nb + 2 > SF_NOALLOC_ENERGY_DOUBLES)
        return sf_fail("sf_plan_energy_noalloc: reduction needs more than the 4096-double "
                       "fixed scratch (device with more than 255 SMs)");
    double* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        scratch = g_noalloc_addr[P->device];
    }
    if (!scratch) return sf_fail("sf_plan_energy_noalloc: scratch address not set up");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float* const* f = P->f[P->cur];
    if (int rc = sf_launch_energy(f[0], f[1], f[2], f[3], P->flags, P->n, P->sms, scratch,
                                  scratch + 2 * nb, st))
        return rc;
    double sums[2];
    SF_CUDA_OK(cudaMemcpyAsync(sums, scratch + 2 * nb, sizeof(sums), cudaMemcpyDeviceToHost, st));
    SF_CUDA_OK(cudaStreamSynchronize(st));
    const double dV = dx * dx * dx;
    *out_host = 0.5 * sums[0] / (rho * c * c) * dV + 0.5 * rho * sums[1] * dV;
    return 0;
}
