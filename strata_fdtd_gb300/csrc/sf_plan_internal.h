// sf_plan_internal.h -- the plan object behind the sf_plan handle, shared by
// the host-side translation units (sf_api.cu, sf_batch.cu).
#pragma once
#include <cuda_runtime.h>

#include "sf_common.cuh"

struct sf_plan {
    sf_grid_desc d{};
    long long n = 0;
    int device = 0;
    int sms = 0;  // SM count of the device (sizes the energy reduction)
    float* f[2][4] = {{nullptr}};
    int cur = 0;
    bool bound = false;
    uint8_t* flags = nullptr;  // owned; null = no geometry (all air)
    float* decay[3] = {nullptr, nullptr, nullptr};  // owned, 1.0f where axis off
    SfSources src{};
    long long* probe_cells = nullptr;  // owned
    int n_probe = 0;
    SfPoles poles{};
    const uint8_t* mat = nullptr;  // caller-owned
    int variant = 0;               // kernel configuration (SF_CFG_*), 0 = auto
    int i_chunk = 0;               // planes per block in march / column kernels (0 = auto)
    int tuned = 0;                 // configuration chosen by sf_plan_autotune (0 = none)
    int tuned_ich = 0;             // its planes per block, when the autotuner chose them
    long long steps_done = 0;      // steps issued so far (alternates the chunk order)
    int n_mic = 0;                 // microphone rows: 8 corner cells and weights each
    long long* mic_idx = nullptr;  // owned
    float* mic_w = nullptr;        // owned
    int* mic_field = nullptr;      // owned: field per row (0 p, 1 vx, 2 vy, 3 vz)
    int ade_lo[3] = {0, 0, 0};     // box holding every material cell (density pre-pass)
    int ade_hi[3] = {0, 0, 0};
    float* nu = nullptr;  // owned, nonuniform grid: face coefficients x, y, z, then
                          // cell inverse spacings x, y, z (nx, ny, nz floats each)
    int n_plane = 0;                    // pressure-plane boundary operations
    sf_plane_bc plane_ops[SF_MAX_PLANE_OPS];
    float* plane_prev = nullptr;        // owned: stored planes, low then high per op
    long long plane_off[SF_MAX_PLANE_OPS][2];
    long long* wsrc_cells[SF_MAX_SOURCES] = {nullptr};  // owned, weighted (membrane) sources
    double* wsrc_w[SF_MAX_SOURCES] = {nullptr};
    long long wsrc_n[SF_MAX_SOURCES] = {0};
    // multi-step pipeline (sf_step_pipe.cu)
    float* pipe_ring = nullptr;  // owned: rings of planes between levels
    size_t pipe_ring_floats = 0;
    int* pipe_ctrl = nullptr;  // owned: claim counter, tiles done per (level, chunk)
    int pipe_ctrl_n = 0;
    int* pipe_err = nullptr;    // owned: [0] wait-expiry flag, [1] a flag nothing sets
    long long pipe_spin_limit = 0;  // sleeps before a pipeline wait gives up (0 = default)
    bool pipe_hold = false;         // expiry test hook: the first item waits on pipe_err[1]
    int* pipe_order = nullptr;  // owned: (level, chunk) claim order
    int pipe_order_n = 0;
    int pipe_key[4] = {0, 0, 0, 0};  // levels, planes per chunk, lag, ring chunks of the order
    int pipe_grid[2] = {0, 0};       // configuration + 1, resident blocks
    int probe_tile_max = 0;          // most probes in one 32 k x 4 row tile column
};

// Planes per block: enough (j,k)-tile x i-chunk blocks for about four waves
// of 8 resident blocks on each of the SMs.  kspan / jspan: cells a block
// covers along k / j.
inline int auto_chunk(const sf_plan* P, int kspan, int jspan = 8) {
    int sms = 152;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long tiles = (long long)((P->d.nz + kspan - 1) / kspan) * ((P->d.ny + jspan - 1) / jspan);
    long long chunks = (4LL * 8 * sms + tiles - 1) / tiles;
    if (chunks < 1) chunks = 1;
    long long ich = (P->d.nx + chunks - 1) / chunks;
    if (ich < 4) ich = 4;
    if (ich > P->d.nx) ich = P->d.nx;
    return (int)ich;
}


// Queue a device buffer (bytes: its size, for the release threshold) or a
// graph for release without a device-wide wait (sf_api.cu).
void sf_defer_free(void* p, size_t bytes);
void sf_defer_graph(cudaGraphExec_t exec, cudaGraph_t graph);

// Makes the plan's device current for the scope of a call.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int now = -1;
        if (prev >= 0 && cudaGetDevice(&now) == cudaSuccess && now != prev) cudaSetDevice(prev);
    }
};
