// sf_kernels.h -- internal launcher declarations shared by the .cu files.
#pragma once
#include <cuda_runtime.h>

#include "sf_common.cuh"

// Step-kernel configuration indices used by sf_plan_set_kernel /
// sf_plan_autotune: 0 = automatic, 1 = per-cell kernel, 2 = slab march,
// SF_CFG_COL_FIRST + c = column kernel configuration c, then the warp-tile
// configurations.
enum { SF_CFG_AUTO = 0, SF_CFG_CELL = 1, SF_CFG_MARCH = 2, SF_CFG_COL_FIRST = 3 };

struct SfColConfig {
    int vec, by, minb, cs;
    const char* name;
};
extern const SfColConfig kSfColConfigs[];
extern const int kSfColConfigCount;

// Warp-tile kernel configurations follow the column ones:
// index SF_CFG_COL_FIRST + kSfColConfigCount + t.
struct SfTileConfig {
    int vec, rows, warps, minb, prefetch;
    const char* name;
};
extern const SfTileConfig kSfTileConfigs[];
extern const int kSfTileConfigCount;
// Whether a warp-tile kernel with `vec` cells per lane runs on this grid.
bool sf_tile_supported(const SfStepArgs& a, int vec);

// Multi-step pipeline configurations follow the warp-tile ones: index
// SF_CFG_COL_FIRST + kSfColConfigCount + kSfTileConfigCount + t.  One launch
// advances the state by `levels` steps (sf_step_pipe.cu).  Claimed-item
// pipelines (stream = 0): level s runs `lag` chunks behind level s-1 and the
// rings between levels hold `ring_chunks` chunks of planes each.  Streaming
// pipelines (stream = 1): one co-resident warp per (level, tile) walks the
// whole x extent; the rings hold `ring_chunks` planes (a power of two).
#define SF_PIPE_MAX_LEVELS 4
struct SfPipeConfig {
    int levels, warps, minb, lag, ring_chunks, stream;
    const char* name;
};
extern const SfPipeConfig kSfPipeConfigs[];
extern const int kSfPipeConfigCount;

// One launch of the pipeline: a.p.. is the input set, a.po.. the output
// set, a.src_val the first step's waveform values (level s uses row s-1),
// a.trace_prev the probe row of the input state.
struct SfPipeArgs {
    SfStepArgs a;
    int levels;   // steps per launch
    int S;        // planes per chunk
    int M;        // chunks per ring
    int nchunks;  // ceil(nx / S)
    int ntk;      // tiles along k (32 cells each)
    int ntiles;   // tiles per chunk
    int ngroups;  // (level, chunk) groups in claim order
    float* ring;        // (levels-1) rings x 4 fields x M*S planes
    const int* order;   // per group: (level << 24) | chunk, level 1-based
    int* ctrl;          // [0] next item; [1 + ((level-1)*nchunks + chunk)*ntiles + tile] done
    int* err;           // nonzero: a bounded wait expired (2)
    float* trace_lvl[SF_PIPE_MAX_LEVELS];  // probe row of level s+1's result, or null
    long long spin_limit;  // sleeps (64-256 ns each) before a wait gives up
    // Expiry test hook, normally null: a flag that nothing ever sets.  The
    // first claimed item (k_step_pipe) or the first warp (k_step_stream)
    // also waits on it, so its wait runs out and the launch fails cleanly.
    const int* hold;
};
// Default bound of every pipeline wait: 2^22 sleeps, about 1 s.
#define SF_PIPE_SPIN_DEFAULT (1LL << 22)
int sf_launch_step_pipe(const SfPipeArgs& P, const SfSources& src, bool geom, int cfg, int grid,
                        cudaStream_t st);
// Resident blocks of pipeline configuration cfg on this device (grid size).
int sf_pipe_grid(int cfg, bool geom, bool nu);
// Streaming pipeline: P.ctrl holds the per-(level, tile) plane progress
// (levels * ntiles ints, zeroed), P.S the publishing interval in planes,
// P.M the ring planes; probe_tile[u] / probe_plane[u] place the probes.
// Returns SF_PIPE_NOFIT (without launching) when its warps cannot all be
// resident at once.
#define SF_PIPE_NOFIT 77
int sf_launch_step_stream(const SfPipeArgs& P, const SfSources& src, bool geom, int cfg,
                          cudaStream_t st);

// Two-step configurations (sf_step_tb.cu) follow the pipeline ones: index
// SF_CFG_COL_FIRST + kSfColConfigCount + kSfTileConfigCount +
// kSfPipeConfigCount + t.  One launch advances the state by two steps;
// warps of 28 output k x `rows` output j, `warps` per block along j;
// trace1 receives the probe row of the state after the first step.
struct SfTbConfig {
    int rows, warps, minb;
    const char* name;
};
extern const SfTbConfig kSfTbConfigs[];
extern const int kSfTbConfigCount;
bool sf_tb_supported(const SfStepArgs& a);
int sf_launch_step_tb(const SfStepArgs& a, const SfSources& src, bool geom, int cfg, int ich,
                      float* trace1, cudaStream_t st);

int sf_launch_build_flags(const uint8_t* geom, uint8_t* flags, int nx, int ny, int nz,
                          cudaStream_t st);
int sf_launch_step(const SfStepArgs& a, const SfSources& src, const SfPoles& poles, bool geom,
                   cudaStream_t st);
int sf_launch_probe_gather(const float* p, const long long* cells, int n, float* out,
                           cudaStream_t st);
int sf_launch_step_march(const SfStepArgs& a, const SfSources& src, bool geom, int ich,
                         cudaStream_t st);
int sf_launch_step_col_cfg(const SfStepArgs& a, const SfSources& src, bool geom, int cfg, int ich,
                           cudaStream_t st);
int sf_launch_step_tile_cfg(const SfStepArgs& a, const SfSources& src, bool geom, int cfg, int ich,
                            cudaStream_t st);
int sf_launch_plane_bc(float* p, float* prev_lo, float* prev_hi, const sf_plane_bc& op, int nx,
                       int ny, int nz, cudaStream_t st);
int sf_launch_inject(float* p, const uint8_t* flags, const sf_source& s, const double* val, int nx,
                     int ny, int nz, cudaStream_t st);
int sf_launch_inject_weighted(float* f, const long long* cells, const double* w, long long n,
                              const double* val, cudaStream_t st);
int sf_launch_mic_gather(const float* p, const float* vx, const float* vy, const float* vz,
                         const int* field, const long long* idx, const float* w, int n, float* out,
                         cudaStream_t st);
// Blocks of the energy reduction over n cells on a device with `sms` SMs
// (at most 8 per SM); its scratch holds 2 partial sums per block + 2 totals.
long long sf_energy_blocks(long long n, int sms);
int sf_launch_energy(const float* p, const float* vx, const float* vy, const float* vz,
                     const uint8_t* flags, long long n, int sms, double* scratch, double* out2,
                     cudaStream_t st);
int sf_launch_voxelize(const sf_sdf_node* prog_dev, int n_nodes, int nx, int ny, int nz,
                       double res, const double* coords_dev, int invert, uint8_t* out,
                       int* err_dev, cudaStream_t st);
int sf_launch_voxelize_materials(const sf_sdf_node* prog_dev, const int* off_dev,
                                 const uint8_t* ids_dev, int n_regions, int nx, int ny, int nz,
                                 double res, const double* coords_dev, uint8_t* geom,
                                 uint8_t* mat, int* err_dev, cudaStream_t st);
int sf_launch_sdf_points(const sf_sdf_node* prog_dev, int n_nodes, const double* pts, long long n,
                         double* out, int* err_dev, cudaStream_t st);
