// sf_step_pipe.cu -- several steps per pass over the state: a persistent
// wavefront pipeline of float4 warp-tile work items.
//
// One launch advances the state by T steps ("levels").  Level 1 reads the
// input set and writes its result into a ring of planes, level s reads the
// ring of level s-1 and writes ring s, level T writes the output set.  The
// rings are small (M chunks of S planes per field) and stay in L2, so HBM
// sees one read of the input set and one write of the output set per T
// steps instead of per step.
//
// Work item = (level s, chunk c of S planes, (j,k) tile of 32 k x 4 rows),
// one warp's job.  Warps claim items from an atomic counter in a fixed
// wavefront order (level s runs `lag` chunks behind level s-1) and run each
// with tile4_run, the routine of the single-step warp-tile kernels, so every
// cell gets the reference's arithmetic in the reference's order and the
// result is bit-identical to T single steps.
//
// An item (s, c, t) waits only for items claimed before it, each tracked by
// its own completion flag:
//   * s > 1: level s-1, chunks c-1 .. c+1, tile t and its four neighbours
//     (the planes c*S-1 .. c*S+S and the edge cells its tile reads);
//   * s < T: the ring slot of chunk c is free, i.e. the readers of chunk c-M
//     (level s+1, chunks c-M-1 .. c-M+1, tile t and its neighbours) are done.
// The claim order puts both before the item (M > lag + 1), so the earliest
// unfinished claimed item never waits on an unfinished one and every wait
// ends whatever the residency of the blocks; a warp claims its next item
// while it works on the current one and always runs what it claimed.  Each
// wait is also bounded: on expiry the kernel raises an error flag, later
// waits and claims return at once and the host reports the failure.  Ring
// data is read through L2 (ld.global.cg: a slot is rewritten every M chunks,
// so L1 copies would be stale).
#include <cuda_runtime.h>

#include "sf_common.cuh"
#include "sf_kernels.h"
#include "sf_tile.cuh"

const SfPipeConfig kSfPipeConfigs[] = {
    // levels, warps, min blocks, lag, ring chunks (streaming: ring planes), streaming, name
    {2, 4, 6, 3, 6, 0, "tile_pipe2_w4"},
    {3, 4, 6, 3, 6, 0, "tile_pipe3_w4"},
    {2, 4, 6, 4, 8, 0, "tile_pipe2_w4_l4"},
    {2, 4, 5, 0, 16, 1, "tile_stream2_w4"},
};
const int kSfPipeConfigCount = sizeof(kSfPipeConfigs) / sizeof(kSfPipeConfigs[0]);

namespace {

// Ring or state-set addressing for one level: input from the previous
// level's ring (IN_RING) or the input set, output to this level's ring
// (OUT_RING) or the output set.  Ring plane of grid plane i: i mod wrap.
template <bool IN_RING, bool OUT_RING>
struct SfRingMem {
    int plane, wrap;
    int i0, r0;  // the item's first plane and its ring plane (i0 mod wrap)
    // ring plane of grid plane i, for i0 - 1 <= i <= i0 + S + 1 (wrap >= S + 2)
    __device__ __forceinline__ int rp(int i) const {
        int r = r0 + (i - i0);
        r += r < 0 ? wrap : 0;
        r -= r >= wrap ? wrap : 0;
        return r;
    }
    __device__ __forceinline__ int in(int i) const { return (IN_RING ? rp(i) : i) * plane; }
    __device__ __forceinline__ int out(int i) const { return (OUT_RING ? rp(i) : i) * plane; }
    __device__ __forceinline__ void before(int) const {}
    __device__ __forceinline__ void after(int) const {}
    __device__ __forceinline__ void ld4(const float* __restrict__ b, int c, float (&v)[4]) const {
        if (IN_RING) {
            const float4 t = __ldcg(reinterpret_cast<const float4*>(b + c));
            v[0] = t.x;
            v[1] = t.y;
            v[2] = t.z;
            v[3] = t.w;
        } else {
            sf_tile::ld4(b, c, v);
        }
    }
    __device__ __forceinline__ float ld1(const float* __restrict__ b, int c) const {
        return IN_RING ? __ldcg(b + c) : __ldg(b + c);
    }
    template <bool WB>
    __device__ __forceinline__ void st4(float* __restrict__ b, int c, const float (&v)[4]) const {
        if (OUT_RING)
            *reinterpret_cast<float4*>(b + c) = make_float4(v[0], v[1], v[2], v[3]);
        else
            __stcs(reinterpret_cast<float4*>(b + c), make_float4(v[0], v[1], v[2], v[3]));
    }
};

__device__ __forceinline__ int ld_relaxed(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Waits until *p != 0 (at most `limit` sleeps), then orders this thread's
// later accesses after the writes the flag publishes.  False when the error
// flag is or gets set.
__device__ bool wait_flag(const int* p, int* err, long long limit) {
    for (long long it = 0;; ++it) {
        if (ld_relaxed(p) != 0) {
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
            return true;
        }
        if (ld_relaxed(err) != 0) return false;
        if (it >= limit) {
            atomicExch(err, 2);
            return false;
        }
        __nanosleep(it < 32 ? 64 : 256);
    }
}

// Completion flag of item (level s, chunk c, tile t), 1-based level.
__device__ __forceinline__ int* done_flag(const SfPipeArgs& P, int s, int c, int t) {
    return P.ctrl + 1 + ((long long)(s - 1) * P.nchunks + c) * P.ntiles + t;
}

// Dependency number d (0..29) of item (s, c, t), or null: d / 5 picks the
// chunk offset (and with d >= 15 the readers of the ring slot), d % 5 the
// tile (itself, -k, +k, -j, +j).
__device__ const int* dep_flag(const SfPipeArgs& P, int s, int c, int t, int d) {
    int lv, cc;
    if (d < 15) {
        if (s == 1) return nullptr;
        lv = s - 1;
        cc = c + d / 5 - 1;
    } else {
        if (s == P.levels) return nullptr;
        lv = s + 1;
        cc = c - P.M + (d - 15) / 5 - 1;
    }
    if (cc < 0 || cc >= P.nchunks) return nullptr;
    const int tk = t % P.ntk, tj = t / P.ntk, ntj = P.ntiles / P.ntk;
    int u = t;
    switch (d % 5) {
        case 1: if (tk == 0) return nullptr; u = t - 1; break;
        case 2: if (tk + 1 >= P.ntk) return nullptr; u = t + 1; break;
        case 3: if (tj == 0) return nullptr; u = t - P.ntk; break;
        case 4: if (tj + 1 >= ntj) return nullptr; u = t + P.ntk; break;
        default: break;
    }
    return done_flag(P, lv, cc, u);
}

template <bool GEOM, bool NU, bool IN_RING, bool OUT_RING>
__device__ __forceinline__ void run_item(const SfTileIo& io, const SfSources& src, int i0, int i1,
                                         int jw, int kw, int plane, int wrap) {
    const SfRingMem<IN_RING, OUT_RING> mem{plane, wrap, i0, i0 % wrap};
    tile4_run<GEOM, 1, false, NU, false>(io, src, i0, i1, jw, kw, mem);
}

// Every warp is its own worker: it claims items (lane 0, one ahead), waits
// for their dependencies (one flag per lane), runs the 32 k x 4 row tile and
// publishes its completion flag; no block-wide barrier is involved.
template <bool GEOM, bool NU, int W, int MINB>
__global__ void __launch_bounds__(32 * W, MINB) k_step_pipe(SfPipeArgs P, SfSources src) {
    using sf_tile::kFull;
    const SfStepArgs& a = P.a;
    const int lane = threadIdx.x;
    if (a.trace_prev != nullptr && blockIdx.x == 0)
        for (int t = threadIdx.y * 32 + lane; t < a.n_probe; t += 32 * W)
            a.trace_prev[t] = a.p[a.probe_cells[t]];
    const int total = P.ngroups * P.ntiles;
    const int plane = a.ny * a.nz;
    const int wrap = P.M * P.S;
    const long long field = (long long)wrap * plane;  // floats per ring field
    int claimed = 0;  // lane 0: the item claimed ahead
    if (lane == 0) claimed = atomicAdd(P.ctrl, 1);
    for (;;) {
        int q = total;
        if (lane == 0) {
            if (ld_relaxed(P.err) == 0) q = claimed;
            if (q < total) claimed = atomicAdd(P.ctrl, 1);  // the next one, while this one runs
        }
        q = __shfl_sync(kFull, q, 0);
        if (q >= total) break;
        const int g = q / P.ntiles, t = q - g * P.ntiles;
        const int code = P.order[g];
        const int s = code >> 24, c = code & 0xffffff;
        bool ok = true;
        if (lane < 30) {
            const int* f = dep_flag(P, s, c, t, lane);
            if (f != nullptr) ok = wait_flag(f, P.err, P.spin_limit);
        } else if (lane == 30 && q == 0 && P.hold != nullptr) {
            ok = wait_flag(P.hold, P.err, P.spin_limit);  // expiry test hook
        }
        if (!__all_sync(kFull, ok)) break;
        const int i0 = c * P.S, i1 = min(i0 + P.S, a.nx);
        const int tk = t % P.ntk, tj = t / P.ntk;

        SfTileIo io;
        io.nx = a.nx;
        io.ny = a.ny;
        io.nz = a.nz;
        io.plane = plane;
        io.cv = a.cv;
        io.cp = a.cp;
        if (s == 1) {
            io.p = a.p;
            io.vx = a.vx;
            io.vy = a.vy;
            io.vz = a.vz;
        } else {
            const float* r = P.ring + (long long)(s - 2) * 4 * field;
            io.p = r;
            io.vx = r + field;
            io.vy = r + 2 * field;
            io.vz = r + 3 * field;
        }
        if (s == P.levels) {
            io.po = a.po;
            io.vxo = a.vxo;
            io.vyo = a.vyo;
            io.vzo = a.vzo;
        } else {
            float* r = P.ring + (long long)(s - 1) * 4 * field;
            io.po = r;
            io.vxo = r + field;
            io.vyo = r + 2 * field;
            io.vzo = r + 3 * field;
        }
        io.flags = a.flags;
        io.dx = a.dx;
        io.dy = a.dy;
        io.dz = a.dz;
        io.src_val = a.src_val != nullptr ? a.src_val + (long long)(s - 1) * src.n : nullptr;
        for (int u = 0; u < 3; ++u) {
            io.nu_cv[u] = a.nu_cv[u];
            io.nu_inv[u] = a.nu_inv[u];
        }
        const int jw = tj * 4, kw = tk * 32;
        if (s == 1 && s == P.levels)
            run_item<GEOM, NU, false, false>(io, src, i0, i1, jw, kw, plane, wrap);
        else if (s == 1)
            run_item<GEOM, NU, false, true>(io, src, i0, i1, jw, kw, plane, wrap);
        else if (s == P.levels)
            run_item<GEOM, NU, true, false>(io, src, i0, i1, jw, kw, plane, wrap);
        else
            run_item<GEOM, NU, true, true>(io, src, i0, i1, jw, kw, plane, wrap);
        __threadfence();
        __syncwarp();
        // probe values of this level's result (kept in its ring)
        if (s < P.levels && P.trace_lvl[s - 1] != nullptr) {
            for (int u = lane; u < a.n_probe; u += 32) {
                const long long cell = a.probe_cells[u];
                const int pi = (int)(cell / plane);
                const int rem = (int)(cell - (long long)pi * plane);
                const int pj = rem / a.nz, pk = rem - pj * a.nz;
                if (pi >= i0 && pi < i1 && pj >= jw && pj < jw + 4 && pk >= kw && pk < kw + 32)
                    P.trace_lvl[s - 1][u] = __ldcg(io.po + (long long)(pi % wrap) * plane + rem);
            }
            __syncwarp();
        }
        if (lane == 0)
            asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(done_flag(P, s, c, t)), "r"(1)
                         : "memory");
    }
}

// Streaming pipeline (k_step_stream): one warp per (level, tile) walks
// planes 0 .. nx-1 of its tile.  Addressing: rings of `wrap` planes (a power
// of two, plane i in slot i & (wrap-1)).  Synchronisation: the warp
// publishes how many planes it has completed every S planes (and before any
// wait); before plane i it needs level s-1's tiles (itself and its four
// neighbours, one lane each) to have completed planes up to i+2, and level
// s+1's tiles to have finished with the slot plane i overwrites (plane
// i - wrap, i.e. completed i - wrap + 1 planes).  A wait for a warp that
// itself waits can only point at lower progress, so with wrap >= S + 3 and
// every warp resident at once (cooperative launch) the chain ends at a warp
// that can advance.
template <bool IN_RING, bool OUT_RING>
struct SfStreamMem {
    const SfPipeArgs& P;  // the launch's parameters (constant bank)
    int plane, s, t;
    int nb;               // this lane's neighbour tile (lanes 0..4), or -1
    int pu, pi, prem;     // this lane's probe: index, plane, offset in the plane (or pu < 0)
    mutable int seen_prev, seen_next, done, published;

    __device__ __forceinline__ int in(int i) const { return (IN_RING ? (i & (P.M - 1)) : i) * plane; }
    __device__ __forceinline__ int out(int i) const { return (OUT_RING ? (i & (P.M - 1)) : i) * plane; }
    __device__ __forceinline__ void ld4(const float* __restrict__ b, int c, float (&v)[4]) const {
        if (IN_RING) {
            const float4 q = __ldcg(reinterpret_cast<const float4*>(b + c));
            v[0] = q.x;
            v[1] = q.y;
            v[2] = q.z;
            v[3] = q.w;
        } else {
            sf_tile::ld4(b, c, v);
        }
    }
    __device__ __forceinline__ float ld1(const float* __restrict__ b, int c) const {
        return IN_RING ? __ldcg(b + c) : __ldg(b + c);
    }
    template <bool WB>
    __device__ __forceinline__ void st4(float* __restrict__ b, int c, const float (&v)[4]) const {
        if (OUT_RING)
            *reinterpret_cast<float4*>(b + c) = make_float4(v[0], v[1], v[2], v[3]);
        else
            __stcs(reinterpret_cast<float4*>(b + c), make_float4(v[0], v[1], v[2], v[3]));
    }
    __device__ __forceinline__ const int* progress(int level) const {  // 1-based level
        return P.ctrl + (long long)(level - 1) * P.ntiles;
    }
    __device__ __forceinline__ void publish() const {
        if (done > published) {
            __threadfence();
            __syncwarp();
            if ((threadIdx.x & 31) == 0)
                asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(progress(s) + t), "r"(done)
                             : "memory");
            published = done;
        }
    }
    __device__ __forceinline__ void before(int i) const {
        const int need_p = i + 3 < P.a.nx ? i + 3 : P.a.nx;
        const int need_n = i - (P.M - 1);
        bool lack = nb >= 0 && ((IN_RING && seen_prev < need_p) || (OUT_RING && seen_next < need_n));
        if (!__any_sync(sf_tile::kFull, lack)) return;
        publish();
        for (long long it = 0; lack; ++it) {
            if (IN_RING) seen_prev = ld_relaxed(progress(s - 1) + nb);
            if (OUT_RING) seen_next = ld_relaxed(progress(s + 1) + nb);
            lack = (IN_RING && seen_prev < need_p) || (OUT_RING && seen_next < need_n);
            if (!lack) break;
            bool give_up = ld_relaxed(P.err) != 0;
            if (!give_up && it >= P.spin_limit) {
                atomicExch(P.err, 2);
                give_up = true;
            }
            if (give_up) {  // the launch is failing: stop waiting, results are void
                seen_prev = seen_next = 0x7fffffff;
                break;
            }
            __nanosleep(it < 32 ? 64 : 256);
        }
        __syncwarp();
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
    }
    __device__ __forceinline__ void after(int i) const {
        done = i + 1;
        if (OUT_RING && P.trace_lvl[s - 1] != nullptr) {
            __syncwarp();
            if (pu >= 0 && pi == i) {
                const float* ring_p = P.ring + (long long)(s - 1) * 4 * P.M * plane;
                P.trace_lvl[s - 1][pu] = __ldcg(ring_p + (i & (P.M - 1)) * plane + prem);
            }
        }
        if (done - published >= P.S || done == P.a.nx) publish();
    }
};

template <bool GEOM, bool NU, bool PF, int W, int MINB>
__global__ void __launch_bounds__(32 * W, MINB) k_step_stream(SfPipeArgs P, SfSources src) {
    __shared__ int s_probe[W][32];
    const SfStepArgs& a = P.a;
    const int lane = threadIdx.x;
    if (a.trace_prev != nullptr && blockIdx.x == 0)
        for (int t = threadIdx.y * 32 + lane; t < a.n_probe; t += 32 * W)
            a.trace_prev[t] = a.p[a.probe_cells[t]];
    const int wid = blockIdx.x * W + threadIdx.y;
    if (wid >= P.levels * P.ntiles) return;  // whole warp; no block barrier follows
    if (P.hold != nullptr && wid == 0) {  // expiry test hook: never satisfied
        bool ok = true;
        if (lane == 0) ok = wait_flag(P.hold, P.err, P.spin_limit);
        if (!__all_sync(sf_tile::kFull, ok)) return;  // the error flag is set
    }
    const int s = wid / P.ntiles + 1, t = wid - (s - 1) * P.ntiles;
    const int tk = t % P.ntk, tj = t / P.ntk, ntj = P.ntiles / P.ntk;
    const int plane = a.ny * a.nz, wrap = P.M;
    const long long field = (long long)wrap * plane;

    SfTileIo io;
    io.nx = a.nx;
    io.ny = a.ny;
    io.nz = a.nz;
    io.plane = plane;
    io.cv = a.cv;
    io.cp = a.cp;
    if (s == 1) {
        io.p = a.p;
        io.vx = a.vx;
        io.vy = a.vy;
        io.vz = a.vz;
    } else {
        const float* r = P.ring + (long long)(s - 2) * 4 * field;
        io.p = r;
        io.vx = r + field;
        io.vy = r + 2 * field;
        io.vz = r + 3 * field;
    }
    if (s == P.levels) {
        io.po = a.po;
        io.vxo = a.vxo;
        io.vyo = a.vyo;
        io.vzo = a.vzo;
    } else {
        float* r = P.ring + (long long)(s - 1) * 4 * field;
        io.po = r;
        io.vxo = r + field;
        io.vyo = r + 2 * field;
        io.vzo = r + 3 * field;
    }
    io.flags = a.flags;
    io.dx = a.dx;
    io.dy = a.dy;
    io.dz = a.dz;
    io.src_val = a.src_val != nullptr ? a.src_val + (long long)(s - 1) * src.n : nullptr;
    for (int u = 0; u < 3; ++u) {
        io.nu_cv[u] = a.nu_cv[u];
        io.nu_inv[u] = a.nu_inv[u];
    }
    int nb = -1;  // lanes 0..4: the tile itself, -k, +k, -j, +j
    if (lane == 0) nb = t;
    else if (lane == 1 && tk > 0) nb = t - 1;
    else if (lane == 2 && tk + 1 < P.ntk) nb = t + 1;
    else if (lane == 3 && tj > 0) nb = t - P.ntk;
    else if (lane == 4 && tj + 1 < ntj) nb = t + P.ntk;
    // probes in this tile column (at most 32, checked by the host)
    float* trace = s < P.levels ? P.trace_lvl[s - 1] : nullptr;
    int pu = -1, ppi = 0, prem = 0;
    if (trace != nullptr) {
        int cnt = 0;
        for (int base = 0; base < a.n_probe; base += 32) {
            const int u = base + lane;
            bool hit = false;
            if (u < a.n_probe) {
                const long long cell = a.probe_cells[u];
                const int rem = (int)(cell % plane);
                const int pj = rem / a.nz, pk = rem - pj * a.nz;
                hit = (pj >> 2) == tj && (pk >> 5) == tk;
            }
            const unsigned m = __ballot_sync(sf_tile::kFull, hit);
            const int slot = cnt + __popc(m & ((1u << lane) - 1u));
            if (hit && slot < 32) s_probe[threadIdx.y][slot] = u;
            cnt += __popc(m);
        }
        __syncwarp();
        if (lane < cnt && lane < 32) {
            pu = s_probe[threadIdx.y][lane];
            const long long cell = a.probe_cells[pu];
            ppi = (int)(cell / plane);
            prem = (int)(cell - (long long)ppi * plane);
        }
    }
    const int jw = tj * 4, kw = tk * 32;
#define SF_STREAM_RUN(IN, OUT)                                                          \
    {                                                                                  \
        const SfStreamMem<IN, OUT> mem{P, plane, s, t, nb, pu, ppi, prem, 0, 0, 0, 0};  \
        tile4_run<GEOM, 1, PF, NU, false>(io, src, 0, a.nx, jw, kw, mem);              \
    }
    if (s == 1) SF_STREAM_RUN(false, true)  // levels >= 2
    else if (s == P.levels) SF_STREAM_RUN(true, false)
    else SF_STREAM_RUN(true, true)
#undef SF_STREAM_RUN
}

template <bool GEOM, bool NU, bool PF, int W, int MINB>
int launch_stream_k(const SfPipeArgs& P, const SfSources& src, int grid, cudaStream_t st) {
    auto kern = k_step_stream<GEOM, NU, PF, W, MINB>;
    int per_sm = 0, dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * W, 0) != cudaSuccess ||
        (long long)per_sm * sms < grid)
        return SF_PIPE_NOFIT;
    SfPipeArgs p = P;
    SfSources s = src;
    void* args[] = {&p, &s};
    const cudaError_t e = cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(32, W, 1),
                                                      args, 0, st);
    return e == cudaSuccess ? 0 : sf_fail_cuda(e, "k_step_stream launch", __FILE__, __LINE__);
}

template <bool PF, int W, int MINB>
int launch_stream_w(const SfPipeArgs& P, const SfSources& src, bool geom, int grid, cudaStream_t st) {
    const bool nu = P.a.nu_cv[0] != nullptr;
    if (nu) return geom ? launch_stream_k<true, true, PF, W, MINB>(P, src, grid, st)
                        : launch_stream_k<false, true, PF, W, MINB>(P, src, grid, st);
    return geom ? launch_stream_k<true, false, PF, W, MINB>(P, src, grid, st)
                : launch_stream_k<false, false, PF, W, MINB>(P, src, grid, st);
}

template <bool GEOM, bool NU, int W, int MINB>
int launch_cfg(const SfPipeArgs& P, const SfSources& src, int grid, cudaStream_t st) {
    k_step_pipe<GEOM, NU, W, MINB><<<grid, dim3(32, W, 1), 0, st>>>(P, src);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_step_pipe launch failed");
}

template <int W, int MINB>
int launch_wm(const SfPipeArgs& P, const SfSources& src, bool geom, int grid, cudaStream_t st) {
    const bool nu = P.a.nu_cv[0] != nullptr;
    if (nu) return geom ? launch_cfg<true, true, W, MINB>(P, src, grid, st)
                        : launch_cfg<false, true, W, MINB>(P, src, grid, st);
    return geom ? launch_cfg<true, false, W, MINB>(P, src, grid, st)
                : launch_cfg<false, false, W, MINB>(P, src, grid, st);
}

template <int W, int MINB>
int blocks_wm(bool geom, bool nu) {
    int per_sm = 0, dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e;
    if (nu) e = geom ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_pipe<true, true, W, MINB>, 32 * W, 0)
                     : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_pipe<false, true, W, MINB>, 32 * W, 0);
    else e = geom ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_pipe<true, false, W, MINB>, 32 * W, 0)
                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_pipe<false, false, W, MINB>, 32 * W, 0);
    if (e != cudaSuccess || per_sm < 1) per_sm = 1;
    return per_sm * (sms > 0 ? sms : 1);
}

}  // namespace

template <bool PF>
int blocks_stream(bool geom, bool nu) {
    int per_sm = 0, dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e;
    if (nu) e = geom ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_stream<true, true, PF, 4, 5>, 128, 0)
                     : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_stream<false, true, PF, 4, 5>, 128, 0);
    else e = geom ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_stream<true, false, PF, 4, 5>, 128, 0)
                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_stream<false, false, PF, 4, 5>, 128, 0);
    if (e != cudaSuccess) per_sm = 0;
    return per_sm * sms;
}

int sf_pipe_grid(int cfg, bool geom, bool nu) {
    const SfPipeConfig& c = kSfPipeConfigs[cfg];
    if (c.stream) return blocks_stream<false>(geom, nu);
    switch (c.warps) {
        case 8: return blocks_wm<8, 3>(geom, nu);
        default: return blocks_wm<4, 6>(geom, nu);
    }
}

int sf_launch_step_stream(const SfPipeArgs& P, const SfSources& src, bool geom, int cfg,
                          cudaStream_t st) {
    if (cfg < 0 || cfg >= kSfPipeConfigCount || !kSfPipeConfigs[cfg].stream)
        return sf_fail("k_step_stream: bad configuration");
    const int W = 4;  // every streaming configuration: 4 warps per block, min blocks 5
    const int grid = (P.levels * P.ntiles + W - 1) / W;
    return launch_stream_w<false, 4, 5>(P, src, geom, grid, st);
}

int sf_launch_step_pipe(const SfPipeArgs& P, const SfSources& src, bool geom, int cfg, int grid,
                        cudaStream_t st) {
    if (cfg < 0 || cfg >= kSfPipeConfigCount) return sf_fail("k_step_pipe: bad configuration");
    if (grid < 1) grid = 1;
    switch (kSfPipeConfigs[cfg].warps) {
        case 8: return launch_wm<8, 3>(P, src, geom, grid, st);
        default: return launch_wm<4, 6>(P, src, geom, grid, st);
    }
}
