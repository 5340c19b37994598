// sf_step_tb.cu -- two time steps per pass over the state: temporal
// blocking with overlapped tiles.
//
// One launch advances the state by two steps.  A block owns an output tile
// of TJ rows x TK columns (j, k) over a chunk of planes i0 .. i1-1 and
// marches it along i.  At plane iteration t it computes the first step
// ("level 1") of plane t and the second step ("level 2") of plane t-1:
//
//   V1  level-1 face velocities of plane t on the tile grown by 2 cells on
//       the low j/k sides and 1 on the high ones (rows j0-2 .. j0+TJ,
//       columns k0-2 .. k0+TK): v0 + cv (p0[+1] - p0), rigid faces zeroed;
//   L1  level-1 pressure of plane t on the tile grown by 1 on every side;
//   V2  level-2 face velocities of plane t-1 on the tile grown by 1 on the
//       low sides, from the level-1 state of planes t-1 and t;
//   O   level-2 pressure of plane t-1 on the tile; the level-2 state of the
//       tile is the only thing written to HBM.
//
// The halo cells of level 1 are the ones the neighbouring blocks own; each
// block recomputes them with the same operations (bit-identical values), so
// no block waits for another and HBM sees one read of the input set and one
// write of the output set per two steps.  The planes of p0 (with a 2-cell
// halo) arrive in shared memory by cp.async two planes ahead; v0 and the
// flag bytes of each thread's own cells are loaded one plane ahead into
// registers.  In-plane neighbour values go through shared memory (three
// block barriers per plane), values a thread needs for its own cells (the
// x faces carried along i, level-1 state of the previous plane) stay in its
// registers: every compute loop uses one mapping of the grown tile onto the
// threads.
//
// Per-cell arithmetic is the single-step kernels' (sf_tile.cuh, after
// fdtd_step.cpp:15-212, pml.cpp:47-149, core/solver.py:2413-2421): FP32
// without contraction, PML on p as three rounded products, sources in FP64
// rounded once, in source order, on air cells -- so two steps of this kernel
// equal two single steps bit for bit.  Level-1 probe samples are written
// from shared memory by the block owning the probe cell; the level-2 ones
// are gathered from the output set like a single step's.
//
// Uniform grids without ADE poles, microphones, plane boundaries or weighted
// sources only (the caller falls back to single steps otherwise); cell
// offsets within a plane and plane bases fit 32 / 64 bits as used below.
#include <cuda_runtime.h>

#include <climits>

#include "sf_common.cuh"
#include "sf_kernels.h"

namespace {

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// 4-byte asynchronous copy global -> shared; zero-filled when !in (no bytes
// are read then; the source address is clamped to the field's base).
__device__ __forceinline__ void cp4(float* dst, const float* src, bool in) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(smem_u32(dst)), "l"(src),
                 "r"(in ? 4u : 0u)
                 : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Pressure update of one cell (update_pressure + PML + sources), the
// operations of tile4_run in the same order.
__device__ __forceinline__ float pressure(float pc, float cp, float uxh, float uxl, float uyh,
                                          float uyl, float uzh, float uzl, bool air, float di,
                                          float dj, float dk) {
    const float dx_ = f_sub(uxh, uxl), dy_ = f_sub(uyh, uyl), dz_ = f_sub(uzh, uzl);
    float pn = air ? f_add(pc, f_mul(cp, f_add(f_add(dx_, dy_), dz_))) : 0.0f;
    return f_mul(f_mul(f_mul(pn, di), dj), dk);
}

__device__ __forceinline__ float inject(float pn, const SfSources& src, unsigned smask,
                                       const double* val, int i, int j, int k, bool air) {
    for (unsigned m = smask; m != 0; m &= m - 1) {
        const int q = __ffs(m) - 1;
        const sf_source& S = src.s[q];
        bool hit;
        if (S.kind == 0) hit = (i == S.a) && (j == S.b) && (k == S.c);
        else if (S.a == 0) hit = (i == S.b);
        else if (S.a == 1) hit = (j == S.b);
        else hit = (k == S.b);
        if (hit && air) pn = __double2float_rn(d_add((double)pn, val[q]));
    }
    return pn;
}

template <bool GEOM, int TJ, int TK, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_step_tb2(SfStepArgs a, SfSources src, int ich,
                                                       float* __restrict__ trace1) {
    constexpr int WA = TK + 4, HA = TJ + 4, SA = WA * HA;  // shared plane: rows j0-2.., cols k0-2..
    constexpr int WV = TK + 3, HV = TJ + 3, NV = WV * HV;  // the compute mapping (V1 region)
    constexpr int M = (NV + NT - 1) / NT;                  // cells per thread
    extern __shared__ __align__(16) float sm[];
    float* P0 = sm;            // p0, 3 plane slots (t, t+1, t+2 in flight)
    float* U1y = P0 + 3 * SA;  // level-1 y / z faces of plane t (pre-decay)
    float* U1z = U1y + SA;
    float* P1 = U1z + SA;      // level-1 pressure, 2 plane slots (t-1, t)
    float* U2y = P1 + 2 * SA;  // level-2 y / z faces of plane t-1 (pre-decay)
    float* U2z = U2y + SA;

    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int plane = ny * nz;
    const int tid = threadIdx.x;
    const int k0 = blockIdx.x * TK, j0 = blockIdx.y * TJ;
    const int chunk = a.reverse ? (int)(gridDim.z - 1 - blockIdx.z) : (int)blockIdx.z;
    const int i0 = chunk * ich;
    const int i1 = min(i0 + ich, nx);
    const float cv = a.cv, cp = a.cp;
    const bool no_flags = !GEOM;

    if (a.trace_prev != nullptr && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0)
        for (int q = tid; q < a.n_probe; q += NT) a.trace_prev[q] = a.p[a.probe_cells[q]];

    // Sources that can reach this block's cells (grown tile, planes i0-1 .. i1).
    unsigned smask = 0;
    for (int q = 0; q < src.n; ++q) {
        const sf_source& S = src.s[q];
        bool can;
        const bool ii = S.a >= i0 - 1 && S.a <= i1;
        if (S.kind == 0)
            can = ii && S.b >= j0 - 2 && S.b <= j0 + TJ && S.c >= k0 - 2 && S.c <= k0 + TK;
        else if (S.a == 0) can = S.b >= i0 - 1 && S.b <= i1;
        else if (S.a == 1) can = S.b >= j0 - 2 && S.b <= j0 + TJ;
        else can = S.b >= k0 - 2 && S.b <= k0 + TK;
        if (can) smask |= 1u << q;
    }
    const double* val1 = a.src_val;
    const double* val2 = a.src_val != nullptr ? a.src_val + src.n : nullptr;

    // Own cells of the mapping: shared offset, in-plane global offset, region bits.
    int so[M], go[M], jj[M], kk[M];
    unsigned ing = 0, inl1 = 0, inv2 = 0, ino = 0;
    float djv[M], dkv[M];
#pragma unroll
    for (int m = 0; m < M; ++m) {
        const int idx = tid + m * NT;
        const int r = idx / WV, c = idx - (idx / WV) * WV;
        const int j = j0 - 2 + r, k = k0 - 2 + c;
        so[m] = r * WA + c;
        jj[m] = j;
        kk[m] = k;
        const bool g = idx < NV && j >= 0 && j < ny && k >= 0 && k < nz;
        go[m] = g ? j * nz + k : 0;
        if (g) ing |= 1u << m;
        if (idx < NV && r >= 1 && c >= 1) inl1 |= 1u << m;
        if (idx < NV && r >= 1 && r <= TJ + 1 && c >= 1 && c <= TK + 1) inv2 |= 1u << m;
        if (idx < NV && r >= 2 && r <= TJ + 1 && c >= 2 && c <= TK + 1) ino |= 1u << m;
        djv[m] = g ? a.dy[j] : 1.0f;
        dkv[m] = g ? a.dz[k] : 1.0f;
    }

    // p0 plane `ip` (zeros outside the grid) into slot `slot`, asynchronously.
    auto load_p0 = [&](int ip, int slot) {
        float* dst = P0 + slot * SA;
        const bool pin = ip >= 0 && ip < nx;
        const float* base = a.p + (pin ? (long long)ip * plane : 0LL);
        for (int q = tid; q < SA; q += NT) {
            const int r = q / WA, c = q - (q / WA) * WA;
            const int j = j0 - 2 + r, k = k0 - 2 + c;
            const bool in = pin && j >= 0 && j < ny && k >= 0 && k < nz;
            cp4(dst + q, in ? base + j * nz + k : a.p, in);
        }
        cp_commit();
    };

    const int tstart = i0 > 0 ? i0 - 1 : 0;
    // v0 and flags of own cells, one plane ahead in registers
    float nvx[M], nvy[M], nvz[M];
    uint32_t nfl[M];
    auto load_v0 = [&](int ip) {
        const bool pin = ip < nx;
        const long long base = (long long)ip * plane;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            nvx[m] = nvy[m] = nvz[m] = 0.0f;
            nfl[m] = SF_ALL;
            if (pin && (ing >> m & 1u)) {
                nvx[m] = __ldg(a.vx + base + go[m]);
                nvy[m] = __ldg(a.vy + base + go[m]);
                nvz[m] = __ldg(a.vz + base + go[m]);
                if (!no_flags) nfl[m] = __ldg(a.flags + base + go[m]);
            }
        }
    };

    // Carried per own cell: level-1 faces of the previous plane (pre-decay),
    // level-1 pressure of the previous plane, the level-2 x face of the
    // plane before that, flags of the previous plane.
    float u1xm[M], u1ym[M], u1zm[M], p1m[M], u2xm[M];
    uint32_t flm[M];
#pragma unroll
    for (int m = 0; m < M; ++m) {
        u1xm[m] = u1ym[m] = u1zm[m] = p1m[m] = u2xm[m] = 0.0f;
        flm[m] = SF_ALL;
        // level-1 x face below the first plane: from plane tstart-1 of the input
        if (tstart > 0 && (ing >> m & 1u)) {
            const long long b = (long long)(tstart - 1) * plane + go[m];
            const float pl = __ldg(a.p + b), ph = __ldg(a.p + b + plane);
            float u = face_update(__ldg(a.vx + b), cv, ph, pl);
            if (!no_flags && !(__ldg(a.flags + b) & SF_OPX)) u = 0.0f;
            u1xm[m] = u;
        }
    }
    load_p0(tstart, tstart % 3);
    load_p0(tstart + 1, (tstart + 1) % 3);
    load_v0(tstart);
    cp_wait_all();
    __syncthreads();

    for (int t = tstart; t <= i1; ++t) {
        const bool l1 = t < nx;                    // level 1 of plane t exists
        const bool l2 = t >= tstart + 1;           // level 2 of plane t-1 (x face or output)
        const bool out = t - 1 >= i0 && t - 1 < i1;  // plane t-1 is written
        const int s0 = t % 3, s1 = (t + 1) % 3, s2 = (t + 2) % 3;
        const float* p0c = P0 + s0 * SA;
        const float* p0n = P0 + s1 * SA;
        float* p1c = P1 + (t & 1) * SA;
        const float* p1p = P1 + ((t + 1) & 1) * SA;  // plane t-1
        // ---- phase 1: next p0 plane in flight, next v0 loads, V1 of plane t
        if (t + 1 <= i1) load_p0(t + 2, s2);
        float vx[M], vy[M], vz[M];
        uint32_t fl[M];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            vx[m] = nvx[m];
            vy[m] = nvy[m];
            vz[m] = nvz[m];
            fl[m] = nfl[m];
        }
        if (t + 1 <= i1) load_v0(t + 1);
        float u1x[M], u1y[M], u1z[M];
        const float di1 = l1 ? a.dx[t] : 1.0f;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            u1x[m] = u1y[m] = u1z[m] = 0.0f;
            if (l1 && (ing >> m & 1u)) {
                const float pc = p0c[so[m]];
                float ux = vx[m], uy = vy[m], uz = vz[m];
                if (t < nx - 1) {
                    ux = face_update(ux, cv, p0n[so[m]], pc);
                    if (!no_flags && !(fl[m] & SF_OPX)) ux = 0.0f;
                }
                if (jj[m] < ny - 1) {
                    uy = face_update(uy, cv, p0c[so[m] + WA], pc);
                    if (!no_flags && !(fl[m] & SF_OPY)) uy = 0.0f;
                }
                if (kk[m] < nz - 1) {
                    uz = face_update(uz, cv, p0c[so[m] + 1], pc);
                    if (!no_flags && !(fl[m] & SF_OPZ)) uz = 0.0f;
                }
                u1x[m] = ux;
                u1y[m] = uy;
                u1z[m] = uz;
            }
            if (m * NT + tid < NV) {
                U1y[so[m]] = u1y[m];
                U1z[so[m]] = u1z[m];
            }
        }
        __syncthreads();  // A
        // ---- phase 2: L1, level-1 pressure of plane t
        float p1[M];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            p1[m] = 0.0f;
            if (l1 && (ing >> m & 1u) && (inl1 >> m & 1u)) {
                const bool air = no_flags || (fl[m] & SF_AIR);
                float pn = pressure(p0c[so[m]], cp, u1x[m], u1xm[m], u1y[m], U1y[so[m] - WA],
                                    u1z[m], U1z[so[m] - 1], air, di1, djv[m], dkv[m]);
                if (smask) pn = inject(pn, src, smask, val1, t, jj[m], kk[m], air);
                p1[m] = pn;
            }
            if (m * NT + tid < NV) p1c[so[m]] = p1[m];
        }
        __syncthreads();  // B
        // ---- phase 3: level-1 probe samples of plane t; V2 of plane t-1
        if (trace1 != nullptr && l1 && t >= i0 && t < i1) {
            for (int q = tid; q < a.n_probe; q += NT) {
                const long long cell = a.probe_cells[q];
                const int pi = (int)(cell / plane);
                if (pi != t) continue;
                const int rem = (int)(cell - (long long)pi * plane);
                const int pj = rem / nz, pk = rem - (rem / nz) * nz;
                if (pj >= j0 && pj < j0 + TJ && pk >= k0 && pk < k0 + TK)
                    trace1[q] = p1c[(pj - j0 + 2) * WA + (pk - k0 + 2)];
            }
        }
        float u2x[M], u2y[M], u2z[M];
        const float dxm = (l2 && t - 1 < nx) ? a.dx[t - 1] : 1.0f;
        if (l2) {
#pragma unroll
            for (int m = 0; m < M; ++m) {
                u2x[m] = u2y[m] = u2z[m] = 0.0f;
                if ((ing >> m & 1u) && (inv2 >> m & 1u)) {
                    const float pc = p1m[m];  // p1 of plane t-1
                    float ux = f_mul(u1xm[m], dxm), uy = f_mul(u1ym[m], djv[m]),
                          uz = f_mul(u1zm[m], dkv[m]);  // the level-1 state after its PML
                    if (t - 1 < nx - 1) {
                        ux = face_update(ux, cv, p1[m], pc);
                        if (!no_flags && !(flm[m] & SF_OPX)) ux = 0.0f;
                    }
                    if (jj[m] < ny - 1) {
                        uy = face_update(uy, cv, p1p[so[m] + WA], pc);
                        if (!no_flags && !(flm[m] & SF_OPY)) uy = 0.0f;
                    }
                    if (kk[m] < nz - 1) {
                        uz = face_update(uz, cv, p1p[so[m] + 1], pc);
                        if (!no_flags && !(flm[m] & SF_OPZ)) uz = 0.0f;
                    }
                    u2x[m] = ux;
                    u2y[m] = uy;
                    u2z[m] = uz;
                }
                if (m * NT + tid < NV) {
                    U2y[so[m]] = u2y[m];
                    U2z[so[m]] = u2z[m];
                }
            }
        }
        cp_wait_all();    // p0 of plane t+2 has landed (read from the next iteration on)
        __syncthreads();  // C
        // ---- phase 4: O, level-2 pressure of plane t-1, written to HBM
        if (l2) {
            const long long base = (long long)(t - 1) * plane;
#pragma unroll
            for (int m = 0; m < M; ++m) {
                if (out && (ing >> m & 1u) && (ino >> m & 1u)) {
                    const bool air = no_flags || (flm[m] & SF_AIR);
                    float pn = pressure(p1m[m], cp, u2x[m], u2xm[m], u2y[m], U2y[so[m] - WA],
                                        u2z[m], U2z[so[m] - 1], air, dxm, djv[m], dkv[m]);
                    if (smask) pn = inject(pn, src, smask, val2, t - 1, jj[m], kk[m], air);
                    const long long c = base + go[m];
                    __stcs(a.po + c, pn);
                    __stcs(a.vxo + c, f_mul(u2x[m], dxm));
                    __stcs(a.vyo + c, f_mul(u2y[m], djv[m]));
                    __stcs(a.vzo + c, f_mul(u2z[m], dkv[m]));
                }
                u2xm[m] = u2x[m];
            }
        }
        // carry plane t's level-1 state into the next iteration
#pragma unroll
        for (int m = 0; m < M; ++m) {
            u1xm[m] = u1x[m];
            u1ym[m] = u1y[m];
            u1zm[m] = u1z[m];
            p1m[m] = p1[m];
            flm[m] = fl[m];
        }
    }
}

// Shared memory of one block: 9 planes of the grown tile.
template <int TJ, int TK>
constexpr size_t tb_smem() {
    return sizeof(float) * 9 * (TK + 4) * (TJ + 4);
}

template <int TJ, int TK, int NT, int MINB>
int launch_tb(const SfStepArgs& a, const SfSources& src, bool geom, int ich, float* trace1,
              cudaStream_t st) {
    constexpr size_t smem = tb_smem<TJ, TK>();
    auto kern = geom ? k_step_tb2<true, TJ, TK, NT, MINB> : k_step_tb2<false, TJ, TK, NT, MINB>;
    if (smem > 48 * 1024) {  // once per device and variant
        static bool attr_set[64][2] = {};
        int dev = 0;
        cudaGetDevice(&dev);
        if (dev < 0 || dev >= 64) return sf_fail("k_step_tb2: device ordinal out of range");
        if (!attr_set[dev][geom]) {
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem) != cudaSuccess)
                return sf_fail("k_step_tb2: shared memory attribute");
            attr_set[dev][geom] = true;
        }
    }
    dim3 grd((a.nz + TK - 1) / TK, (a.ny + TJ - 1) / TJ, (a.nx + ich - 1) / ich);
    kern<<<grd, NT, smem, st>>>(a, src, ich, trace1);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_step_tb2 launch failed");
}

}  // namespace

// Two-step configurations: output tile rows x columns, threads, min blocks.
const SfTbConfig kSfTbConfigs[] = {
    {8, 80, 320, 2, "tb2_j8_k80"},
    {16, 80, 544, 1, "tb2_j16_k80"},
    {8, 60, 256, 3, "tb2_j8_k60"},
    {12, 64, 384, 2, "tb2_j12_k64"},
};
const int kSfTbConfigCount = sizeof(kSfTbConfigs) / sizeof(kSfTbConfigs[0]);

bool sf_tb_supported(const SfStepArgs& a) {
    return a.nu_cv[0] == nullptr && (long long)a.ny * a.nz + 2LL * a.nz + 8 < (long long)INT_MAX &&
           a.nx >= 1;
}

int sf_launch_step_tb(const SfStepArgs& a, const SfSources& src, bool geom, int cfg, int ich,
                      float* trace1, cudaStream_t st) {
    if (ich < 1) ich = 1;
    switch (cfg) {
        case 0: return launch_tb<8, 80, 320, 2>(a, src, geom, ich, trace1, st);
        case 1: return launch_tb<16, 80, 544, 1>(a, src, geom, ich, trace1, st);
        case 2: return launch_tb<8, 60, 256, 3>(a, src, geom, ich, trace1, st);
        case 3: return launch_tb<12, 64, 384, 2>(a, src, geom, ich, trace1, st);
    }
    return sf_fail("k_step_tb2: bad configuration");
}
