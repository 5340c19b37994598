// sf_step_col.cu -- the fused step as independent thread columns along i.
//
// Same per-cell arithmetic as k_step (sf_step.cu), which restates the
// reference passes listed there.  Each thread owns VEC consecutive cells
// along k (VEC = 2 / 4: one float2 / float4 per field, needs nz % VEC == 0)
// in one j row, and walks a chunk of i planes with no block barrier:
//   * the plane-(i+1) velocities and flags and p(i+2) are loaded one step
//     ahead, so their latency overlaps the current plane's arithmetic;
//   * the new x-face velocity and the pressure of plane i are carried in
//     registers into plane i+1;
//   * j +- 1 and k +- 1 neighbours are read straight from global memory and
//     mostly hit L1 (the block's other threads read the same lines).
// DRAM traffic per cell and step: 17 bytes read (p, vx, vy, vz, flags) and
// 16 written, plus one plane of re-reads per chunk of i planes.
//
// The family is templated on the vector width, the block height (rows of 32
// threads), a minimum resident-block count (register cap) and streaming
// (evict-first) stores; sf_plan_autotune picks the fastest for a grid.
#include <cuda_runtime.h>

#include "sf_common.cuh"
#include "sf_kernels.h"

namespace {

template <int VEC>
__device__ __forceinline__ void load_f(const float* __restrict__ base, long long c, float (&v)[VEC]) {
    if constexpr (VEC == 4) {
        const float4 t = __ldg(reinterpret_cast<const float4*>(base + c));
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    } else if constexpr (VEC == 2) {
        const float2 t = __ldg(reinterpret_cast<const float2*>(base + c));
        v[0] = t.x; v[1] = t.y;
    } else {
        v[0] = __ldg(base + c);
    }
}

template <int VEC>
__device__ __forceinline__ void load_b(const uint8_t* __restrict__ base, long long c,
                                       uint8_t (&v)[VEC]) {
    if constexpr (VEC == 4) {
        const uchar4 t = __ldg(reinterpret_cast<const uchar4*>(base + c));
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    } else if constexpr (VEC == 2) {
        const uchar2 t = __ldg(reinterpret_cast<const uchar2*>(base + c));
        v[0] = t.x; v[1] = t.y;
    } else {
        v[0] = __ldg(base + c);
    }
}

template <int VEC, bool CS>
__device__ __forceinline__ void store_f(float* __restrict__ base, long long c, const float (&v)[VEC]) {
    if constexpr (VEC == 4) {
        const float4 t = make_float4(v[0], v[1], v[2], v[3]);
        if (CS) __stcs(reinterpret_cast<float4*>(base + c), t);
        else *reinterpret_cast<float4*>(base + c) = t;
    } else if constexpr (VEC == 2) {
        const float2 t = make_float2(v[0], v[1]);
        if (CS) __stcs(reinterpret_cast<float2*>(base + c), t);
        else *reinterpret_cast<float2*>(base + c) = t;
    } else {
        if (CS) __stcs(base + c, v[0]);
        else base[c] = v[0];
    }
}

template <bool GEOM, int VEC, int BY, int MINB, bool CS>
__global__ void __launch_bounds__(32 * BY, MINB) k_step_col(SfStepArgs a, SfSources src, int ich) {
    const int k = (blockIdx.x * 32 + threadIdx.x) * VEC;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    // On alternate steps the chunks are dispatched from high i to low i, so a
    // step starts on the planes the previous step wrote last (still in L2).
    const int chunk = a.reverse ? (int)(gridDim.z - 1 - blockIdx.z) : (int)blockIdx.z;
    const int i0 = chunk * ich;
    const int i1 = min(i0 + ich, nx);

    if (a.trace_prev != nullptr && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0) {
        for (int t = threadIdx.y * 32 + threadIdx.x; t < a.n_probe; t += 32 * BY)
            a.trace_prev[t] = a.p[a.probe_cells[t]];
    }
    if (k >= nz || j >= ny) return;

    const long long plane = a.plane;
    const long long col = (long long)j * nz + k;
    const float cv = a.cv, cp = a.cp;
    const float dj = a.dy[j];
    float dk[VEC];
#pragma unroll
    for (int e = 0; e < VEC; ++e) dk[e] = a.dz[k + e];
    const bool has_jm = j > 0, has_jp = j < ny - 1, has_km = k > 0, has_kp = k + VEC < nz;
    // Sources that can reach this thread's column of cells, in source order:
    // a point source in this (j, k) range, a plane across i, a plane at this
    // j, or a plane at one of this thread's k.
    unsigned smask = 0;
    for (int q = 0; q < src.n; ++q) {
        const sf_source& S = src.s[q];
        bool can;
        if (S.kind == 0) can = (S.b == j) && (S.c >= k) && (S.c < k + VEC);
        else if (S.a == 0) can = true;
        else if (S.a == 1) can = (S.b == j);
        else can = (S.b >= k) && (S.b < k + VEC);
        if (can) smask |= 1u << q;
    }

    float pc[VEC], pn[VEC], vx[VEC], vy[VEC], vz[VEC], vxm[VEC];
    uint8_t fc[VEC];
    {
        const long long c = (long long)i0 * plane + col;
        load_f<VEC>(a.p, c, pc);
        load_f<VEC>(a.vx, c, vx);
        load_f<VEC>(a.vy, c, vy);
        load_f<VEC>(a.vz, c, vz);
        if (GEOM) {
            load_b<VEC>(a.flags, c, fc);
        } else {
#pragma unroll
            for (int e = 0; e < VEC; ++e) fc[e] = SF_ALL;
        }
        if (i0 + 1 < nx) {
            load_f<VEC>(a.p, c + plane, pn);
        } else {
#pragma unroll
            for (int e = 0; e < VEC; ++e) pn[e] = 0.0f;
        }
#pragma unroll
        for (int e = 0; e < VEC; ++e) vxm[e] = 0.0f;
        if (i0 > 0) {  // chunk start: low x face from plane i0-1
            float pm[VEC], vm[VEC];
            uint8_t fm[VEC];
            load_f<VEC>(a.p, c - plane, pm);
            load_f<VEC>(a.vx, c - plane, vm);
            if (GEOM) load_b<VEC>(a.flags, c - plane, fm);
#pragma unroll
            for (int e = 0; e < VEC; ++e) {
                vxm[e] = face_update(vm[e], cv, pc[e], pm[e]);
                if (GEOM && !(fm[e] & SF_OPX)) vxm[e] = 0.0f;
            }
        }
    }

    for (int i = i0; i < i1; ++i) {
        const long long c = (long long)i * plane + col;
        // next plane's state (loaded now, used next iteration)
        float pnn[VEC], vxn[VEC], vyn[VEC], vzn[VEC];
        uint8_t fnn[VEC];
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            pnn[e] = 0.0f;
            vxn[e] = vyn[e] = vzn[e] = 0.0f;
            fnn[e] = SF_ALL;
        }
        if (i + 1 < i1) {
            load_f<VEC>(a.vx, c + plane, vxn);
            load_f<VEC>(a.vy, c + plane, vyn);
            load_f<VEC>(a.vz, c + plane, vzn);
            if (GEOM) load_b<VEC>(a.flags, c + plane, fnn);
            if (i + 2 < nx) load_f<VEC>(a.p, c + 2 * plane, pnn);
        }
        // in-plane neighbours (L1)
        float pjm[VEC], pjp[VEC], vyjm[VEC];
        uint8_t fjm[VEC];
        if (has_jm) {
            load_f<VEC>(a.p, c - nz, pjm);
            load_f<VEC>(a.vy, c - nz, vyjm);
            if (GEOM) load_b<VEC>(a.flags, c - nz, fjm);
        }
        if (has_jp) load_f<VEC>(a.p, c + nz, pjp);
        float pkm = 0.0f, vzkm = 0.0f, pkp = 0.0f;
        uint8_t fkm = SF_ALL;
        if (has_km) {
            pkm = __ldg(a.p + c - 1);
            vzkm = __ldg(a.vz + c - 1);
            if (GEOM) fkm = __ldg(a.flags + c - 1);
        }
        if (has_kp) pkp = __ldg(a.p + c + VEC);

        float ux[VEC], uy[VEC], uz[VEC], uym[VEC], uzm[VEC];
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            ux[e] = vx[e];
            if (i < nx - 1) {
                ux[e] = face_update(vx[e], cv, pn[e], pc[e]);
                if (GEOM && !(fc[e] & SF_OPX)) ux[e] = 0.0f;
            }
            uy[e] = vy[e];
            if (has_jp) {
                uy[e] = face_update(vy[e], cv, pjp[e], pc[e]);
                if (GEOM && !(fc[e] & SF_OPY)) uy[e] = 0.0f;
            }
            uz[e] = vz[e];
            if (k + e < nz - 1) {
                const float phi = (e + 1 < VEC) ? pc[e + 1] : pkp;
                uz[e] = face_update(vz[e], cv, phi, pc[e]);
                if (GEOM && !(fc[e] & SF_OPZ)) uz[e] = 0.0f;
            }
            uym[e] = 0.0f;
            if (has_jm) {
                uym[e] = face_update(vyjm[e], cv, pc[e], pjm[e]);
                if (GEOM && !(fjm[e] & SF_OPY)) uym[e] = 0.0f;
            }
        }
        uzm[0] = 0.0f;
        if (has_km) {
            uzm[0] = face_update(vzkm, cv, pc[0], pkm);
            if (GEOM && !(fkm & SF_OPZ)) uzm[0] = 0.0f;
        }
#pragma unroll
        for (int e = 1; e < VEC; ++e) uzm[e] = uz[e - 1];

        const float di = a.dx[i];
        float po[VEC], ox[VEC], oy[VEC], oz[VEC];
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            const bool air = (fc[e] & SF_AIR) != 0;
            float pnew = air ? f_add(pc[e], f_mul(cp, f_add(f_add(f_sub(ux[e], vxm[e]),
                                                                  f_sub(uy[e], uym[e])),
                                                            f_sub(uz[e], uzm[e]))))
                             : 0.0f;
            ox[e] = f_mul(ux[e], di);
            oy[e] = f_mul(uy[e], dj);
            oz[e] = f_mul(uz[e], dk[e]);
            pnew = f_mul(f_mul(f_mul(pnew, di), dj), dk[e]);
            if (smask != 0) {
                for (unsigned m = smask; m != 0; m &= m - 1) {
                    const int q = __ffs(m) - 1;
                    const sf_source& S = src.s[q];
                    bool hit;
                    if (S.kind == 0)
                        hit = (i == S.a) && (k + e == S.c);
                    else
                        hit = (S.a == 0) ? (i == S.b) : ((S.a == 1) ? true : (k + e == S.b));
                    if (hit && air) pnew = __double2float_rn(d_add((double)pnew, a.src_val[q]));
                }
            }
            po[e] = pnew;
        }
        store_f<VEC, CS>(a.vxo, c, ox);
        store_f<VEC, CS>(a.vyo, c, oy);
        store_f<VEC, CS>(a.vzo, c, oz);
        store_f<VEC, CS>(a.po, c, po);

#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            vxm[e] = ux[e];
            pc[e] = pn[e];
            pn[e] = pnn[e];
            vx[e] = vxn[e];
            vy[e] = vyn[e];
            vz[e] = vzn[e];
            fc[e] = fnn[e];
        }
    }
}

template <int VEC, int BY, int MINB, bool CS>
int launch(const SfStepArgs& a, const SfSources& src, bool geom, int ich, cudaStream_t st) {
    const int kthreads = (a.nz + VEC - 1) / VEC;
    dim3 blk(32, BY, 1);
    dim3 grd((kthreads + 31) / 32, (a.ny + BY - 1) / BY, (a.nx + ich - 1) / ich);
    if (geom) k_step_col<true, VEC, BY, MINB, CS><<<grd, blk, 0, st>>>(a, src, ich);
    else k_step_col<false, VEC, BY, MINB, CS><<<grd, blk, 0, st>>>(a, src, ich);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_step_col launch failed");
}

}  // namespace

// Column-kernel configurations (index = SF_CFG_COL_FIRST + position).
const SfColConfig kSfColConfigs[] = {
    // vec, by, minb, cs, name
    {1, 8, 1, 0, "col1"},
    {4, 8, 1, 0, "col4"},
    {1, 8, 8, 1, "col1_b8_m8_cs"},
    {1, 16, 4, 1, "col1_b16_m4_cs"},
    {1, 4, 16, 1, "col1_b4_m16_cs"},
    {2, 8, 6, 1, "col2_b8_m6_cs"},
    {2, 4, 12, 1, "col2_b4_m12_cs"},
    {4, 8, 4, 1, "col4_b8_m4_cs"},
    {4, 4, 8, 1, "col4_b4_m8_cs"},
};
const int kSfColConfigCount = sizeof(kSfColConfigs) / sizeof(kSfColConfigs[0]);

int sf_launch_step_col_cfg(const SfStepArgs& a, const SfSources& src, bool geom, int cfg, int ich,
                           cudaStream_t st) {
    if (ich < 1) ich = 1;
    if (cfg < 0 || cfg >= kSfColConfigCount) return sf_fail("k_step_col: bad configuration");
    if (a.nz % kSfColConfigs[cfg].vec != 0) cfg = 0;  // vector width must divide nz
    switch (cfg) {
        case 0: return launch<1, 8, 1, false>(a, src, geom, ich, st);
        case 1: return launch<4, 8, 1, false>(a, src, geom, ich, st);
        case 2: return launch<1, 8, 8, true>(a, src, geom, ich, st);
        case 3: return launch<1, 16, 4, true>(a, src, geom, ich, st);
        case 4: return launch<1, 4, 16, true>(a, src, geom, ich, st);
        case 5: return launch<2, 8, 6, true>(a, src, geom, ich, st);
        case 6: return launch<2, 4, 12, true>(a, src, geom, ich, st);
        case 7: return launch<4, 8, 4, true>(a, src, geom, ich, st);
        case 8: return launch<4, 4, 8, true>(a, src, geom, ich, st);
    }
    return sf_fail("k_step_col: bad configuration");
}
