// sf_voxel.cu -- SDF/CSG voxelisation on the GPU.
//
// Restates SDFPrimitive.voxelize (geometry/sdf.py:99-125 of
// rjwalters/strata-fdtd): the mask is sdf(cell centre) <= 0 with cell centres
// np.arange(n)*res + res/2 (core/grid.py:86-88).  Each thread evaluates one
// cell in FP64 with the reference's operation order and no fused
// multiply-add, so the mask matches NumPy bit for bit:
//   Box      sdf.py:274-293  |p-c| - size/2; norm(max(q,0)) + min(max_d q, 0)
//   Sphere   sdf.py:320-332  norm(p-c) - r
//   Cylinder sdf.py:382-424  projection, clamp, radial/axial distance
//   Union / Intersection / Difference  sdf.py:566-584, 629-647, 704-721
//   Translate / Scale        sdf.py:1225-1236, 1285-1294
//   Rotate                   sdf.py:1351-1355: point @ R (rows of R^T
//                            dotted in the order ((p0 m0 + p1 m1) + p2 m2))
//   Cone                     sdf.py:490-530  projection over the length,
//                            linearly interpolated radius, capped ends
//   Horn                     sdf.py:1085-1133  surface of revolution with
//                            the conical / exponential / hyperbolic /
//                            tractrix radius of sdf.py:1039-1060
//   HelicalTube, SpiralHorn  sdf.py:1666-1695, 1505-1554: distance to a
//                            polyline sampled on the host (paths.py:226-294)
//                            minus the radius at the nearest sample, the
//                            spiral in the xy plane and extruded over z
//   SmoothUnion / SmoothIntersection / SmoothDifference  sdf.py:760-781,
//                            827-847, 903-920: polynomial blends of two
// np.linalg.norm over three components sums ((x0^2 + x1^2) + x2^2).  The
// axis projections of cylinders, cones, horns and path segments use np.dot
// (BLAS), whose rounding depends on the BLAS build; here they are
// ((v0*a0 + v1*a1) + v2*a2), which equals any BLAS result exactly when the
// axis is a coordinate axis.  The horn radii call CUDA's exp, cosh and cos,
// which may differ from NumPy's in the last place: masks can then differ
// only at cells whose distance is within that rounding of zero.
#include <cuda_runtime.h>

#include "sf_common.cuh"

namespace {

constexpr int VX_DSTACK = 32;
constexpr int VX_PSTACK = 12;

__device__ __forceinline__ double norm3(double a, double b, double c) {
    return __dsqrt_rn(d_add(d_add(d_mul(a, a), d_mul(b, b)), d_mul(c, c)));
}
__device__ __forceinline__ double dmax(double a, double b) {  // np.maximum
    return (a >= b || a != a) ? a : b;
}
__device__ __forceinline__ double dmin(double a, double b) {  // np.minimum
    return (a <= b || a != a) ? a : b;
}

__device__ __forceinline__ double clip01(double t) { return dmin(dmax(t, 0.0), 1.0); }

// distance_to_polyline (paths.py:226-294) from (x, y, z) -- or (x, y) when
// dims == 2 -- to the path in nodes d[0 .. m-1] (a = vertex, b = the vertex's
// segment to the next one and s1 = its squared length, both computed on the
// host as the reference does; s0 = the radius there), minus the radius at the
// nearest vertex (the first of equal distances, as np.argmin).
__device__ double path_distance(const sf_sdf_node* __restrict__ d, int m, int dims, double x,
                                double y, double z) {
    double best = __longlong_as_double(0x7ff0000000000000LL);  // +inf
    double near = best;
    double radius = 0.0;
    for (int q = 0; q < m; ++q) {
        const sf_sdf_node& P = d[q];
        const double w0 = d_sub(x, P.a[0]), w1 = d_sub(y, P.a[1]);
        const double w2 = dims == 3 ? d_sub(z, P.a[2]) : 0.0;
        // nearest vertex: norm(path - point), squares as those of point - path
        const double dv = dims == 3 ? norm3(w0, w1, w2)
                                    : __dsqrt_rn(d_add(d_mul(w0, w0), d_mul(w1, w1)));
        if (dv < near) {
            near = dv;
            radius = P.s0;
        }
        if (q + 1 == m) break;
        double ds;
        if (P.s1 < 1e-14) {  // a degenerate segment is its first vertex
            ds = dv;
        } else {
            double t = d_add(d_mul(w0, P.b[0]), d_mul(w1, P.b[1]));
            if (dims == 3) t = d_add(t, d_mul(w2, P.b[2]));
            const double tc = clip01(__ddiv_rn(t, P.s1));
            const double c0 = d_add(P.a[0], d_mul(tc, P.b[0]));
            const double c1 = d_add(P.a[1], d_mul(tc, P.b[1]));
            if (dims == 3) {
                const double c2 = d_add(P.a[2], d_mul(tc, P.b[2]));
                ds = norm3(d_sub(x, c0), d_sub(y, c1), d_sub(z, c2));
            } else {
                const double e0 = d_sub(x, c0), e1 = d_sub(y, c1);
                ds = __dsqrt_rn(d_add(d_mul(e0, e0), d_mul(e1, e1)));
            }
        }
        best = dmin(best, ds);
    }
    return d_sub(best, radius);
}

__device__ double eval_sdf(const sf_sdf_node* __restrict__ prog, int n, double x, double y,
                           double z, int* err) {
    double ds[VX_DSTACK];
    double px[VX_PSTACK], py[VX_PSTACK], pz[VX_PSTACK];
    int dtop = 0, ptop = 0;
    px[0] = x;
    py[0] = y;
    pz[0] = z;
    for (int q = 0; q < n; ++q) {
        const sf_sdf_node& N = prog[q];
        const double X = px[ptop], Y = py[ptop], Z = pz[ptop];
        switch (N.op) {
            case 1: {  // BOX
                const double q0 = d_sub(fabs(d_sub(X, N.a[0])), d_mul(N.b[0], 0.5));
                const double q1 = d_sub(fabs(d_sub(Y, N.a[1])), d_mul(N.b[1], 0.5));
                const double q2 = d_sub(fabs(d_sub(Z, N.a[2])), d_mul(N.b[2], 0.5));
                const double out = norm3(dmax(q0, 0.0), dmax(q1, 0.0), dmax(q2, 0.0));
                const double ins = dmin(fmax(fmax(q0, q1), q2), 0.0);
                if (dtop >= VX_DSTACK) { *err = 1; return 1.0; }
                ds[dtop++] = d_add(out, ins);
                break;
            }
            case 2: {  // SPHERE
                if (dtop >= VX_DSTACK) { *err = 1; return 1.0; }
                ds[dtop++] = d_sub(norm3(d_sub(X, N.a[0]), d_sub(Y, N.a[1]), d_sub(Z, N.a[2])), N.s0);
                break;
            }
            case 3: {  // CYLINDER: a = p1, b = unit axis, s0 = length, s1 = radius
                const double v0 = d_sub(X, N.a[0]), v1 = d_sub(Y, N.a[1]), v2 = d_sub(Z, N.a[2]);
                const double t = d_add(d_add(d_mul(v0, N.b[0]), d_mul(v1, N.b[1])), d_mul(v2, N.b[2]));
                const double L = N.s0;
                const double tc = dmin(dmax(t, 0.0), L);
                const double c0 = d_add(N.a[0], d_mul(tc, N.b[0]));
                const double c1 = d_add(N.a[1], d_mul(tc, N.b[1]));
                const double c2 = d_add(N.a[2], d_mul(tc, N.b[2]));
                const double radial = norm3(d_sub(X, c0), d_sub(Y, c1), d_sub(Z, c2));
                const double half = d_mul(L, 0.5);
                const double axial = dmax(0.0, d_sub(fabs(d_sub(t, half)), half));
                const bool inside = (t >= 0.0) && (t <= L);
                const double rr = d_sub(radial, N.s1);
                if (dtop >= VX_DSTACK) { *err = 1; return 1.0; }
                ds[dtop++] = inside ? rr : __dsqrt_rn(d_add(d_mul(rr, rr), d_mul(axial, axial)));
                break;
            }
            case 4: {  // CONE: a = p1, b = unit axis, s0 = length, s1 = r1; next node a[0] = r2 - r1
                if (q + 1 >= n || prog[q + 1].op != 27) { *err = 4; return 1.0; }
                const double dr = prog[q + 1].a[0];
                ++q;
                const double v0 = d_sub(X, N.a[0]), v1 = d_sub(Y, N.a[1]), v2 = d_sub(Z, N.a[2]);
                const double L = N.s0;
                const double t = __ddiv_rn(
                    d_add(d_add(d_mul(v0, N.b[0]), d_mul(v1, N.b[1])), d_mul(v2, N.b[2])), L);
                const double tc = clip01(t);
                const double rt = d_add(N.s1, d_mul(tc, dr));
                const double tl = d_mul(tc, L);
                const double c0 = d_add(N.a[0], d_mul(tl, N.b[0]));
                const double c1 = d_add(N.a[1], d_mul(tl, N.b[1]));
                const double c2 = d_add(N.a[2], d_mul(tl, N.b[2]));
                const double radial = norm3(d_sub(X, c0), d_sub(Y, c1), d_sub(Z, c2));
                const double axial = d_mul(dmax(0.0, d_sub(fabs(d_sub(t, 0.5)), 0.5)), L);
                const bool inside = (t >= 0.0) && (t <= 1.0);
                const double rr = d_sub(radial, rt);
                if (dtop >= VX_DSTACK) { *err = 1; return 1.0; }
                ds[dtop++] = inside ? rr : __dsqrt_rn(d_add(d_mul(rr, rr), d_mul(axial, axial)));
                break;
            }
            case 5: {  // HORN: a = throat, b = unit axis, s0 = length, s1 = throat radius,
                       // n = profile; next node a[0] = m, alpha, alpha or R
                if (q + 1 >= n || prog[q + 1].op != 27) { *err = 4; return 1.0; }
                const double k = prog[q + 1].a[0];
                ++q;
                const double v0 = d_sub(X, N.a[0]), v1 = d_sub(Y, N.a[1]), v2 = d_sub(Z, N.a[2]);
                const double L = N.s0;
                const double t = d_add(d_add(d_mul(v0, N.b[0]), d_mul(v1, N.b[1])), d_mul(v2, N.b[2]));
                const double tc = clip01(__ddiv_rn(t, L));
                const double r = norm3(d_sub(v0, d_mul(t, N.b[0])), d_sub(v1, d_mul(t, N.b[1])),
                                       d_sub(v2, d_mul(t, N.b[2])));
                const double xa = d_mul(tc, L);
                double hr;
                if (N.n == 0) hr = d_mul(N.s1, d_add(1.0, d_mul(k, tc)));  // conical
                else if (N.n == 1) hr = d_mul(N.s1, exp(d_mul(k, xa)));   // exponential
                else if (N.n == 2) hr = d_mul(N.s1, cosh(d_mul(k, xa)));  // hyperbolic
                else {                                                     // tractrix
                    const double c = cos(__ddiv_rn(xa, k));
                    hr = __ddiv_rn(N.s1, d_mul(c, c));
                }
                const double rd = d_sub(r, hr);
                const double cap = dmax(-t, d_sub(t, L));
                const bool inside = (t >= 0.0) && (t <= L);
                if (dtop >= VX_DSTACK) { *err = 1; return 1.0; }
                ds[dtop++] = inside ? rd : __dsqrt_rn(d_add(d_mul(rd, rd), d_mul(cap, cap)));
                break;
            }
            case 6:    // TUBE along a 3-D path: n vertices in the next n nodes
            case 7: {  // SPIRAL: the same in the xy plane, extruded over 0 <= z <= s0
                if (N.n < 2 || q + N.n >= n) { *err = 4; return 1.0; }
                const double rd = path_distance(prog + q + 1, N.n, N.op == 6 ? 3 : 2, X, Y, Z);
                double d = rd;
                if (N.op == 7) {
                    const double zd = dmax(0.0, dmax(-Z, d_sub(Z, N.s0)));
                    const bool inside = (Z >= 0.0) && (Z <= N.s0);
                    d = inside ? rd : __dsqrt_rn(d_add(d_mul(rd, rd), d_mul(zd, zd)));
                }
                q += N.n;
                if (dtop >= VX_DSTACK) { *err = 1; return 1.0; }
                ds[dtop++] = d;
                break;
            }
            case 13:    // SMOOTH_UNION: pop b, a; s0 = blend radius
            case 14:    // SMOOTH_INTERSECTION
            case 15: {  // SMOOTH_DIFFERENCE (the subtracted shape negated)
                if (dtop < 2) { *err = 2; return 1.0; }
                const double d1 = ds[dtop - 2];
                const double d2 = (N.op == 15) ? -ds[dtop - 1] : ds[dtop - 1];
                const double k = N.s0;
                const double h = clip01(d_add(0.5, __ddiv_rn(d_mul(0.5, d_sub(d2, d1)), k)));
                const double mix = d_add(d_mul(d2, d_sub(1.0, h)), d_mul(d1, h));
                const double bump = d_mul(d_mul(k, h), d_sub(1.0, h));
                dtop -= 2;
                ds[dtop++] = (N.op == 13) ? d_sub(mix, bump) : d_add(mix, bump);
                break;
            }
            case 10:    // UNION n
            case 11: {  // INTERSECTION n
                if (N.n == 0) {
                    if (dtop >= VX_DSTACK) { *err = 1; return 1.0; }
                    ds[dtop++] = (N.op == 10) ? __longlong_as_double(0x7ff0000000000000LL)
                                              : __longlong_as_double((long long)0xfff0000000000000ULL);
                    break;
                }
                if (N.n > dtop) { *err = 2; return 1.0; }
                const int base = dtop - N.n;
                double r = ds[base];
                for (int c = 1; c < N.n; ++c) r = (N.op == 10) ? dmin(r, ds[base + c]) : dmax(r, ds[base + c]);
                dtop = base;
                ds[dtop++] = r;
                break;
            }
            case 12: {  // DIFFERENCE n: base, then subtracted
                if (N.n > dtop || N.n < 1) { *err = 2; return 1.0; }
                const int base = dtop - N.n;
                double r = ds[base];
                for (int c = 1; c < N.n; ++c) r = dmax(r, -ds[base + c]);
                dtop = base;
                ds[dtop++] = r;
                break;
            }
            case 20:    // PUSH_TRANSLATE
            case 21: {  // PUSH_SCALE
                if (ptop + 1 >= VX_PSTACK) { *err = 3; return 1.0; }
                ++ptop;
                if (N.op == 20) {
                    px[ptop] = d_sub(X, N.a[0]);
                    py[ptop] = d_sub(Y, N.a[1]);
                    pz[ptop] = d_sub(Z, N.a[2]);
                } else {
                    px[ptop] = __ddiv_rn(X, N.a[0]);
                    py[ptop] = __ddiv_rn(Y, N.a[1]);
                    pz[ptop] = __ddiv_rn(Z, N.a[2]);
                }
                break;
            }
            case 25: {  // PUSH_ROTATE: rows 0, 1 here (a, b), row 2 in the next node's a
                if (ptop + 1 >= VX_PSTACK || q + 1 >= n || prog[q + 1].op != 26) { *err = 3; return 1.0; }
                const sf_sdf_node& N2 = prog[q + 1];
                ++ptop;
                px[ptop] = d_add(d_add(d_mul(X, N.a[0]), d_mul(Y, N.a[1])), d_mul(Z, N.a[2]));
                py[ptop] = d_add(d_add(d_mul(X, N.b[0]), d_mul(Y, N.b[1])), d_mul(Z, N.b[2]));
                pz[ptop] = d_add(d_add(d_mul(X, N2.a[0]), d_mul(Y, N2.a[1])), d_mul(Z, N2.a[2]));
                ++q;  // the row-2 node is consumed
                break;
            }
            case 22:
                if (ptop == 0) { *err = 3; return 1.0; }
                --ptop;
                break;
            case 23:
                if (dtop < 1) { *err = 2; return 1.0; }
                ds[dtop - 1] = d_mul(ds[dtop - 1], N.s0);
                break;
            case 24:
                if (dtop < 1) { *err = 2; return 1.0; }
                ds[dtop - 1] = -ds[dtop - 1];
                break;
            default:
                *err = 4;
                return 1.0;
        }
    }
    if (dtop != 1) { *err = 2; return 1.0; }
    return ds[0];
}

// coords (nx + ny + nz doubles, may be null): the cell centres of a
// nonuniform grid, else centres at (index + 1/2) * res.
__global__ void k_voxelize(const sf_sdf_node* __restrict__ prog, int n_nodes, int nx, int ny,
                           int nz, double res, const double* __restrict__ coords, int invert,
                           uint8_t* __restrict__ out, int* __restrict__ err_flag) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= nz || j >= ny) return;
    double x, y, z;
    if (coords) {
        x = coords[i];
        y = coords[nx + j];
        z = coords[nx + ny + k];
    } else {
        const double half = d_mul(res, 0.5);
        x = d_add(d_mul((double)i, res), half);
        y = d_add(d_mul((double)j, res), half);
        z = d_add(d_mul((double)k, res), half);
    }
    int err = 0;
    const double d = eval_sdf(prog, n_nodes, x, y, z, &err);
    if (err) atomicExch(err_flag, err);
    const bool inside = d <= 0.0;
    out[((long long)i * ny + j) * nz + k] = (uint8_t)(inside != (invert != 0));
}

// MaterializedGeometry.voxelize_with_materials (geometry/
// material_assignment.py:133-171) in one pass: program 0 (nodes
// off[0]..off[1]-1) is the geometry, inside = air; programs 1..n_regions are
// the material regions in assignment order, region r giving id ids[r-1].  A
// cell's id is that of the last region containing it, within air only, else
// 0 -- the reference's ordered overwrites.  Regions are tried from the last
// down and the first hit wins, which gives the same id with fewer programs
// evaluated.
__global__ void k_voxelize_materials(const sf_sdf_node* __restrict__ prog,
                                     const int* __restrict__ off, const uint8_t* __restrict__ ids,
                                     int n_regions, int nx, int ny, int nz, double res,
                                     const double* __restrict__ coords,
                                     uint8_t* __restrict__ geom, uint8_t* __restrict__ mat,
                                     int* __restrict__ err_flag) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= nz || j >= ny) return;
    double x, y, z;
    if (coords) {
        x = coords[i];
        y = coords[nx + j];
        z = coords[nx + ny + k];
    } else {
        const double half = d_mul(res, 0.5);
        x = d_add(d_mul((double)i, res), half);
        y = d_add(d_mul((double)j, res), half);
        z = d_add(d_mul((double)k, res), half);
    }
    int err = 0;
    const bool air = eval_sdf(prog + off[0], off[1] - off[0], x, y, z, &err) <= 0.0;
    uint8_t m = 0;
    if (air) {
        for (int r = n_regions; r >= 1; --r) {
            if (eval_sdf(prog + off[r], off[r + 1] - off[r], x, y, z, &err) <= 0.0) {
                m = ids[r - 1];
                break;
            }
        }
    }
    if (err) atomicExch(err_flag, err);
    const long long c = ((long long)i * ny + j) * nz + k;
    geom[c] = (uint8_t)air;
    mat[c] = m;
}

__global__ void k_sdf_points(const sf_sdf_node* __restrict__ prog, int n_nodes,
                             const double* __restrict__ pts, long long n, double* __restrict__ out,
                             int* __restrict__ err_flag) {
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        int err = 0;
        out[q] = eval_sdf(prog, n_nodes, pts[3 * q], pts[3 * q + 1], pts[3 * q + 2], &err);
        if (err) atomicExch(err_flag, err);
    }
}

}  // namespace

int sf_launch_sdf_points(const sf_sdf_node* prog_dev, int n_nodes, const double* pts, long long n,
                         double* out, int* err_dev, cudaStream_t st) {
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    if (blocks < 1) blocks = 1;
    k_sdf_points<<<(int)blocks, 256, 0, st>>>(prog_dev, n_nodes, pts, n, out, err_dev);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_sdf_points launch failed");
}

int sf_launch_voxelize(const sf_sdf_node* prog_dev, int n_nodes, int nx, int ny, int nz,
                       double res, const double* coords_dev, int invert, uint8_t* out,
                       int* err_dev, cudaStream_t st) {
    dim3 blk(32, 8, 1), grd((nz + 31) / 32, (ny + 7) / 8, nx);
    k_voxelize<<<grd, blk, 0, st>>>(prog_dev, n_nodes, nx, ny, nz, res, coords_dev, invert, out,
                                    err_dev);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_voxelize launch failed");
}

int sf_launch_voxelize_materials(const sf_sdf_node* prog_dev, const int* off_dev,
                                 const uint8_t* ids_dev, int n_regions, int nx, int ny, int nz,
                                 double res, const double* coords_dev, uint8_t* geom,
                                 uint8_t* mat, int* err_dev, cudaStream_t st) {
    dim3 blk(32, 8, 1), grd((nz + 31) / 32, (ny + 7) / 8, nx);
    k_voxelize_materials<<<grd, blk, 0, st>>>(prog_dev, off_dev, ids_dev, n_regions, nx, ny, nz,
                                              res, coords_dev, geom, mat, err_dev);
    return cudaGetLastError() == cudaSuccess ? 0 : sf_fail("k_voxelize_materials launch failed");
}
