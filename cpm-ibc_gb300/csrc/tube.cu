// Tube construction on the device (compiled with -fmad=false: every a*b+c in
// this file rounds twice, as the reference's host code does, so grid
// coordinates, base points and tricubic weights are bit-identical to the
// reference given the same closest points).
//
//   K1  closest point + band test per grid node        (src/Tube.cpp:429-454, src/Surface.cpp)
//   K3  6-connected component of the seed, union-find  (replaces the BFS queue, src/Tube.cpp:321-454)
//   K4  Morton-ordered 4^3 brick tables                (replaces m_tube_indices_on_grid + SetNeighbours)
//   K5  base points + 1-D tricubic weights             (src/Tube.cpp:464-531, src/Interpolation.cpp:128-225)
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

#include <math_constants.h>

#include "cpm_internal.h"

namespace cpm {

// ============================================================ closest points
// Each function restates the reference's closest-point formula for its kind;
// CUDA's atan2/acos/sin/cos may differ from glibc by an ulp, so parity tests
// compare the tube built from identical closest points (cpm_tube_build_from_cp).

__device__ __forceinline__ void cp_sphere(const double *p, const double x[3], double cp[3], double &dist) {
    // cpSphere, src/Surface.cpp:710-741
    double c0 = p[1], c1 = p[2], c2 = p[3];
    double R = p[0];
    double xs0 = x[0] - c0, xs1 = x[1] - c1, xs2 = x[2] - c2;
    double theta = atan2(xs1, xs0);
    dist = sqrt(xs0 * xs0 + xs1 * xs1 + xs2 * xs2);
    double phi = (dist != 0) ? acos(xs2 / dist) : 0.0;
    double sp = sin(phi);
    cp[0] = R * sp * cos(theta) + c0;
    cp[1] = R * sp * sin(theta) + c1;
    cp[2] = R * cos(phi) + c2;
    dist -= R;
}

__device__ __forceinline__ void cp_torus(const double *p, const double x[3], double cp[3], double &dist) {
    // cpTorus + cpInnerTorusCircle, src/Surface.cpp:800-838
    double theta = atan2(x[1], x[0]);
    double r = sqrt(x[0] * x[0] + x[1] * x[1]);
    double Rmaj = p[0], rmin = p[1];
    double s0 = r - Rmaj, s1 = x[2] - 0.0;
    double th = atan2(s1, s0);
    double c0 = rmin * cos(th) + Rmaj;
    double c1 = rmin * sin(th) + 0.0;
    double a = r - c0, b = x[2] - c1;
    double acc = 0.0;
    acc += a * a;
    acc += b * b;
    dist = sqrt(acc);
    cp[0] = c0 * cos(theta);
    cp[1] = c0 * sin(theta);
    cp[2] = c1;
}

__device__ __forceinline__ double dot3(const double a[3], const double b[3]) {
    double s = 0.0;
    s += a[0] * b[0];
    s += a[1] * b[1];
    s += a[2] * b[2];
    return s;
}

__device__ __forceinline__ void cp_circle3d(const double *p, const double x[3], double cp[3], double &dist) {
    // cpCircle3D with ComputeOrthogonalBasis, src/Surface.cpp:443-504
    double R = p[0];
    double cen[3] = {p[1], p[2], p[3]}, n[3] = {p[4], p[5], p[6]};
    double t1[3], t2[3];
    if (fabs(n[0]) > fabs(n[1])) {
        t1[0] = -n[2]; t1[1] = 0; t1[2] = n[0];
    } else {
        t1[0] = 0; t1[1] = n[2]; t1[2] = -n[1];
    }
    t2[0] = n[1] * t1[2] - n[2] * t1[1];
    t2[1] = n[2] * t1[0] - n[0] * t1[2];
    t2[2] = n[0] * t1[1] - n[1] * t1[0];
    double ctx[3] = {x[0] - cen[0], x[1] - cen[1], x[2] - cen[2]};
    double a = dot3(n, n) * dot3(t1, ctx);
    double b = dot3(t2, ctx);
    double s[3] = {a * t1[0] + b * t2[0], a * t1[1] + b * t2[1], a * t1[2] + b * t2[2]};
    double ns = sqrt(dot3(s, s));
    if (ns > 0) {
        for (int d = 0; d < 3; ++d) cp[d] = cen[d] + (R * s[d]) / ns;
        double h = dot3(n, ctx);
        double cr[3] = {n[1] * ctx[2] - n[2] * ctx[1], n[2] * ctx[0] - n[0] * ctx[2], n[0] * ctx[1] - n[1] * ctx[0]};
        double radial = sqrt(dot3(cr, cr)) - R;
        dist = sqrt(h * h + radial * radial);
    } else {
        double n1 = sqrt(dot3(t1, t1)), n2 = sqrt(dot3(t2, t2));
        const double *tt = (n1 > n2) ? t1 : t2;
        double nn = (n1 > n2) ? n1 : n2;
        for (int d = 0; d < 3; ++d) cp[d] = cen[d] + (R * tt[d]) / nn;
        dist = R;
    }
}

__device__ __forceinline__ void cp_point(const double *p, const double x[3], double cp[3], double &dist) {
    // cpPoint, src/Surface.cpp:840-848
    double acc = 0.0;
    for (int d = 0; d < 3; ++d) {
        cp[d] = p[d];
        double t = x[d] - cp[d];
        acc += t * t;
    }
    dist = sqrt(acc);
}

// Ericson, Real-Time Collision Detection (2005) 5.1.5: closest point on a triangle.
__device__ void cp_triangle(const double *pt, const double *a, const double *b, const double *c, double out[3]) {
    double ab[3], ac[3], ap[3];
    for (int d = 0; d < 3; ++d) {
        ab[d] = b[d] - a[d];
        ac[d] = c[d] - a[d];
        ap[d] = pt[d] - a[d];
    }
    double d1 = dot3(ab, ap), d2 = dot3(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) {
        for (int d = 0; d < 3; ++d) out[d] = a[d];
        return;
    }
    double bp[3];
    for (int d = 0; d < 3; ++d) bp[d] = pt[d] - b[d];
    double d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    if (d3 >= 0.0 && d4 <= d3) {
        for (int d = 0; d < 3; ++d) out[d] = b[d];
        return;
    }
    double vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        double v = d1 / (d1 - d3);
        for (int d = 0; d < 3; ++d) out[d] = a[d] + v * ab[d];
        return;
    }
    double cpp[3];
    for (int d = 0; d < 3; ++d) cpp[d] = pt[d] - c[d];
    double d5 = dot3(ab, cpp), d6 = dot3(ac, cpp);
    if (d6 >= 0.0 && d5 <= d6) {
        for (int d = 0; d < 3; ++d) out[d] = c[d];
        return;
    }
    double vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        double w = d2 / (d2 - d6);
        for (int d = 0; d < 3; ++d) out[d] = a[d] + w * ac[d];
        return;
    }
    double va = d3 * d6 - d5 * d4;
    if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
        double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        for (int d = 0; d < 3; ++d) out[d] = b[d] + w * (c[d] - b[d]);
        return;
    }
    double denom = 1.0 / (va + vb + vc);
    double v = vb * denom, w = vc * denom;
    for (int d = 0; d < 3; ++d) out[d] = a[d] + (v * ab[d] + w * ac[d]);
}

// Ericson 5.1.2: closest point on a segment.
__device__ void cp_segment(const double *pt, const double *a, const double *b, double out[3]) {
    double ab[3], ap[3];
    for (int d = 0; d < 3; ++d) {
        ab[d] = b[d] - a[d];
        ap[d] = pt[d] - a[d];
    }
    double t = dot3(ap, ab);
    if (t <= 0.0) {
        for (int d = 0; d < 3; ++d) out[d] = a[d];
        return;
    }
    double den = dot3(ab, ab);
    if (t >= den) {
        for (int d = 0; d < 3; ++d) out[d] = b[d];
        return;
    }
    t = t / den;
    for (int d = 0; d < 3; ++d) out[d] = a[d] + t * ab[d];
}

// Nearest mesh primitive through the uniform cell grid: rings of cells (by
// Chebyshev distance) around the cell of x clamped into the grid box, until
// the best distance is below the reach of the unsearched cells.  For y in the
// box and x' the projection of x onto the box, |x - y| >= |x' - y|, so the
// reach bound also holds for points outside the box.  Exact minimum over all
// primitives (ties: lower primitive index).  With max_dist finite the search
// stops once nothing within max_dist can remain and reports dist > max_dist;
// max_dist = +inf scans every primitive.
__device__ void cp_mesh(const SurfaceParams &s, const double x[3], double cp[3], double &dist, double max_dist) {
    const bool tri = s.kind == CPM_TRIANGULATION;
    double best2 = 1e300;
    int64_t bestp = -1;
    double bestcp[3] = {0, 0, 0};
    int c[3];
    bool inside = isfinite(max_dist);
    for (int d = 0; d < 3; ++d) {
        double f = floor((x[d] - s.glo[d]) / s.gh);
        c[d] = (int)fmin(fmax(f, 0.0), (double)(s.gn[d] - 1));
    }
    auto test = [&](int64_t p) {
        double q[3];
        if (tri) {
            const int32_t *f = s.prims + 3 * p;
            cp_triangle(x, s.verts + 3 * f[0], s.verts + 3 * f[1], s.verts + 3 * f[2], q);
        } else {
            const int32_t *f = s.prims + 2 * p;
            cp_segment(x, s.verts + 3 * f[0], s.verts + 3 * f[1], q);
        }
        double dd[3] = {x[0] - q[0], x[1] - q[1], x[2] - q[2]};
        double d2 = dot3(dd, dd);
        if (d2 < best2 || (d2 == best2 && p < bestp)) {
            best2 = d2;
            bestp = p;
            bestcp[0] = q[0];
            bestcp[1] = q[1];
            bestcp[2] = q[2];
        }
    };
    if (!inside) {
        for (int64_t p = 0; p < s.nprims; ++p) test(p);
    } else {
        int maxring = max(s.gn[0], max(s.gn[1], s.gn[2]));
        for (int ring = 0; ring <= maxring; ++ring) {
            for (int i = c[0] - ring; i <= c[0] + ring; ++i)
                for (int j = c[1] - ring; j <= c[1] + ring; ++j)
                    for (int k = c[2] - ring; k <= c[2] + ring; ++k) {
                        if (max(abs(i - c[0]), max(abs(j - c[1]), abs(k - c[2]))) != ring) continue;
                        if (i < 0 || j < 0 || k < 0 || i >= s.gn[0] || j >= s.gn[1] || k >= s.gn[2]) continue;
                        size_t cc = ((size_t)i * s.gn[1] + j) * s.gn[2] + k;
                        for (int32_t t = s.cell_start[cc]; t < s.cell_start[cc + 1]; ++t) test(s.cell_items[t]);
                    }
            double reach = ring * s.gh;
            if (best2 <= reach * reach) break;
            if (reach > max_dist) break;  // nothing within max_dist remains unsearched
        }
    }
    cp[0] = bestcp[0];
    cp[1] = bestcp[1];
    cp[2] = bestcp[2];
    dist = sqrt(best2);
}

// max_dist bounds the mesh search only (analytic kinds are exact everywhere).
__device__ __forceinline__ void closest_point(const SurfaceParams &s, const double x[3], double cp[3], double &dist,
                                              double max_dist) {
    switch (s.kind) {
        case CPM_SPHERE: cp_sphere(s.p, x, cp, dist); break;
        case CPM_TORUS: cp_torus(s.p, x, cp, dist); break;
        case CPM_CIRCLE3D: cp_circle3d(s.p, x, cp, dist); break;
        case CPM_POINT: cp_point(s.p, x, cp, dist); break;
        default: cp_mesh(s, x, cp, dist, max_dist); break;
    }
}

// unbounded query (scans every mesh primitive)
__device__ __forceinline__ void closest_point(const SurfaceParams &s, const double x[3], double cp[3], double &dist) {
    closest_point(s, x, cp, dist, CUDART_INF);
}

__global__ void k_closest_points(SurfaceParams s, int64_t n, const double *__restrict__ x, double *__restrict__ cp,
                                 double *__restrict__ dist, double max_dist) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double xi[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]}, c[3], d;
    closest_point(s, xi, c, d, max_dist);
    cp[3 * i] = c[0];
    cp[3 * i + 1] = c[1];
    cp[3 * i + 2] = c[2];
    dist[i] = d;
}

int closest_points_dev(const SurfaceParams &sp, int64_t n, const double *x, double *cp, double *dist, double max_dist) {
    if (n <= 0) return 0;
    int bs = 128;
    k_closest_points<<<(unsigned)((n + bs - 1) / bs), bs, 0, stream()>>>(sp, n, x, cp, dist, max_dist);
    CPM_CUDA_TRY(cudaGetLastError());
    return 0;
}

// ============================================================ surfaces

SurfaceParams SurfaceObj::params() const {
    SurfaceParams s;
    memset(&s, 0, sizeof(s));
    s.kind = desc.kind;
    for (int i = 0; i < 8; ++i) s.p[i] = desc.params[i];
    if (desc.kind == CPM_SPHERE && desc.nparams < 4) s.p[1] = s.p[2] = s.p[3] = 0.0;
    s.verts = mesh.verts.p;
    s.prims = mesh.prims.p;
    s.nprims = mesh.nprims;
    s.cell_start = mesh.cell_start.p;
    s.cell_items = mesh.cell_items.p;
    for (int d = 0; d < 3; ++d) {
        s.glo[d] = mesh.glo[d];
        s.gn[d] = mesh.gn[d];
    }
    s.gh = mesh.gh;
    return s;
}

// Cell-grid build for mesh primitives (counting pass + scatter pass on the device).
__global__ void k_prim_cells(int tri, const double *__restrict__ v, const int32_t *__restrict__ prims, int64_t np, double lo0,
                             double lo1, double lo2, double h, int n0, int n1, int n2, int32_t *__restrict__ counts,
                             const int32_t *__restrict__ starts, int32_t *__restrict__ fill, int32_t *__restrict__ items) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    int nv = tri ? 3 : 2;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int k = 0; k < nv; ++k) {
        const double *q = v + 3 * prims[nv * p + k];
        for (int d = 0; d < 3; ++d) {
            lo[d] = fmin(lo[d], q[d]);
            hi[d] = fmax(hi[d], q[d]);
        }
    }
    double g[3] = {lo0, lo1, lo2};
    int n[3] = {n0, n1, n2}, a[3], b[3];
    for (int d = 0; d < 3; ++d) {
        a[d] = max(0, min(n[d] - 1, (int)floor((lo[d] - g[d]) / h)));
        b[d] = max(0, min(n[d] - 1, (int)floor((hi[d] - g[d]) / h)));
    }
    for (int i = a[0]; i <= b[0]; ++i)
        for (int j = a[1]; j <= b[1]; ++j)
            for (int k = a[2]; k <= b[2]; ++k) {
                size_t c = ((size_t)i * n1 + j) * n2 + k;
                if (!starts) {
                    atomicAdd(&counts[c], 1);
                } else {
                    int slot = atomicAdd(&fill[c], 1);
                    items[starts[c] + slot] = (int32_t)p;
                }
            }
}

// Cell lists are sorted on the host so the candidate order (and thus the tie
// break among equidistant primitives) does not depend on atomic ordering.
int surface_init(SurfaceObj &s, const cpm_surface_desc *d, double cell_h) {
    s.desc = *d;
    s.desc.verts = nullptr;
    s.desc.prims = nullptr;
    if (d->kind < 0 || d->kind > CPM_POLYLINE) return fail(CPM_ERR_INVALID_ARG, "unknown surface kind");
    if (d->kind != CPM_TRIANGULATION && d->kind != CPM_POLYLINE) return 0;
    if (d->nverts <= 0 || d->nprims <= 0 || !d->verts || !d->prims) return fail(CPM_ERR_INVALID_ARG, "mesh surface without vertices");
    const bool tri = d->kind == CPM_TRIANGULATION;
    const int nv = tri ? 3 : 2;
    std::vector<int32_t> prims((size_t)d->nprims * nv);
    for (size_t i = 0; i < prims.size(); ++i) {
        if (d->prims[i] < 0 || d->prims[i] >= d->nverts) return fail(CPM_ERR_INVALID_ARG, "mesh index out of range");
        prims[i] = (int32_t)d->prims[i];
    }
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t i = 0; i < d->nverts; ++i)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], d->verts[3 * i + k]);
            hi[k] = std::max(hi[k], d->verts[3 * i + k]);
        }
    double ext = std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
    double margin = 0.05 * ext + 1e-9;
    // cell size: the tube radius when known (queries are bounded by a few radii),
    // otherwise about sqrt(#primitives) cells per axis; at most 512 cells per axis.
    int res = (int)std::ceil(std::sqrt((double)d->nprims) * 0.7);
    res = std::max(4, std::min(res, 512));
    double h = 0;
    for (int k = 0; k < 3; ++k) {
        s.mesh.glo[k] = lo[k] - margin;
        h = std::max(h, (hi[k] + margin - s.mesh.glo[k]) / res);
    }
    if (cell_h > 0) h = std::max(cell_h, (ext + 2 * margin) / 512.0);
    s.mesh.gh = h;
    size_t ncell = 1;
    for (int k = 0; k < 3; ++k) {
        s.mesh.gn[k] = std::max(1, (int)std::ceil((hi[k] + margin - s.mesh.glo[k]) / h));
        ncell *= (size_t)s.mesh.gn[k];
    }
    s.mesh.nprims = d->nprims;
    CPM_TRY(s.mesh.verts.upload(d->verts, (size_t)d->nverts * 3));
    CPM_TRY(s.mesh.prims.upload(prims));
    DBuf<int32_t> counts;
    CPM_TRY(counts.alloc(ncell));
    CPM_TRY(counts.zero());
    int bs = 128;
    unsigned nb = (unsigned)((d->nprims + bs - 1) / bs);
    k_prim_cells<<<nb, bs, 0, stream()>>>(tri, s.mesh.verts.p, s.mesh.prims.p, d->nprims, s.mesh.glo[0], s.mesh.glo[1],
                                          s.mesh.glo[2], h, s.mesh.gn[0], s.mesh.gn[1], s.mesh.gn[2], counts.p, nullptr,
                                          nullptr, nullptr);
    CPM_CUDA_TRY(cudaGetLastError());
    std::vector<int32_t> hc;
    CPM_TRY(counts.download(hc, ncell));
    std::vector<int32_t> start(ncell + 1, 0);
    for (size_t c = 0; c < ncell; ++c) start[c + 1] = start[c] + hc[c];
    CPM_TRY(s.mesh.cell_start.upload(start));
    CPM_TRY(s.mesh.cell_items.alloc(std::max<size_t>(1, (size_t)start[ncell])));
    CPM_TRY(counts.zero());
    k_prim_cells<<<nb, bs, 0, stream()>>>(tri, s.mesh.verts.p, s.mesh.prims.p, d->nprims, s.mesh.glo[0], s.mesh.glo[1],
                                          s.mesh.glo[2], h, s.mesh.gn[0], s.mesh.gn[1], s.mesh.gn[2], nullptr,
                                          s.mesh.cell_start.p, counts.p, s.mesh.cell_items.p);
    CPM_CUDA_TRY(cudaGetLastError());
    std::vector<int32_t> items;
    CPM_TRY(s.mesh.cell_items.download(items, (size_t)start[ncell]));
    for (size_t c = 0; c < ncell; ++c) std::sort(items.begin() + start[c], items.begin() + start[c + 1]);
    if (!items.empty())
        CPM_CUDA_TRY(cudaMemcpyAsync(s.mesh.cell_items.p, items.data(), items.size() * 4, cudaMemcpyHostToDevice, stream()));
    return 0;
}

// ============================================================ tube build

// Grid sizing of Tube::ConstructTube / ComputeTubeRadius (src/Tube.cpp:131-157).
static void grid_setup(const cpm_surface_desc *d, int p, double dx, GridParams &g, int &n) {
    const size_t order = 2, dim = 3;
    double factor = 1.0001 * std::sqrt((dim - 1) * std::pow(0.5 * (p + 1), 2) + std::pow(0.5 * (order + p + 1), 2));
    g.radius = factor * dx;
    const size_t pad = 5;
    size_t spacings = (size_t)std::ceil((d->bbox[1] - d->bbox[0]) / dx);
    n = (int)(size_t)std::ceil(std::log2((double)(spacings + 2 * pad)));
    size_t diff = (size_t)std::ceil(0.5 * (std::pow(2, (size_t)n) - spacings - 2 * pad));
    g.xstart = d->bbox[0] - (pad + diff) * dx;
    g.dx = dx;
    g.N1d = (int)(size_t)(std::pow(2.0, n) + 1);
    g.NB = (g.N1d + 3) / 4;
}

__device__ __forceinline__ double grid_coord(double xstart, int idx, double dx) { return xstart + (double)idx * dx; }

// K1a: brick candidates. Distance is 1-Lipschitz, so a brick whose centre is
// farther than r + dx + (brick half-diagonal) from the surface holds no tube
// node and no grid node adjacent to one.
__global__ void k_brick_candidates(SurfaceParams s, GridParams g, double thresh, int32_t *__restrict__ flag) {
    int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t nb3 = (int64_t)g.NB * g.NB * g.NB;
    if (b >= nb3) return;
    int bk = (int)(b % g.NB), bj = (int)((b / g.NB) % g.NB), bi = (int)(b / ((int64_t)g.NB * g.NB));
    double x[3] = {g.xstart + (4.0 * bi + 1.5) * g.dx, g.xstart + (4.0 * bj + 1.5) * g.dx, g.xstart + (4.0 * bk + 1.5) * g.dx};
    double cp[3], d;
    closest_point(s, x, cp, d, thresh);
    flag[b] = (fabs(d) <= thresh) ? 1 : 0;
}

// K1b: closest point + band test for the 64 nodes of every candidate brick.
__global__ void k_candidate_nodes(SurfaceParams s, GridParams g, int64_t nc, const uint32_t *__restrict__ cand,
                                  double *__restrict__ cp, double *__restrict__ dist, uint8_t *__restrict__ band) {
    int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nc * 64) return;
    uint32_t bc = cand[v >> 6];
    int l = (int)(v & 63);
    int i = 4 * unpack_i(bc) + (l >> 4), j = 4 * unpack_j(bc) + ((l >> 2) & 3), k = 4 * unpack_k(bc) + (l & 3);
    if (i >= g.N1d || j >= g.N1d || k >= g.N1d) {
        band[v] = 0;
        dist[v] = 1e300;
        return;
    }
    double x[3] = {grid_coord(g.xstart, i, g.dx), grid_coord(g.xstart, j, g.dx), grid_coord(g.xstart, k, g.dx)}, c[3], d;
    closest_point(s, x, c, d, g.radius + g.dx);
    cp[3 * v] = c[0];
    cp[3 * v + 1] = c[1];
    cp[3 * v + 2] = c[2];
    dist[v] = d;
    band[v] = (fabs(d) <= g.radius) ? 1 : 0;
}

struct CandView {
    const int32_t *cmap;  // NB^3 -> candidate index or -1
    int NB, N1d;
};

__device__ __forceinline__ int64_t cand_slot(const CandView &c, int i, int j, int k) {
    if (i < 0 || j < 0 || k < 0 || i >= c.N1d || j >= c.N1d || k >= c.N1d) return -1;
    int ci = c.cmap[((size_t)(i >> 2) * c.NB + (j >> 2)) * c.NB + (k >> 2)];
    if (ci < 0) return -1;
    return (int64_t)ci * 64 + (((i & 3) << 4) | ((j & 3) << 2) | (k & 3));
}

__device__ int uf_find(int32_t *parent, int v, int32_t *err) {
    // path halving; at most one pass over a path of the forest
    for (int it = 0; it < (1 << 26); ++it) {
        int p = parent[v];
        if (p == v) return v;
        int gp = parent[p];
        if (gp != p) atomicCAS(&parent[v], p, gp);
        v = p;
    }
    atomicExch(err, 1);
    return v;
}

// K3: union-find hooking over +x,+y,+z band neighbours (lock-free, link the
// larger root under the smaller; bounded retries).
__global__ void k_uf_hook(CandView cv, int64_t nc, const uint32_t *__restrict__ cand, const uint8_t *__restrict__ band,
                          int32_t *parent, int32_t *err) {
    int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nc * 64 || !band[v]) return;
    uint32_t bc = cand[v >> 6];
    int l = (int)(v & 63);
    int i = 4 * unpack_i(bc) + (l >> 4), j = 4 * unpack_j(bc) + ((l >> 2) & 3), k = 4 * unpack_k(bc) + (l & 3);
    int64_t nb[3] = {cand_slot(cv, i + 1, j, k), cand_slot(cv, i, j + 1, k), cand_slot(cv, i, j, k + 1)};
    for (int d = 0; d < 3; ++d) {
        int64_t u = nb[d];
        if (u < 0 || !band[u]) continue;
        for (int it = 0; it < (1 << 20); ++it) {
            int rv = uf_find(parent, (int)v, err), ru = uf_find(parent, (int)u, err);
            if (rv == ru) break;
            int lo = min(rv, ru), hi = max(rv, ru);
            if (atomicCAS(&parent[hi], hi, lo) == hi) break;
            if (it == (1 << 20) - 1) atomicExch(err, 2);
        }
    }
}

__global__ void k_uf_init(int64_t n, int32_t *parent) {
    int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v < n) parent[v] = (int32_t)v;
}

// Tube membership = band nodes in the seed's component; per-candidate 64-bit mask.
__global__ void k_tube_mask(int64_t nc, const uint8_t *__restrict__ band, int32_t *parent, int root, uint64_t *__restrict__ mask,
                            int32_t *err) {
    int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= nc) return;
    uint64_t m = 0;
    for (int l = 0; l < 64; ++l) {
        int64_t v = c * 64 + l;
        if (band[v] && uf_find(parent, (int)v, err) == root) m |= (1ull << l);
    }
    mask[c] = m;
}

// Grid nodes the reference's BFS evaluates: tube nodes and their 6-neighbours.
__global__ void k_count_visited(CandView cv, int64_t nc, const uint32_t *__restrict__ cand, const uint64_t *__restrict__ mask,
                                unsigned long long *count) {
    int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nc * 64) return;
    uint32_t bc = cand[v >> 6];
    int l = (int)(v & 63);
    int i = 4 * unpack_i(bc) + (l >> 4), j = 4 * unpack_j(bc) + ((l >> 2) & 3), k = 4 * unpack_k(bc) + (l & 3);
    if (i >= cv.N1d || j >= cv.N1d || k >= cv.N1d) return;
    bool vis = (mask[v >> 6] >> l) & 1ull;
    const int di[6] = {1, -1, 0, 0, 0, 0}, dj[6] = {0, 0, 1, -1, 0, 0}, dk[6] = {0, 0, 0, 0, 1, -1};
    for (int d = 0; d < 6 && !vis; ++d) {
        int64_t u = cand_slot(cv, i + di[d], j + dj[d], k + dk[d]);
        if (u >= 0 && ((mask[u >> 6] >> (u & 63)) & 1ull)) vis = true;
    }
    if (vis) atomicAdd(count, 1ull);
}

// Scatter tube nodes from candidate slots to the compact Morton-brick order.
__global__ void k_scatter_nodes(int64_t nc, const uint32_t *__restrict__ cand, const uint64_t *__restrict__ mask,
                                const int32_t *__restrict__ cand_rank, const int32_t *__restrict__ bstart,
                                const double *__restrict__ ccp, const double *__restrict__ cdist, uint32_t *__restrict__ key,
                                double *__restrict__ cp, double *__restrict__ dist) {
    int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nc * 64) return;
    int64_t c = v >> 6;
    int l = (int)(v & 63);
    uint64_t m = mask[c];
    if (!((m >> l) & 1ull)) return;
    int r = cand_rank[c];
    int64_t node = (int64_t)bstart[r] + __popcll(m & ((1ull << l) - 1ull));
    uint32_t bc = cand[c];
    key[node] = pack3(4 * unpack_i(bc) + (l >> 4), 4 * unpack_j(bc) + ((l >> 2) & 3), 4 * unpack_k(bc) + (l & 3));
    cp[3 * node] = ccp[3 * v];
    cp[3 * node + 1] = ccp[3 * v + 1];
    cp[3 * node + 2] = ccp[3 * v + 2];
    dist[node] = cdist[v];
}

// K5: base point (floor((xq - xstart)/dx) - 1, src/Tube.cpp:502-531) and the
// 1-D barycentric Lagrange weights of BuildInterpolationWeights1D
// (src/Interpolation.cpp:162-200), uniform weights (1,-3,3,-1).  err bits:
// 1 base point outside the grid or not a tube node, 2 stencil node missing.
__global__ void k_interp_weights(BrickView bv, GridParams g, int64_t n, const double *__restrict__ xq, uint32_t *__restrict__ base,
                                 double *__restrict__ w, int32_t *__restrict__ err) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    int bt[3];
    bool ok = true;
    for (int d = 0; d < 3; ++d) {
        double f = floor((xq[3 * q + d] - g.xstart) / g.dx);
        if (!(f >= 1.0 && f + 2.0 < (double)g.N1d)) ok = false;
        bt[d] = ok ? (int)f - 1 : 0;
    }
    if (!ok || node_at(bv, bt[0], bt[1], bt[2]) < 0) {
        atomicOr(err, 1);
        base[q] = 0;
        for (int t = 0; t < 12; ++t) w[12 * q + t] = 0.0;
        return;
    }
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b)
            for (int c = 0; c < 4; ++c)
                if (node_at(bv, bt[0] + a, bt[1] + b, bt[2] + c) < 0) ok = false;
    if (!ok) atomicOr(err, 2);
    base[q] = pack3(bt[0], bt[1], bt[2]);
    const double cu[4] = {1.0, -3.0, 3.0, -1.0};
    for (int d = 0; d < 3; ++d) {
        double x[4], wd[4];
        double xqd = xq[3 * q + d];
        bool exact = false;
        int ip = 0;
        for (int j = 0; j < 4; ++j) {
            x[j] = grid_coord(g.xstart, bt[d] + j, g.dx);
            if (fabs(xqd - x[j]) < 1e-17) {
                exact = true;
                ip = j;
            }
        }
        if (exact) {
            for (int j = 0; j < 4; ++j) wd[j] = 0.0;
            wd[ip] = 1.0;
        } else {
            double sum = 0.0;
            for (int j = 0; j < 4; ++j) {
                wd[j] = cu[j] / (xqd - x[j]);
                sum += wd[j];
            }
            for (int j = 0; j < 4; ++j) wd[j] = wd[j] / sum;
        }
        for (int j = 0; j < 4; ++j) w[12 * q + 4 * d + j] = wd[j];
    }
}

int interp_weights_dev(const cpm_tube_s *t, int64_t n, const double *xq, uint32_t *base, double *w, int32_t *err) {
    if (n <= 0) return 0;
    int bs = 128;
    k_interp_weights<<<(unsigned)((n + bs - 1) / bs), bs, 0, stream()>>>(t->view(), t->g, n, xq, base, w, err);
    CPM_CUDA_TRY(cudaGetLastError());
    return 0;
}

static uint32_t spread3(uint32_t v) {
    uint32_t r = 0;
    for (int b = 0; b < 10; ++b) r |= ((v >> b) & 1u) << (3 * b);
    return r;
}

// Shared tail of both build entry points: candidate slots with cp/dist/band on
// the device -> connectivity -> brick tables -> nodes -> weights.
static int finish_build(cpm_tube_s *t, const std::vector<uint32_t> &cand_h, std::vector<int32_t> &cmap_h, DBuf<uint32_t> &cand,
                        DBuf<double> &ccp, DBuf<double> &cdist, DBuf<uint8_t> &band, const int seed[3]) {
    const GridParams &g = t->g;
    const int64_t nc = (int64_t)cand_h.size();
    const int bs = 256;
    for (int d = 0; d < 3; ++d) t->seed[d] = seed[d];
    DBuf<int32_t> cmap, parent, err;
    CPM_TRY(cmap.upload(cmap_h));
    CPM_TRY(parent.alloc((size_t)nc * 64));
    CPM_TRY(err.alloc(1));
    CPM_TRY(err.zero());
    CandView cv{cmap.p, g.NB, g.N1d};
    // the seed joins the tube without the band test (src/Tube.cpp:323-327)
    size_t sb = ((size_t)(seed[0] >> 2) * g.NB + (seed[1] >> 2)) * g.NB + (seed[2] >> 2);
    if (seed[0] < 0 || seed[1] < 0 || seed[2] < 0 || seed[0] >= g.N1d || seed[1] >= g.N1d || seed[2] >= g.N1d || cmap_h[sb] < 0)
        return fail(CPM_ERR_INVALID_ARG, "tube seed node lies outside the candidate band");
    int64_t seed_slot = (int64_t)cmap_h[sb] * 64 + (((seed[0] & 3) << 4) | ((seed[1] & 3) << 2) | (seed[2] & 3));
    uint8_t one = 1;
    CPM_CUDA_TRY(cudaMemcpyAsync(band.p + seed_slot, &one, 1, cudaMemcpyHostToDevice, stream()));
    unsigned gs = (unsigned)((nc * 64 + bs - 1) / bs);
    k_uf_init<<<gs, bs, 0, stream()>>>(nc * 64, parent.p);
    k_uf_hook<<<gs, bs, 0, stream()>>>(cv, nc, cand.p, band.p, parent.p, err.p);
    CPM_CUDA_TRY(cudaGetLastError());
    // root of the seed (a tiny host-side walk over the final forest)
    std::vector<int32_t> par;
    CPM_TRY(parent.download(par, (size_t)nc * 64));
    int root = (int)seed_slot;
    for (int it = 0; it < (1 << 26) && par[root] != root; ++it) root = par[root];
    DBuf<uint64_t> mask;
    CPM_TRY(mask.alloc((size_t)nc));
    k_tube_mask<<<(unsigned)((nc + bs - 1) / bs), bs, 0, stream()>>>(nc, band.p, parent.p, root, mask.p, err.p);
    CPM_CUDA_TRY(cudaGetLastError());
    DBuf<unsigned long long> vcount;
    CPM_TRY(vcount.alloc(1));
    CPM_TRY(vcount.zero());
    k_count_visited<<<gs, bs, 0, stream()>>>(cv, nc, cand.p, mask.p, vcount.p);
    CPM_CUDA_TRY(cudaGetLastError());
    std::vector<int32_t> herr;
    CPM_TRY(err.download(herr, 1));
    if (herr[0]) return fail(CPM_ERR_CUDA, "tube connectivity did not converge");
    std::vector<uint64_t> mask_h;
    CPM_TRY(mask.download(mask_h, (size_t)nc));
    std::vector<unsigned long long> vc;
    CPM_TRY(vcount.download(vc, 1));
    t->nvisited = (int64_t)vc[0];

    // K4: occupied bricks in Morton order, first-node offsets, dense brick map.
    std::vector<std::pair<uint32_t, int64_t>> occ;
    for (int64_t c = 0; c < nc; ++c)
        if (mask_h[c]) {
            uint32_t bc = cand_h[c];
            uint32_t m = (spread3((uint32_t)unpack_i(bc)) << 2) | (spread3((uint32_t)unpack_j(bc)) << 1) | spread3((uint32_t)unpack_k(bc));
            occ.push_back({m, c});
        }
    std::sort(occ.begin(), occ.end());
    const int64_t nbk = (int64_t)occ.size();
    std::vector<int32_t> bstart(nbk), cand_rank(nc, -1), bmap((size_t)g.NB * g.NB * g.NB, -1);
    std::vector<uint64_t> bmask(nbk);
    int64_t total = 0;
    for (int64_t r = 0; r < nbk; ++r) {
        int64_t c = occ[r].second;
        bstart[r] = (int32_t)total;
        bmask[r] = mask_h[c];
        cand_rank[c] = (int32_t)r;
        total += __builtin_popcountll(mask_h[c]);
        uint32_t bc = cand_h[c];
        bmap[((size_t)unpack_i(bc) * g.NB + unpack_j(bc)) * g.NB + unpack_k(bc)] = (int32_t)r;
    }
    if (total >= (int64_t)INT32_MAX) return fail(CPM_ERR_UNSUPPORTED, "tube too large for 32-bit node indices");
    t->N = total;
    t->nbricks = nbk;
    CPM_TRY(t->bmap.upload(bmap));
    CPM_TRY(t->bstart.upload(bstart));
    CPM_TRY(t->bmask.upload(bmask));
    DBuf<int32_t> crank;
    CPM_TRY(crank.upload(cand_rank));
    CPM_TRY(t->key.alloc(total));
    CPM_TRY(t->cp.alloc(3 * total));
    CPM_TRY(t->dist.alloc(total));
    k_scatter_nodes<<<gs, bs, 0, stream()>>>(nc, cand.p, mask.p, crank.p, t->bstart.p, ccp.p, cdist.p, t->key.p, t->cp.p,
                                             t->dist.p);
    CPM_CUDA_TRY(cudaGetLastError());
    CPM_TRY(t->base.alloc(total));
    CPM_TRY(t->w.alloc(12 * total));
    CPM_TRY(err.zero());
    CPM_TRY(interp_weights_dev(t, total, t->cp.p, t->base.p, t->w.p, err.p));
    CPM_TRY(err.download(herr, 1));
    if (herr[0]) return fail(CPM_ERR_BASEPOINT_OUTSIDE_TUBE, "Tube::ComputeBasePoints - Interpolation base point is not within the tube");
    return 0;
}

static int tube_common_setup(cpm_tube_s *t, const cpm_surface_desc *d, int32_t p, double dx) {
    if (!d || dx <= 0) return fail(CPM_ERR_INVALID_ARG, "invalid tube arguments");
    if (p != 3) return fail(CPM_ERR_UNSUPPORTED, "only tricubic interpolation (p = 3) is implemented");
    int n;
    grid_setup(d, p, dx, t->g, n);
    CPM_TRY(surface_init(t->surf, d, t->g.radius));
    t->p = p;
    if (t->g.N1d > 1024) return fail(CPM_ERR_UNSUPPORTED, "grid larger than 1024 nodes per axis");
    return 0;
}

// FindStartingPoint (src/Tube.cpp:540-551): cp of the xstart corner, rounded.
__global__ void k_seed(SurfaceParams s, GridParams g, int32_t *seed) {
    double x[3] = {g.xstart, g.xstart, g.xstart}, cp[3], d;
    closest_point(s, x, cp, d);
    for (int k = 0; k < 3; ++k) seed[k] = (int32_t)round((cp[k] - g.xstart) / g.dx);
}

}  // namespace cpm

using namespace cpm;

extern "C" int cpm_tube_build(const cpm_surface_desc *surface, int32_t p, double dx, cpm_tube_t *out) {
    if (!out) return fail(CPM_ERR_INVALID_ARG, "null output handle");
    *out = nullptr;
    cpm_tube_s *t = new cpm_tube_s();
    auto bail = [&](int rc) {
        delete t;
        return rc;
    };
    int rc = tube_common_setup(t, surface, p, dx);
    if (rc) return bail(rc);
    const GridParams &g = t->g;
    SurfaceParams sp = t->surf.params();
    const int bs = 256;
    int64_t nb3 = (int64_t)g.NB * g.NB * g.NB;
    DBuf<int32_t> flag, seed;
    if ((rc = flag.alloc(nb3)) || (rc = seed.alloc(3))) return bail(rc);
    double thresh = g.radius + g.dx + 1.5 * std::sqrt(3.0) * g.dx + 1e-9 * (1.0 + g.radius);
    k_brick_candidates<<<(unsigned)((nb3 + bs - 1) / bs), bs, 0, stream()>>>(sp, g, thresh, flag.p);
    k_seed<<<1, 1, 0, stream()>>>(sp, g, seed.p);
    if (cudaGetLastError() != cudaSuccess) return bail(fail(CPM_ERR_CUDA, "candidate kernel launch failed"));
    std::vector<int32_t> fh, sh;
    if ((rc = flag.download(fh, nb3)) || (rc = seed.download(sh, 3))) return bail(rc);
    std::vector<uint32_t> cand_h;
    std::vector<int32_t> cmap_h((size_t)nb3, -1);
    for (int64_t b = 0; b < nb3; ++b)
        if (fh[b]) {
            int bk = (int)(b % g.NB), bj = (int)((b / g.NB) % g.NB), bi = (int)(b / ((int64_t)g.NB * g.NB));
            cmap_h[b] = (int32_t)cand_h.size();
            cand_h.push_back(pack3(bi, bj, bk));
        }
    int64_t nc = (int64_t)cand_h.size();
    DBuf<uint32_t> cand;
    DBuf<double> ccp, cdist;
    DBuf<uint8_t> band;
    if ((rc = cand.upload(cand_h)) || (rc = ccp.alloc(3 * nc * 64)) || (rc = cdist.alloc(nc * 64)) || (rc = band.alloc(nc * 64)))
        return bail(rc);
    k_candidate_nodes<<<(unsigned)((nc * 64 + bs - 1) / bs), bs, 0, stream()>>>(sp, g, nc, cand.p, ccp.p, cdist.p, band.p);
    if (cudaGetLastError() != cudaSuccess) return bail(fail(CPM_ERR_CUDA, "candidate node kernel launch failed"));
    int sd[3] = {sh[0], sh[1], sh[2]};
    if ((rc = finish_build(t, cand_h, cmap_h, cand, ccp, cdist, band, sd))) return bail(rc);
    *out = t;
    return 0;
}

extern "C" int cpm_tube_build_from_cp(const cpm_surface_desc *surface, int32_t p, double dx, int64_t n, const int64_t *keys,
                                      const double *cp, const double *dist, cpm_tube_t *out) {
    if (!out || n <= 0 || !keys || !cp || !dist) return fail(CPM_ERR_INVALID_ARG, "invalid arguments");
    *out = nullptr;
    cpm_tube_s *t = new cpm_tube_s();
    auto bail = [&](int rc) {
        delete t;
        return rc;
    };
    int rc = tube_common_setup(t, surface, p, dx);
    if (rc) return bail(rc);
    const GridParams &g = t->g;
    const int64_t N1 = g.N1d;
    int64_t nb3 = (int64_t)g.NB * g.NB * g.NB;
    std::vector<int32_t> cmap_h((size_t)nb3, -1);
    std::vector<uint32_t> cand_h;
    for (int64_t q = 0; q < n; ++q) {
        int64_t key = keys[q];
        if (key < 0 || key >= N1 * N1 * N1) return bail(fail(CPM_ERR_INVALID_ARG, "grid key out of range"));
        int i = (int)(key / (N1 * N1)), j = (int)((key / N1) % N1), k = (int)(key % N1);
        size_t b = ((size_t)(i >> 2) * g.NB + (j >> 2)) * g.NB + (k >> 2);
        if (cmap_h[b] < 0) {
            cmap_h[b] = (int32_t)cand_h.size();
            cand_h.push_back(pack3(i >> 2, j >> 2, k >> 2));
        }
    }
    int64_t nc = (int64_t)cand_h.size();
    std::vector<double> ccp_h(3 * nc * 64, 0.0), cdist_h(nc * 64, 1e300);
    std::vector<uint8_t> band_h(nc * 64, 0);
    for (int64_t q = 0; q < n; ++q) {
        int64_t key = keys[q];
        int i = (int)(key / (N1 * N1)), j = (int)((key / N1) % N1), k = (int)(key % N1);
        size_t b = ((size_t)(i >> 2) * g.NB + (j >> 2)) * g.NB + (k >> 2);
        int64_t v = (int64_t)cmap_h[b] * 64 + (((i & 3) << 4) | ((j & 3) << 2) | (k & 3));
        for (int d = 0; d < 3; ++d) ccp_h[3 * v + d] = cp[3 * q + d];
        cdist_h[v] = dist[q];
        band_h[v] = std::fabs(dist[q]) <= g.radius ? 1 : 0;
    }
    // seed from the supplied closest point of the xstart corner is not available:
    // use the device closest point of the corner, as cpm_tube_build does.
    DBuf<int32_t> seed;
    if ((rc = seed.alloc(3))) return bail(rc);
    k_seed<<<1, 1, 0, stream()>>>(t->surf.params(), g, seed.p);
    std::vector<int32_t> sh;
    if ((rc = seed.download(sh, 3))) return bail(rc);
    DBuf<uint32_t> cand;
    DBuf<double> ccp, cdist;
    DBuf<uint8_t> band;
    if ((rc = cand.upload(cand_h)) || (rc = ccp.upload(ccp_h)) || (rc = cdist.upload(cdist_h)) || (rc = band.upload(band_h)))
        return bail(rc);
    int sd[3] = {sh[0], sh[1], sh[2]};
    if ((rc = finish_build(t, cand_h, cmap_h, cand, ccp, cdist, band, sd))) return bail(rc);
    *out = t;
    return 0;
}

extern "C" int cpm_tube_info_get(cpm_tube_t t, cpm_tube_info *info) {
    if (!t || !info) return fail(CPM_ERR_INVALID_ARG, "null argument");
    info->n_nodes = t->N;
    info->n1d = t->g.N1d;
    info->n_bricks = t->nbricks;
    info->n_visited = t->nvisited;
    info->dx = t->g.dx;
    info->xstart = t->g.xstart;
    info->radius = t->g.radius;
    info->p = t->p;
    info->pad = 0;
    return 0;
}

namespace cpm {
__global__ void k_tube_export_nbr(BrickView bv, int64_t n, const uint32_t *__restrict__ key, int64_t *__restrict__ nbr) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    uint32_t kk = key[q];
    int i = unpack_i(kk), j = unpack_j(kk), k = unpack_k(kk);
    const int di[6] = {1, -1, 0, 0, 0, 0}, dj[6] = {0, 0, 1, -1, 0, 0}, dk[6] = {0, 0, 0, 0, 1, -1};
    for (int d = 0; d < 6; ++d) nbr[6 * q + d] = node_at(bv, i + di[d], j + dj[d], k + dk[d]);
}
}  // namespace cpm

extern "C" int cpm_tube_export(cpm_tube_t t, int64_t *rec, double *x, double *cp, double *dist, int64_t *bpt_rec, int64_t *nbr,
                               double *w) {
    if (!t) return fail(CPM_ERR_INVALID_ARG, "null tube");
    const int64_t N = t->N, N1 = t->g.N1d;
    std::vector<uint32_t> key;
    CPM_TRY(t->key.download(key, N));
    if (rec || x)
        for (int64_t q = 0; q < N; ++q) {
            int i = unpack_i(key[q]), j = unpack_j(key[q]), k = unpack_k(key[q]);
            if (rec) rec[q] = ((int64_t)i * N1 + j) * N1 + k;
            if (x) {
                // CoordinateFromTriplet (src/Grid.cpp:28-39)
                x[3 * q] = t->g.xstart + (double)i * t->g.dx;
                x[3 * q + 1] = t->g.xstart + (double)j * t->g.dx;
                x[3 * q + 2] = t->g.xstart + (double)k * t->g.dx;
            }
        }
    if (cp) {
        std::vector<double> h;
        CPM_TRY(t->cp.download(h, 3 * N));
        std::copy(h.begin(), h.end(), cp);
    }
    if (dist) {
        std::vector<double> h;
        CPM_TRY(t->dist.download(h, N));
        std::copy(h.begin(), h.end(), dist);
    }
    if (bpt_rec) {
        std::vector<uint32_t> b;
        CPM_TRY(t->base.download(b, N));
        for (int64_t q = 0; q < N; ++q) bpt_rec[q] = ((int64_t)unpack_i(b[q]) * N1 + unpack_j(b[q])) * N1 + unpack_k(b[q]);
    }
    if (w) {
        std::vector<double> h;
        CPM_TRY(t->w.download(h, 12 * N));
        std::copy(h.begin(), h.end(), w);
    }
    if (nbr) {
        DBuf<int64_t> d;
        CPM_TRY(d.alloc(6 * N));
        k_tube_export_nbr<<<(unsigned)((N + 255) / 256), 256, 0, stream()>>>(t->view(), N, t->key.p, d.p);
        CPM_CUDA_TRY(cudaGetLastError());
        std::vector<int64_t> h;
        CPM_TRY(d.download(h, 6 * N));
        std::copy(h.begin(), h.end(), nbr);
    }
    return 0;
}

// The reference numbers tube nodes in the order its breadth-first flood
// discovers them (Tube::BuildTube, src/Tube.cpp:321-454): the seed first, then
// each dequeued node's in-band neighbours in the order +x,-x,+y,-y,+z,-z
// (src/Tube.cpp:431-435).  The device tube is that flood's node set; a
// breadth-first walk of its neighbour table from the seed gives the order.
extern "C" int cpm_tube_reference_order(cpm_tube_t t, int64_t *order) {
    if (!t || !order) return fail(CPM_ERR_INVALID_ARG, "tube_reference_order: null argument");
    const int64_t N = t->N;
    std::vector<uint32_t> key;
    CPM_TRY(t->key.download(key, N));
    const uint32_t sk = pack3(t->seed[0], t->seed[1], t->seed[2]);
    int64_t s0 = -1;
    for (int64_t q = 0; q < N && s0 < 0; ++q)
        if (key[q] == sk) s0 = q;
    if (s0 < 0) return fail(CPM_ERR_CUDA, "tube_reference_order: the seed node is not in the tube");
    std::vector<int64_t> nbr((size_t)6 * N);
    CPM_TRY(cpm_tube_export(t, nullptr, nullptr, nullptr, nullptr, nullptr, nbr.data(), nullptr));
    std::vector<char> seen((size_t)N, 0);
    int64_t head = 0, tail = 0;
    order[tail++] = s0;
    seen[s0] = 1;
    while (head < tail) {
        const int64_t q = order[head++];
        for (int d = 0; d < 6; ++d) {
            const int64_t m = nbr[6 * q + d];
            if (m >= 0 && !seen[m]) {
                seen[m] = 1;
                order[tail++] = m;
            }
        }
    }
    if (tail != N) return fail(CPM_ERR_CUDA, "tube_reference_order: the tube is not connected");
    return 0;
}

namespace cpm {
// E row entries of query points: value w2[k]*w1[j]*w0[i], walk +x outer (src/Interpolation.cpp:83-117).
__global__ void k_interp_rows(BrickView bv, int64_t n, const uint32_t *__restrict__ base, const double *__restrict__ w,
                              int64_t *__restrict__ cols, double *__restrict__ vals) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    uint32_t b = base[q];
    int bi = unpack_i(b), bj = unpack_j(b), bk = unpack_k(b);
    const double *wq = w + 12 * q;
    int s = 0;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            for (int k = 0; k < 4; ++k, ++s) {
                cols[64 * q + s] = node_at(bv, bi + i, bj + j, bk + k);
                vals[64 * q + s] = wq[8 + k] * wq[4 + j] * wq[i];
            }
}
}  // namespace cpm

extern "C" int cpm_interp_query(cpm_tube_t t, int64_t n, const double *xq, int64_t *cols, double *vals) {
    if (!t || n < 0 || (n > 0 && (!xq || !cols || !vals))) return fail(CPM_ERR_INVALID_ARG, "invalid arguments");
    if (n == 0) return 0;
    DBuf<double> dx, dw, dv;
    DBuf<uint32_t> db;
    DBuf<int64_t> dc;
    DBuf<int32_t> err;
    CPM_TRY(dx.upload(xq, 3 * n));
    CPM_TRY(db.alloc(n));
    CPM_TRY(dw.alloc(12 * n));
    CPM_TRY(err.alloc(1));
    CPM_TRY(err.zero());
    CPM_TRY(interp_weights_dev(t, n, dx.p, db.p, dw.p, err.p));
    std::vector<int32_t> he;
    CPM_TRY(err.download(he, 1));
    if (he[0]) return fail(CPM_ERR_BASEPOINT_OUTSIDE_TUBE, "Tube::ComputeBasePoints - Interpolation base point is not within the tube");
    CPM_TRY(dc.alloc(64 * n));
    CPM_TRY(dv.alloc(64 * n));
    k_interp_rows<<<(unsigned)((n + 127) / 128), 128, 0, stream()>>>(t->view(), n, db.p, dw.p, dc.p, dv.p);
    CPM_CUDA_TRY(cudaGetLastError());
    std::vector<int64_t> hc;
    std::vector<double> hv;
    CPM_TRY(dc.download(hc, 64 * n));
    CPM_TRY(dv.download(hv, 64 * n));
    std::copy(hc.begin(), hc.end(), cols);
    std::copy(hv.begin(), hv.end(), vals);
    return 0;
}

extern "C" int cpm_tube_destroy(cpm_tube_t t) {
    delete t;
    return 0;
}

// Surface::ClosestPoint (src/Surface.cpp:61-190) for n points of any surface kind
extern "C" int cpm_closest_points(const cpm_surface_desc *surface, int64_t n, const double *x, double max_dist, double *cp,
                                  double *dist) {
    if (!surface || n < 0 || (n > 0 && (!x || !cp || !dist))) return fail(CPM_ERR_INVALID_ARG, "closest_points: invalid arguments");
    if (n == 0) return 0;
    SurfaceObj s;
    CPM_TRY(surface_init(s, surface, max_dist > 0 ? max_dist : 0.0));
    DBuf<double> dx, dcp, dd;
    CPM_TRY(dx.upload(x, 3 * (size_t)n));
    CPM_TRY(dcp.alloc(3 * (size_t)n));
    CPM_TRY(dd.alloc((size_t)n));
    CPM_TRY(closest_points_dev(s.params(), n, dx.p, dcp.p, dd.p, max_dist > 0 ? max_dist : (double)INFINITY));
    std::vector<double> hc, hd;
    CPM_TRY(dcp.download(hc, 3 * (size_t)n));
    CPM_TRY(dd.download(hd, (size_t)n));
    std::copy(hc.begin(), hc.end(), cp);
    std::copy(hd.begin(), hd.end(), dist);
    return 0;
}
