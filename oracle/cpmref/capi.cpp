// ORACLE — test infrastructure only. Not part of the product library.
//
// C entry points of the CPU restatement, loaded by the tests and by the
// cpu_baseline / reference legs of bench.py through ctypes.  Nothing in the
// product library links or calls this file.
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <stdexcept>
#include <cstring>
#include <exception>
#include <memory>
#include <string>
#include <vector>

#include "problems.h"

using namespace cpmref;

extern "C" {

// Layout shared with the tests' ctypes descriptor (tests/oracle_lib.py).
typedef struct {
    int32_t kind;  // 0 sphere, 1 torus, 2 circle3d, 3 point, 4 triangulation, 5 polyline
    int32_t nparams;
    double params[8];
    double bbox[2];
    int64_t nverts;
    const double *verts;  // 3 * nverts
    int64_t nprims;
    const int64_t *prims;  // 3 * nprims (triangles) or 2 * nprims (segments)
    // IBC metadata (used when the surface is an interior boundary)
    int32_t boundary_order;
    int32_t boundary_type[2];
    int32_t is_oriented;
    int32_t has_point_on_side1;
    int32_t use_cp_diff_directions;
    int32_t use_Jcp_surface_normals;
    int32_t pad0;
    double on_ibc_tolerance;
    double point_on_side1[3];
    double dof_radius_scale;
} cpmref_surface_desc;

static thread_local std::string g_err;
const char *cpmref_last_error() { return g_err.c_str(); }

static SurfaceSpec ToSpec(const cpmref_surface_desc *d) {
    SurfaceSpec s;
    s.kind = (SurfaceKind)d->kind;
    s.params.assign(d->params, d->params + d->nparams);
    s.bbox[0] = d->bbox[0];
    s.bbox[1] = d->bbox[1];
    if (s.kind == SurfaceKind::Triangulation || s.kind == SurfaceKind::Polyline) {
        s.vertices.resize(d->nverts);
        for (int64_t i = 0; i < d->nverts; ++i) s.vertices[i] = V3{d->verts[3 * i], d->verts[3 * i + 1], d->verts[3 * i + 2]};
        if (s.kind == SurfaceKind::Triangulation) {
            s.faces.resize(d->nprims);
            for (int64_t i = 0; i < d->nprims; ++i)
                s.faces[i] = {(size_t)d->prims[3 * i], (size_t)d->prims[3 * i + 1], (size_t)d->prims[3 * i + 2]};
        } else {
            s.segments.resize(d->nprims);
            for (int64_t i = 0; i < d->nprims; ++i) s.segments[i] = {(size_t)d->prims[2 * i], (size_t)d->prims[2 * i + 1]};
        }
    }
    s.meta.boundary_order = (size_t)d->boundary_order;
    s.meta.boundary_type[0] = (size_t)d->boundary_type[0];
    s.meta.boundary_type[1] = (size_t)d->boundary_type[1];
    s.meta.is_oriented = d->is_oriented != 0;
    if (d->has_point_on_side1) s.meta.point_on_side1.assign(d->point_on_side1, d->point_on_side1 + 3);
    s.meta.use_cp_diff_directions = d->use_cp_diff_directions != 0;
    s.meta.use_Jcp_surface_normals = d->use_Jcp_surface_normals != 0;
    s.meta.on_ibc_tolerance = d->on_ibc_tolerance;
    s.meta.ibc_DOFSubset_radius_scale = d->dof_radius_scale;
    return s;
}

struct Handle {
    std::unique_ptr<Problem> prob;
    // every grid node whose closest point the BFS evaluated: (rec, cp, dist, bdy)
    std::vector<int64_t> vis_rec;
    std::vector<double> vis_cp, vis_dist;
    std::vector<int64_t> vis_bdy;
    SpMat plot;
    bool plot_built = false;
    std::vector<SpMat> dc;  // whole-tube gradient matrices, built on first use
    double last_setup_s = 0;
};

#define GUARD_BEGIN try {
#define GUARD_END                 \
    }                             \
    catch (const std::exception &e) { \
        g_err = e.what();         \
        return -1;                \
    }

int cpmref_problem_create(const cpmref_surface_desc *surf, int32_t n_ibc, const cpmref_surface_desc *ibcs, int32_t p,
                          double dx, int32_t record_visited, void **out) {
    GUARD_BEGIN
    auto t0 = std::chrono::steady_clock::now();
    auto h = new Handle();
    SurfaceSpec ss = ToSpec(surf);
    std::vector<SurfaceSpec> is;
    for (int c = 0; c < n_ibc; ++c) is.push_back(ToSpec(&ibcs[c]));
    if (record_visited) {
        // same BFS; the closest-point function records every evaluation
        Surface *sp = nullptr;
        auto cpf = [&](size_t rec, const V3 &x, V3 &cp, double &dist, size_t &bdy) {
            sp->ClosestPoint(x, cp, dist, bdy);
            h->vis_rec.push_back((int64_t)rec);
            for (int d = 0; d < 3; ++d) h->vis_cp.push_back(cp[d]);
            h->vis_dist.push_back(dist);
            h->vis_bdy.push_back((int64_t)bdy);
        };
        Surface s(ss);
        sp = &s;
        h->prob.reset(new Problem(ss, (size_t)p, dx, cpf, true));
        if (n_ibc > 0) h->prob->Assemble(is);
    } else {
        h->prob.reset(new Problem(ss, is, (size_t)p, dx));
    }
    h->last_setup_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    *out = h;
    return 0;
    GUARD_END
}

// Tube from caller-supplied closest points, keyed by grid linear index
// (sorted keys; missing keys are an error).
int cpmref_problem_create_from_cp(const cpmref_surface_desc *surf, int32_t p, double dx, int64_t n, const int64_t *keys,
                                  const double *cp, const double *dist, void **out) {
    GUARD_BEGIN
    auto h = new Handle();
    SurfaceSpec ss = ToSpec(surf);
    auto cpf = [&](size_t rec, const V3 &, V3 &c, double &d, size_t &b) {
        const int64_t *it = std::lower_bound(keys, keys + n, (int64_t)rec);
        if (it == keys + n || *it != (int64_t)rec) throw std::runtime_error("create_from_cp: grid node without a supplied closest point");
        size_t k = it - keys;
        c = V3{cp[3 * k], cp[3 * k + 1], cp[3 * k + 2]};
        d = dist[k];
        b = 0;
    };
    h->prob.reset(new Problem(ss, (size_t)p, dx, cpf, true));
    *out = h;
    return 0;
    GUARD_END
}

void cpmref_problem_destroy(void *hp) { delete (Handle *)hp; }

// sizes: [N, D, N1d, total_ibc_dofs, num_2nd_order_rows, n_ibc, n_visited, nnz(Lfull), nnz(Efull), n_plot]
int cpmref_problem_sizes(void *hp, int64_t *out) {
    Handle *h = (Handle *)hp;
    Problem &P = *h->prob;
    out[0] = (int64_t)P.tube.nNodes();
    out[1] = (int64_t)P.D();
    out[2] = (int64_t)P.tube.N1d();
    out[3] = P.has_ibc ? (int64_t)P.ibc.TotalIBCDOFs() : 0;
    out[4] = P.has_ibc ? (int64_t)P.ibc.Num2ndOrderDirichletRows() : 0;
    out[5] = P.has_ibc ? (int64_t)P.ibc.NumIBCs() : 0;
    out[6] = (int64_t)h->vis_rec.size();
    out[7] = (int64_t)P.Lfull.nnz();
    out[8] = (int64_t)P.Efull.nnz();
    out[9] = (int64_t)P.tube.surface().xp().size();
    return 0;
}

// grid: [dx, xstart, radius]
int cpmref_problem_grid(void *hp, double *out) {
    Problem &P = *((Handle *)hp)->prob;
    out[0] = P.tube.dx();
    out[1] = P.tube.xstart();
    out[2] = P.tube.TubeRadius();
    return 0;
}

double cpmref_setup_seconds(void *hp) { return ((Handle *)hp)->last_setup_s; }

int cpmref_tube_export(void *hp, int64_t *rec, double *x, double *cp, double *dist, int64_t *bpt, int64_t *nbr) {
    Problem &P = *((Handle *)hp)->prob;
    const Tube &t = P.tube;
    for (size_t i = 0; i < t.nNodes(); ++i) {
        if (rec) rec[i] = (int64_t)t.recIndex()[i];
        for (int d = 0; d < 3; ++d) {
            if (x) x[3 * i + d] = t.x()[i][d];
            if (cp) cp[3 * i + d] = t.cpx()[i][d];
        }
        if (dist) dist[i] = t.dist()[i];
        if (bpt) bpt[i] = (int64_t)t.bpt()[i];
        if (nbr)
            for (int k = 0; k < 6; ++k) nbr[6 * i + k] = t.neighbour((int64_t)i, k);
    }
    return 0;
}

int cpmref_visited_export(void *hp, int64_t *rec, double *cp, double *dist) {
    Handle *h = (Handle *)hp;
    std::copy(h->vis_rec.begin(), h->vis_rec.end(), rec);
    std::copy(h->vis_cp.begin(), h->vis_cp.end(), cp);
    std::copy(h->vis_dist.begin(), h->vis_dist.end(), dist);
    return 0;
}

// Per-node 1-D tricubic weights w[q][d][j] (q-major, 12 per node).
int cpmref_weights_export(void *hp, double *w) {
    Problem &P = *((Handle *)hp)->prob;
    Interpolation interp(P.tube);
    const auto &W = interp.weights();
    size_t N = P.tube.nNodes();
    for (size_t q = 0; q < N; ++q)
        for (int d = 0; d < 3; ++d)
            for (int j = 0; j < 4; ++j) w[12 * q + 4 * d + j] = W[d][q][j];
    return 0;
}

static const SpMat &Pick(Handle *h, int which) {
    Problem &P = *h->prob;
    switch (which) {
        case 0: return P.Lfull;
        case 1: return P.Efull;
        case 2: return P.L;
        case 3: return P.E;
        case 5:
        case 6:
        case 7:  // FDMatrices::BuildGradientMatrices on the whole tube (src/FDMatrices.cpp:66-92)
            if (h->dc.empty()) BuildGradientMatrices(P.tube, h->dc);
            return h->dc[which - 5];
        default:
            if (!h->plot_built) {
                h->plot = P.PlotMatrix();
                h->plot_built = true;
            }
            return h->plot;
    }
}

int64_t cpmref_csr_nnz(void *hp, int32_t which) { return (int64_t)Pick((Handle *)hp, which).nnz(); }
int64_t cpmref_csr_rows(void *hp, int32_t which) { return (int64_t)Pick((Handle *)hp, which).rows; }

int cpmref_csr_export(void *hp, int32_t which, int64_t *ptr, int64_t *idx, double *val) {
    const SpMat &A = Pick((Handle *)hp, which);
    for (size_t i = 0; i <= A.rows; ++i) ptr[i] = (int64_t)A.ptr[i];
    for (size_t k = 0; k < A.nnz(); ++k) {
        idx[k] = (int64_t)A.idx[k];
        val[k] = A.val[k];
    }
    return 0;
}

// y = A x for one of the exported matrices (rows summed in ascending column order)
int cpmref_csr_multiply(void *hp, int32_t which, const double *x, double *y) {
    GUARD_BEGIN
    const SpMat &A = Pick((Handle *)hp, which);
    std::vector<double> xv(x, x + A.cols), yv;
    A.Multiply(xv, yv);
    std::copy(yv.begin(), yv.end(), y);
    return 0;
    GUARD_END
}

int cpmref_rows_export(void *hp, uint8_t *identity, int32_t *kind, int32_t *ibc, double *point) {
    Problem &P = *((Handle *)hp)->prob;
    for (size_t r = 0; r < P.D(); ++r) {
        if (identity) identity[r] = P.identity_rows[r] ? 1 : 0;
        if (kind) kind[r] = P.row_kind[r];
        if (ibc) ibc[r] = P.row_ibc[r];
        if (point)
            for (int d = 0; d < 3; ++d) point[3 * r + d] = P.row_point[r][d];
    }
    return 0;
}

// IBCDOFSubset::which_side of every IBC DOF row and Dirichlet value row (0 elsewhere),
// as PoissonWithIBC::GetRHS hands it to the boundary-value function
int cpmref_row_sides(void *hp, int32_t *side) {
    Problem &P = *((Handle *)hp)->prob;
    for (size_t r = 0; r < P.D(); ++r) side[r] = 0;
    if (!P.has_ibc) return 0;
    for (size_t c = 0; c < P.ibc.NumIBCs(); ++c) {
        const IBCDOFSubset &dof = P.ibc.DOFSubset()[c];
        const IBCMeta &mc = P.ibc.meta(c);
        for (size_t i = 0; i < dof.size(); ++i) {
            const int32_t w = (int32_t)dof.which_side()[i];
            side[i + P.ibc.IBCColumnStartIndex(c)] = w;
            const size_t bc = mc.is_oriented ? dof.which_side()[i] - 1 : 0;
            if (mc.boundary_type[bc] == 0) side[DirichletValueRow(P.ibc, c, i)] = w;
        }
    }
    return 0;
}

int cpmref_xp_export(void *hp, double *xp) {
    Problem &P = *((Handle *)hp)->prob;
    const auto &v = P.tube.surface().xp();
    for (size_t i = 0; i < v.size(); ++i)
        for (int d = 0; d < 3; ++d) xp[3 * i + d] = v[i][d];
    return 0;
}

// IBC subsets: sizes [tagging size, dof size, column start, dirichlet column start]
int cpmref_ibc_sizes(void *hp, int32_t c, int64_t *out) {
    Problem &P = *((Handle *)hp)->prob;
    out[0] = (int64_t)P.ibc.TaggingSubset()[c].size();
    out[1] = (int64_t)P.ibc.DOFSubset()[c].size();
    out[2] = (int64_t)P.ibc.IBCColumnStartIndex(c);
    out[3] = (int64_t)P.ibc.DirichletIBCColumnStartIndex(c);
    out[4] = (int64_t)P.ibc.IdentityRowsStart();
    return 0;
}

int cpmref_ibc_export(void *hp, int32_t c, int64_t *tag_set, double *tag_dist, double *tag_dir, int64_t *dof_set,
                      double *dof_cp, double *dof_cpbar, double *tag_cpdiff) {
    Problem &P = *((Handle *)hp)->prob;
    const IBCSubset &ts = P.ibc.TaggingSubset()[c];
    const IBCDOFSubset &ds = P.ibc.DOFSubset()[c];
    for (size_t i = 0; i < ts.size(); ++i) {
        if (tag_set) tag_set[i] = (int64_t)ts.SetIndexFromSubsetIndex()[i];
        if (tag_dist) tag_dist[i] = ts.dist()[i];
        for (int d = 0; d < 3; ++d) {
            if (tag_dir) tag_dir[3 * i + d] = ts.directions()[i][d];
            if (tag_cpdiff) tag_cpdiff[3 * i + d] = ts.cp_diff()[i][d];
        }
    }
    for (size_t i = 0; i < ds.size(); ++i) {
        if (dof_set) dof_set[i] = (int64_t)ds.SetIndexFromSubsetIndex()[i];
        for (int d = 0; d < 3; ++d) {
            if (dof_cp) dof_cp[3 * i + d] = ds.cpx()[i][d];
            if (dof_cpbar && !ds.cpbar().empty()) dof_cpbar[3 * i + d] = ds.cpbar()[i][d];
        }
    }
    return 0;
}

int cpmref_apply(void *hp, double m, double n, const double *x, double *y) {
    Problem &P = *((Handle *)hp)->prob;
    GeneralizedSystem sys;
    sys.SetComponents(m, n, P.Lfull, P.Efull, Preconditioner::diagonal, P.identity_rows);
    std::vector<double> xv(x, x + P.D()), yv;
    sys.Multiply(xv, yv);
    std::copy(yv.begin(), yv.end(), y);
    return 0;
}

// precond: 0 identity, 1 diagonal, 2 jacobi (precond_iters sweeps).
// stats out: [iterations, restarts, final_rel_residual2, seconds]
int cpmref_solve(void *hp, double m, double n, int32_t precond, int32_t precond_iters, const double *b, double *x, double tol,
                 int32_t max_iters, double *stats) {
    GUARD_BEGIN
    Problem &P = *((Handle *)hp)->prob;
    Solver sv;
    sv.Init(m, n, P.Lfull, P.Efull, (Preconditioner)precond, P.identity_rows);
    sv.SetPrecond(precond_iters);
    std::vector<double> bv(b, b + P.D());
    auto t0 = std::chrono::steady_clock::now();
    std::vector<double> u = sv.Solve(bv, tol, max_iters);
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::copy(u.begin(), u.end(), x);
    if (stats) {
        stats[0] = sv.stats().iterations;
        stats[1] = sv.stats().restarts;
        stats[2] = sv.stats().final_rel_residual2;
        stats[3] = secs;
    }
    return 0;
    GUARD_END
}

int cpmref_geodesic(void *hp, double dt, int32_t step1_jacobi_iters, double *phi, int32_t *iters_out) {
    GUARD_BEGIN
    Problem &P = *((Handle *)hp)->prob;
    std::vector<int> its;
    std::vector<double> r = P.GeodesicDistance(dt, step1_jacobi_iters, &its);
    std::copy(r.begin(), r.end(), phi);
    if (iters_out)
        for (size_t i = 0; i < its.size(); ++i) iters_out[i] = its[i];
    return 0;
    GUARD_END
}

int cpmref_geodesic_nearest(void *hp, int64_t n_ibc, const int64_t *ibc_idx, int64_t n_inside, const int64_t *inside_idx,
                            const double *inside_dist, double dt, int32_t step1_jacobi_iters, double *phi,
                            int32_t *iters_out) {
    GUARD_BEGIN
    Problem &P = *((Handle *)hp)->prob;
    std::vector<size_t> a((size_t)n_ibc), b((size_t)n_inside);
    std::vector<double> d((size_t)n_inside);
    for (int64_t i = 0; i < n_ibc; ++i) a[i] = (size_t)ibc_idx[i];
    for (int64_t i = 0; i < n_inside; ++i) {
        b[i] = (size_t)inside_idx[i];
        d[i] = inside_dist[i];
    }
    std::vector<int> its;
    std::vector<double> r = P.GeodesicDistanceNearest(a, b, d, dt, step1_jacobi_iters, &its);
    std::copy(r.begin(), r.end(), phi);
    if (iters_out)
        for (size_t i = 0; i < its.size(); ++i) iters_out[i] = its[i];
    return 0;
    GUARD_END
}

int cpmref_heat_nearest(void *hp, int64_t n_ibc, const int64_t *ibc_idx, int64_t n_inside, const int64_t *inside_idx,
                        const double *inside_dist, double dt, int32_t step1_jacobi_iters, double *u_out) {
    GUARD_BEGIN
    Problem &P = *((Handle *)hp)->prob;
    std::vector<size_t> a((size_t)n_ibc), b((size_t)n_inside);
    std::vector<double> d((size_t)n_inside);
    for (int64_t i = 0; i < n_ibc; ++i) a[i] = (size_t)ibc_idx[i];
    for (int64_t i = 0; i < n_inside; ++i) {
        b[i] = (size_t)inside_idx[i];
        d[i] = inside_dist[i];
    }
    std::vector<double> u = P.HeatNearest(a, b, d, dt, step1_jacobi_iters);
    std::copy(u.begin(), u.end(), u_out);
    return 0;
    GUARD_END
}

// Row loops of the sparse products on OpenMP threads (1) or serial (0, the default).
int cpmref_set_parallel_rows(int32_t on) {
    ParallelRows() = on != 0;
    return 0;
}

// OpenMP threads of the vector operations (the timed CPU baselines run with all
// host threads and with one).
int cpmref_set_num_threads(int32_t n) {
    if (n < 1) return -1;
    omp_set_num_threads(n);
    return 0;
}

// Closest point of an arbitrary point set to a surface (CP-accuracy tests).
int cpmref_closest_points(const cpmref_surface_desc *surf, int64_t n, const double *x, double *cp, double *dist) {
    GUARD_BEGIN
    Surface s(ToSpec(surf));
    for (int64_t i = 0; i < n; ++i) {
        V3 xi{x[3 * i], x[3 * i + 1], x[3 * i + 2]}, c;
        double d;
        size_t b;
        s.ClosestPoint(xi, c, d, b);
        for (int k = 0; k < 3; ++k) cp[3 * i + k] = c[k];
        dist[i] = d;
    }
    return 0;
    GUARD_END
}

}  // extern "C"
