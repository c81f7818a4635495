// Heat-method geodesic distance on the device (K12), restating
// GeodesicDistance::ComputeDistance (problems/GeodesicDistance.cpp:11-69):
//   Step1 (:75-173)  heat solve (I - dt L#) u = smoothed point indicator,
//                    Dirichlet values on the point IBC's DOF rows
//   Step2 (:179-311) g = E (Dc u), normal component projected out, normalised
//   ComputeDivergence (:317-327)  div = sum_d Dc_d g_d
//   Step3 (:330-413) Poisson solve L# phi = div (Dirichlet 0 at the source),
//                    phi -= min phi; Step2/3 repeated twice on E phi.
// The heat solve is preconditioned by damped Jacobi sweeps (2000 per
// preconditioner call, :117-119), which resolve the heat kernel's far field to
// far below the solver tolerance: the normalised gradient there follows those
// small values, so the heat solve always runs in FP64 (FP32 would also flush
// them to zero once the kernel falls below 1e-38).  The Poisson solves use the
// diagonal preconditioner (:360) and the requested precision.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "opset.h"

namespace cpm {

// central differences along d (FDMatrices::BuildGradientMatrices: +-0.5/dx at the +-e_d neighbours)
__global__ void k_grad3(int64_t N, const int32_t *__restrict__ nbr6, double dx, const double *__restrict__ u,
                        double *__restrict__ g) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= N) return;
    const double cp = 0.5 / dx, cm = -0.5 / dx;
    for (int d = 0; d < 3; ++d) {
        int a = nbr6[6 * q + 2 * d], b = nbr6[6 * q + 2 * d + 1];
        double s = 0.0;
        if (a >= 0) s += cp * u[a];
        if (b >= 0) s += cm * u[b];
        g[3 * q + d] = s;
    }
}

// E g for a 3-wide [N][3] vector on the plain tube stencil
__global__ void k_extend3(OpView<double> op, const double *__restrict__ g, double *__restrict__ eg) {
    int64_t gid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t r = gid / 3;
    int s = (int)(gid % 3);
    if (r >= op.N) return;
    eg[3 * r + s] = e_row_thread<double, 3>(op, r, s, g);
}

// E u for one vector on the plain tube stencil
__global__ void k_extend1(OpView<double> op, const double *__restrict__ u, double *__restrict__ eu) {
    int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= op.N) return;
    eu[r] = e_row_thread<double, 1>(op, r, 0, u);
}

// g -= (g.n) n ; g /= |g| (if |g| != 0)   (problems/GeodesicDistance.cpp:221-256)
__global__ void k_project_normalise(int64_t N, const double *__restrict__ nrm, double *__restrict__ g) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= N) return;
    double v[3] = {g[3 * q], g[3 * q + 1], g[3 * q + 2]}, n[3] = {nrm[3 * q], nrm[3 * q + 1], nrm[3 * q + 2]};
    double dn = 0.0;
    for (int d = 0; d < 3; ++d) dn += v[d] * n[d];
    for (int d = 0; d < 3; ++d) v[d] = v[d] - dn * n[d];
    double nn = 0.0;
    for (int d = 0; d < 3; ++d) nn += v[d] * v[d];
    nn = sqrt(nn);
    if (nn != 0.0)
        for (int d = 0; d < 3; ++d) v[d] /= nn;
    for (int d = 0; d < 3; ++d) g[3 * q + d] = v[d];
}

// div = sum_d Dc_d g_d (tube rows); rows >= N of the right-hand side are 0
__global__ void k_divergence(int64_t N, int64_t D, const int32_t *__restrict__ nbr6, double dx, const double *__restrict__ g,
                             double *__restrict__ b) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= D) return;
    if (q >= N) {
        b[q] = 0.0;
        return;
    }
    const double cp = 0.5 / dx, cm = -0.5 / dx;
    double div = 0.0;
    for (int d = 0; d < 3; ++d) {
        int a = nbr6[6 * q + 2 * d], c = nbr6[6 * q + 2 * d + 1];
        double s = 0.0;
        if (a >= 0) s += cp * g[3 * (int64_t)a + d];
        if (c >= 0) s += cm * g[3 * (int64_t)c + d];
        div = div + s;
    }
    b[q] = div;
}

__global__ void k_negate(int64_t n, const double *__restrict__ a, double *__restrict__ b) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = -a[i];
}

__global__ void k_block_min(int64_t n, const double *__restrict__ a, double *__restrict__ part) {
    __shared__ double sh[256];
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double v = 1.7976931348623157e308;
    for (; i < n; i += (int64_t)gridDim.x * blockDim.x) v = fmin(v, a[i]);
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h) sh[threadIdx.x] = fmin(sh[threadIdx.x], sh[threadIdx.x + h]);
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// phi -= min(phi) with the minimum reduced in one block
__global__ void k_sub_min(int64_t n, int nparts, const double *__restrict__ part, double *__restrict__ a) {
    __shared__ double mn;
    if (threadIdx.x == 0) {
        double v = 1.7976931348623157e308;
        for (int p = 0; p < nparts; ++p) v = fmin(v, part[p]);
        mn = v;
    }
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) a[i] -= mn;
}

}  // namespace cpm

using namespace cpm;

struct cpm_geodesic_s {
    cpm_tube_s *tube = nullptr;
    cpm_opset_t op_ibc = nullptr, op_plain = nullptr;
    int64_t N = 0, D = 0;
    std::vector<double> rhs_heat;  // Step1 right-hand side (host, D)
    ~cpm_geodesic_s() {
        if (op_ibc) cpm_opset_destroy(op_ibc);
        if (op_plain) cpm_opset_destroy(op_plain);
    }
};

extern "C" int cpm_geodesic_create(cpm_tube_t t, const double *source, cpm_geodesic_t *out, int64_t *D_out) {
    if (!t || !source || !out) return fail(CPM_ERR_INVALID_ARG, "geodesic_create: null argument");
    *out = nullptr;
    cpm_geodesic_s *g = new cpm_geodesic_s();
    g->tube = t;
    cpm_surface_desc pd;
    memset(&pd, 0, sizeof(pd));
    pd.kind = CPM_POINT;
    pd.nparams = 3;
    for (int d = 0; d < 3; ++d) pd.params[d] = source[d];
    pd.bbox[0] = t->surf.desc.bbox[0];
    pd.bbox[1] = t->surf.desc.bbox[1];
    pd.boundary_order = 1;  // IBCMetaData default (src/IBCMetaData.h:15)
    pd.use_Jcp_surface_normals = 1;
    pd.on_ibc_tolerance = 0.1 * t->g.dx * t->g.dx;  // as the reference's geodesic drivers set it
    pd.dof_radius_scale = 1.0;
    int rc = cpm_opset_create(t, 1, &pd, &g->op_ibc);
    if (!rc) rc = cpm_opset_create(t, 0, nullptr, &g->op_plain);
    if (rc) {
        delete g;
        return rc;
    }
    g->N = g->op_ibc->N;
    g->D = g->op_ibc->D;
    // Step1 right-hand side: SmoothH(t) = 0.5 tanh(-scale t) + 0.5, scale = atanh(1 - dx) / r
    const double extent = t->g.radius, tol = t->g.dx;
    const double scale = std::atanh(1 - tol) / extent;
    auto smooth = [scale](double x) { return 0.5 * std::tanh(-scale * x) + 0.5; };
    g->rhs_heat.assign(g->D, 0.0);
    const auto &dof = g->op_ibc->dof_set[0];
    const auto &cd = g->op_ibc->dof_cpdiff[0];
    const int64_t start = g->op_ibc->col_start[0] + g->op_ibc->identity_rows_start;
    for (size_t i = 0; i < dof.size(); ++i) {
        double n2 = 0.0;
        for (int k = 0; k < 3; ++k) n2 += cd[3 * i + k] * cd[3 * i + k];
        g->rhs_heat[start + (int64_t)i] = smooth(-std::sqrt(n2));
    }
    for (size_t i = 0; i < dof.size(); ++i) {
        double n2 = 0.0;
        for (int k = 0; k < 3; ++k) n2 += cd[3 * i + k] * cd[3 * i + k];
        g->rhs_heat[dof[i]] = smooth(std::sqrt(n2));
    }
    if (D_out) *D_out = g->D;
    *out = g;
    return 0;
}

extern "C" int cpm_geodesic_run(cpm_geodesic_t g, double dt, int32_t precision, double tol, int32_t heat_sweeps,
                                double *phi_out, int32_t *iters_out) {
    if (!g || !phi_out || dt <= 0) return fail(CPM_ERR_INVALID_ARG, "geodesic_run: invalid arguments");
    const int64_t N = g->N, D = g->D;
    const double dx = g->tube->g.dx;
    auto plain = g->op_plain->view<double>();
    const int32_t *nbr6 = g->op_ibc->nbr6.p;  // tube-row neighbours (moves only affect IBC rows' columns)
    // the plain operator's neighbour table: Dc uses the original 6-neighbourhood
    nbr6 = g->op_plain->nbr6.p;
    DBuf<double> b, x, u, gr, eg, part;
    CPM_TRY(b.alloc(D));
    CPM_TRY(x.alloc(D));
    CPM_TRY(u.alloc(N));
    CPM_TRY(gr.alloc(3 * N));
    CPM_TRY(eg.alloc(3 * N));
    const int nparts = 256;
    CPM_TRY(part.alloc(nparts));
    cudaStream_t st = stream();
    cpm_solve_opts o;
    memset(&o, 0, sizeof(o));
    o.tol = tol > 0 ? tol : 1e-10;
    o.max_iters = 100000;
    o.precision = 0;
    o.precond = 2;
    o.precond_iters = heat_sweeps > 0 ? heat_sweeps : 2000;
    cpm_solve_stats ss;
    cpm_solver_t heat = nullptr, pois = nullptr;
    CPM_TRY(cpm_solver_create(g->op_ibc, 1.0, -dt, 1, &heat));
    int rc = cpm_solver_create(g->op_ibc, 0.0, 1.0, 1, &pois);
    auto cleanup = [&](int r) {
        if (heat) cpm_solver_destroy(heat);
        if (pois) cpm_solver_destroy(pois);
        return r;
    };
    if (rc) return cleanup(rc);
    const unsigned bN = (unsigned)((N + 255) / 256), bD = (unsigned)((D + 255) / 256);
    // Step1: heat flow from the point; u = -ufull[0:N]
    CPM_CUDA_TRY(cudaMemcpyAsync(b.p, g->rhs_heat.data(), D * 8, cudaMemcpyHostToDevice, st));
    if ((rc = cpm_solve_device(heat, 1, b.p, x.p, &o, &ss))) return cleanup(rc);
    if (iters_out) iters_out[0] = ss.iterations;
    o.precision = precision;
    o.precond = 1;
    o.precond_iters = 0;
    k_negate<<<bN, 256, 0, st>>>(N, x.p, u.p);
    count_launches(1);
    for (int round = 0; round < 3; ++round) {
        if (round > 0) {  // u = E phi[0:N]
            k_extend1<<<bN, 256, 0, st>>>(plain, x.p, u.p);
            count_launches(1);
        }
        // Step2 + ComputeDivergence
        k_grad3<<<bN, 256, 0, st>>>(N, nbr6, dx, u.p, gr.p);
        k_extend3<<<(unsigned)((3 * N + 255) / 256), 256, 0, st>>>(plain, gr.p, eg.p);
        k_project_normalise<<<bN, 256, 0, st>>>(N, g->op_ibc->normals.p, eg.p);
        k_divergence<<<bD, 256, 0, st>>>(N, D, nbr6, dx, eg.p, b.p);
        count_launches(4);
        CPM_CUDA_TRY(cudaGetLastError());
        // Step3: Poisson solve, then phi -= min phi
        if ((rc = cpm_solve_device(pois, 1, b.p, x.p, &o, &ss))) return cleanup(rc);
        if (iters_out) iters_out[1 + round] = ss.iterations;
        // the rounds solve with the same operator: once its FP32 iteration has had to
        // fall back to FP64, the later rounds go to FP64 directly
        if (ss.fp64_fallback) o.precision = 0;
        k_block_min<<<nparts, 256, 0, st>>>(D, x.p, part.p);
        k_sub_min<<<bD, 256, 0, st>>>(D, nparts, part.p, x.p);
        count_launches(2);
    }
    CPM_CUDA_TRY(cudaMemcpyAsync(phi_out, x.p, D * 8, cudaMemcpyDeviceToHost, st));
    CPM_CUDA_TRY(cudaStreamSynchronize(st));
    return cleanup(0);
}

extern "C" int cpm_geodesic_destroy(cpm_geodesic_t g) {
    delete g;
    return 0;
}
