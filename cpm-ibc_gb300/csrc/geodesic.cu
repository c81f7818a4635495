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


// ---------------------------------------------------------------------------
// GeodesicDistanceNearest (problems/GeodesicDistanceNearest.cpp:11-345): the
// plain tube operator with identity rows at the constraint nodes.  Its heat
// step solves the TRANSPOSE of the implicit-Euler matrix
// I - dt (diag(L) + (L - diag(L)) E) (Helpers::ImplicitEulerMatrix,
// src/Helpers.cpp:292-299; the reference factorises Afull.transpose() with a
// sparse LU, :103-133) whose constraint rows are then identity rows.  L is
// symmetric (the 7-point stencil over tube neighbours), so row k of that
// matrix applied to v is
//   v_k - dt (L_kk v_k + sum_q E_qk w_q),   w_q = sum_{c != q} L_qc v_c,
// and the E^T gather runs over the base groups: column k lies in the 4^3
// stencil of group g at offset (i, j, l) exactly when g's base node is
// k - (i, j, l).  The sums run in a fixed order (deterministic).

// grp_of[node] = the base group whose base point is that tube node
__global__ void k_group_of_base(OpView<double> op, int32_t *__restrict__ grp_of, int32_t *__restrict__ err) {
    const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g >= op.n_grp) return;
    const uint32_t b = op.base[op.ord[op.grp[g]]];
    const int nd = node_at(op.bv, unpack_i(b), unpack_j(b), unpack_k(b));
    if (nd < 0) {
        atomicExch(err, 1);
        return;
    }
    grp_of[nd] = (int32_t)g;
}

// w_q = sum over q's tube neighbours c of L_qc v_c
__global__ void k_loff_sum(int64_t N, const int32_t *__restrict__ nbr6, double Loff, const double *__restrict__ v,
                           double *__restrict__ w) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= N) return;
    double s = 0.0;
    for (int e = 0; e < 6; ++e) {
        const int c = nbr6[6 * q + e];
        if (c >= 0) s += Loff * v[c];
    }
    w[q] = s;
}

// y = A^T v (in == nullptr), or one damped Jacobi sweep y = v + omega (in - A^T v) / d
// with the matrix-free diagonal d = 1 - dt L_kk (1 on identity rows), as the
// reference's Jacobi preconditioner forms it (src/GeneralizedBiCGStabSystem.h:281-385)
__global__ void k_heat_transposed(OpView<double> op, const int32_t *__restrict__ grp_of, const uint8_t *__restrict__ ident,
                                  double dt, const double *__restrict__ v, const double *__restrict__ w,
                                  const double *__restrict__ in, double omega, double *__restrict__ y) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= op.N) return;
    const double vk = v[k];
    double ak, d = 1.0;
    if (ident[k] & F_IDENT) {
        ak = vk;
    } else {
        const uint32_t key = op.key[k];
        const int ci = unpack_i(key), cj = unpack_j(key), ck = unpack_k(key);
        double z = 0.0;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j)
                for (int l = 0; l < 4; ++l) {
                    const int nd = node_at(op.bv, ci - i, cj - j, ck - l);
                    if (nd < 0) continue;
                    const int g = grp_of[nd];
                    if (g < 0) continue;
                    const int p1 = op.grp[g + 1];
                    for (int p = op.grp[g]; p < p1; ++p) {
                        const double *wp = op.w_ord + 12 * (int64_t)p;
                        z += ((wp[8 + l] * wp[4 + j]) * wp[i]) * w[op.ord[p]];
                    }
                }
        ak = vk - dt * (op.Ldiag * vk + z);
        d = 1.0 + op.Ldiag * (-dt);
    }
    y[k] = in ? vk + omega * ((in[k] - ak) / d) : ak;
}

// deterministic dot product: fixed grid of block partials, summed in order by one thread
constexpr int NEAREST_DOT_BLOCKS = 304;
// the Jacobi-preconditioned heat step converges in a few iterations; each costs
// 4 x (sweeps) launches, so the cap bounds a non-converging run to seconds
constexpr int NEAREST_HEAT_MAX_ITERS = 1000;
__global__ void k_dot_parts(int64_t n, const double *__restrict__ a, const double *__restrict__ b, double *__restrict__ part) {
    __shared__ double sh[256];
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += a[i] * b[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
__global__ void k_sum_parts(int nparts, const double *__restrict__ part, double *__restrict__ out) {
    double s = 0.0;
    for (int p = 0; p < nparts; ++p) s += part[p];
    *out = s;
}

// BiCGStab vector steps in the reference's operation order (src/BiCGStab.h:64-100)
__global__ void k_bicg_p(int64_t n, double beta, double w, const double *__restrict__ r, const double *__restrict__ v,
                         double *__restrict__ p) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double pi = -w * v[i] + p[i];
    pi *= beta;
    p[i] = pi + r[i];
}
__global__ void k_bicg_s(int64_t n, double alpha, const double *__restrict__ r, const double *__restrict__ v,
                         double *__restrict__ s) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) s[i] = -alpha * v[i] + r[i];
}
__global__ void k_bicg_xr(int64_t n, double alpha, double w, const double *__restrict__ y, const double *__restrict__ z,
                          const double *__restrict__ s, const double *__restrict__ t, double *__restrict__ x,
                          double *__restrict__ r) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double xi = alpha * y[i] + x[i];
    x[i] = w * z[i] + xi;
    r[i] = -w * t[i] + s[i];
}
__global__ void k_sub(int64_t n, const double *__restrict__ a, const double *__restrict__ b, double *__restrict__ c) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) c[i] = a[i] - b[i];
}
__global__ void k_zero_rows(int64_t n, const int32_t *__restrict__ rows, double *__restrict__ b) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[rows[i]] = 0.0;
}
// ---- the same steps for 32-slot batches ([rows][32], one source per slot)

// central differences along each axis of every slot: gx, gy, gz ([D][32]; rows >= N untouched)
__global__ void k_grad3_32(int64_t N, const int32_t *__restrict__ nbr6, double dx, const double *__restrict__ u,
                           double *__restrict__ gx, double *__restrict__ gy, double *__restrict__ gz) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= N * 32) return;
    const int64_t q = i >> 5;
    const int k = (int)(i & 31);
    const double cp = 0.5 / dx, cm = -0.5 / dx;
    double *g[3] = {gx, gy, gz};
    for (int d = 0; d < 3; ++d) {
        const int a = nbr6[6 * q + 2 * d], b = nbr6[6 * q + 2 * d + 1];
        double s = 0.0;
        if (a >= 0) s += cp * u[(int64_t)a * 32 + k];
        if (b >= 0) s += cm * u[(int64_t)b * 32 + k];
        g[d][i] = s;
    }
}

// g -= (g.n) n ; g /= |g| for every tube row and slot
__global__ void k_project_normalise32(int64_t N, const double *__restrict__ nrm, double *__restrict__ gx, double *__restrict__ gy,
                                      double *__restrict__ gz) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= N * 32) return;
    const int64_t q = i >> 5;
    double v[3] = {gx[i], gy[i], gz[i]}, n[3] = {nrm[3 * q], nrm[3 * q + 1], nrm[3 * q + 2]};
    double dn = 0.0;
    for (int d = 0; d < 3; ++d) dn += v[d] * n[d];
    for (int d = 0; d < 3; ++d) v[d] = v[d] - dn * n[d];
    double nn = 0.0;
    for (int d = 0; d < 3; ++d) nn += v[d] * v[d];
    nn = sqrt(nn);
    if (nn != 0.0)
        for (int d = 0; d < 3; ++d) v[d] /= nn;
    gx[i] = v[0];
    gy[i] = v[1];
    gz[i] = v[2];
}

// div = sum_d Dc_d g_d on the tube rows of every slot; rows >= N are 0
__global__ void k_divergence32(int64_t N, int64_t D, const int32_t *__restrict__ nbr6, double dx, const double *__restrict__ gx,
                               const double *__restrict__ gy, const double *__restrict__ gz, double *__restrict__ b) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= D * 32) return;
    const int64_t q = i >> 5;
    const int k = (int)(i & 31);
    if (q >= N) {
        b[i] = 0.0;
        return;
    }
    const double cp = 0.5 / dx, cm = -0.5 / dx;
    const double *g[3] = {gx, gy, gz};
    double div = 0.0;
    for (int d = 0; d < 3; ++d) {
        const int a = nbr6[6 * q + 2 * d], c = nbr6[6 * q + 2 * d + 1];
        double s = 0.0;
        if (a >= 0) s += cp * g[d][(int64_t)a * 32 + k];
        if (c >= 0) s += cm * g[d][(int64_t)c * 32 + k];
        div = div + s;
    }
    b[i] = div;
}

// b = -a on the first n rows of a [rows][32] batch
__global__ void k_negate32(int64_t n, const double *__restrict__ a, double *__restrict__ b) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n * 32) b[i] = -a[i];
}

// per-slot minimum over D rows: block partial minima part[block][32]
__global__ void k_colmin32(int64_t D, const double *__restrict__ a, double *__restrict__ part) {
    __shared__ double sh[8][32];
    const int k = threadIdx.x & 31, rw = threadIdx.x >> 5;
    double v = 1.7976931348623157e308;
    for (int64_t q = (int64_t)blockIdx.x * 8 + rw; q < D; q += (int64_t)gridDim.x * 8) v = fmin(v, a[q * 32 + k]);
    sh[rw][k] = v;
    __syncthreads();
    if (rw == 0) {
        for (int j = 1; j < 8; ++j) v = fmin(v, sh[j][k]);
        part[(int64_t)blockIdx.x * 32 + k] = v;
    }
}

// phi -= min over the slot's rows (the partial minima of k_colmin32)
__global__ void k_sub_colmin32(int64_t D, int nparts, const double *__restrict__ part, double *__restrict__ a) {
    __shared__ double mn[32];
    if (threadIdx.x < 32) {
        double v = 1.7976931348623157e308;
        for (int p = 0; p < nparts; ++p) v = fmin(v, part[(int64_t)p * 32 + threadIdx.x]);
        mn[threadIdx.x] = v;
    }
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D * 32; i += (int64_t)gridDim.x * blockDim.x)
        a[i] -= mn[i & 31];
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

// ---------------------------------------------------------------------------
// The heat-method geodesic distance from up to 32 sources at once.  No
// counterpart in the reference, whose GeodesicDistance::ComputeDistance
// (problems/GeodesicDistance.cpp:11-69) serves one source per call with its own
// point-IBC operator.  Here the sources share one operator: the tube's bulk
// stencils with every source's point IBC as per-slot patch records
// (opset_create_point_batch), so each step is one 32-slot solve in which every
// slot carries exactly its own source's operator; Step 2 runs on all slots at
// once.  Each source's result equals its one-source run up to rounding.
struct cpm_geodesic_batch_s {
    cpm_tube_s *tube = nullptr;
    cpm_opset_s *op = nullptr;
    PointBatchInfo info;
    int n_src = 0;
    int64_t N = 0, D = 0;
    ~cpm_geodesic_batch_s() { delete op; }
};

extern "C" int cpm_geodesic_batch_create(cpm_tube_t t, int32_t n_src, const double *sources, cpm_geodesic_batch_t *out,
                                         int64_t *D_out) {
    if (!t || !sources || !out || n_src < 1 || n_src > 32)
        return fail(CPM_ERR_INVALID_ARG, "geodesic_batch_create: 1 to 32 sources");
    *out = nullptr;
    cpm_geodesic_batch_s *g = new cpm_geodesic_batch_s();
    g->tube = t;
    g->n_src = n_src;
    const int rc = opset_create_point_batch(t, n_src, sources, &g->op, g->info);
    if (rc) {
        delete g;
        return rc;
    }
    g->N = g->op->N;
    g->D = g->op->D;
    if (D_out) *D_out = g->D;
    *out = g;
    return 0;
}

extern "C" int cpm_geodesic_batch_run(cpm_geodesic_batch_t g, double dt, double tol, int32_t heat_sweeps, double *phi_out,
                                      int32_t *iters_out) {
    if (!g || !phi_out || dt <= 0) return fail(CPM_ERR_INVALID_ARG, "geodesic_batch_run: invalid arguments");
    const int64_t N = g->N, D = g->D;
    const int K = 32, ns = g->n_src;
    const double dx = g->tube->g.dx;
    const int32_t *nbr6 = g->op->nbr6.p;  // tube rows: the plain neighbours (no L moves in the bulk)
    cudaStream_t st = stream();
    // Step 1 right-hand sides: SmoothH at the DOF rows (Dirichlet values) and at the DOF nodes' tube rows
    const double extent = g->tube->g.radius, tolr = g->tube->g.dx;
    const double scale = std::atanh(1 - tolr) / extent;
    auto smooth = [scale](double x) { return 0.5 * std::tanh(-scale * x) + 0.5; };
    std::vector<double> hb((size_t)D * K, 0.0);
    for (int k = 0; k < ns; ++k) {
        const auto &dof = g->info.dof_set[k];
        const auto &cd = g->info.dof_cpdiff[k];
        for (size_t i = 0; i < dof.size(); ++i) {
            double n2 = 0.0;
            for (int c = 0; c < 3; ++c) n2 += cd[3 * i + c] * cd[3 * i + c];
            hb[(size_t)(N + (int64_t)i) * K + k] = smooth(-std::sqrt(n2));
        }
        for (size_t i = 0; i < dof.size(); ++i) {
            double n2 = 0.0;
            for (int c = 0; c < 3; ++c) n2 += cd[3 * i + c] * cd[3 * i + c];
            hb[(size_t)dof[i] * K + k] = smooth(std::sqrt(n2));
        }
    }
    DBuf<double> b, x, u, gx, gy, gz, part;
    CPM_TRY(b.upload(hb));
    for (auto *a : {&x, &u, &gx, &gy, &gz}) {
        CPM_TRY(a->alloc((size_t)D * K));
        CPM_TRY(a->zero());
    }
    const int nparts = 256;
    CPM_TRY(part.alloc((size_t)nparts * K));
    cpm_solve_opts o;
    memset(&o, 0, sizeof(o));
    o.tol = tol > 0 ? tol : 1e-10;
    o.max_iters = 100000;
    o.precision = 0;
    o.precond = 2;
    o.precond_iters = heat_sweeps > 0 ? heat_sweeps : 2000;
    std::vector<cpm_solve_stats> ss(ns);
    cpm_solver_t heat = nullptr, pois = nullptr;
    CPM_TRY(cpm_solver_create(g->op, 1.0, -dt, K, &heat));
    int rc = cpm_solver_create(g->op, 0.0, 1.0, K, &pois);
    auto cleanup = [&](int r) {
        if (heat) cpm_solver_destroy(heat);
        if (pois) cpm_solver_destroy(pois);
        return r;
    };
    if (rc) return cleanup(rc);
    const unsigned bN = (unsigned)((N * K + 255) / 256), bD = (unsigned)((D * K + 255) / 256);
    // Step 1: heat flow from each source; u = -x[0:N]
    if ((rc = cpm_solve_device(heat, ns, b.p, x.p, &o, ss.data()))) return cleanup(rc);
    if (iters_out)
        for (int k = 0; k < ns; ++k) iters_out[4 * k] = ss[k].iterations;
    o.precond = 1;
    o.precond_iters = 0;
    k_negate32<<<bN, 256, 0, st>>>(N, x.p, u.p);
    count_launches(1);
    for (int round = 0; round < 3; ++round) {
        if (round > 0) CPM_TRY(epass64_batch(g->op, false, x.p, u.p));  // u = E phi (plain E)
        // Step 2 + ComputeDivergence
        k_grad3_32<<<bN, 256, 0, st>>>(N, nbr6, dx, u.p, gx.p, gy.p, gz.p);
        count_launches(1);
        for (DBuf<double> *gd : {&gx, &gy, &gz}) {
            CPM_TRY(epass64_batch(g->op, false, gd->p, b.p));
            CPM_CUDA_TRY(cudaMemcpyAsync(gd->p, b.p, (size_t)N * K * 8, cudaMemcpyDeviceToDevice, st));
        }
        k_project_normalise32<<<bN, 256, 0, st>>>(N, g->op->normals.p, gx.p, gy.p, gz.p);
        k_divergence32<<<bD, 256, 0, st>>>(N, D, nbr6, dx, gx.p, gy.p, gz.p, b.p);
        count_launches(2);
        CPM_CUDA_TRY(cudaGetLastError());
        // Step 3: Poisson solve of every slot, then phi -= min phi per slot
        if ((rc = cpm_solve_device(pois, ns, b.p, x.p, &o, ss.data()))) return cleanup(rc);
        if (iters_out)
            for (int k = 0; k < ns; ++k) iters_out[4 * k + 1 + round] = ss[k].iterations;
        k_colmin32<<<nparts, 256, 0, st>>>(D, x.p, part.p);
        k_sub_colmin32<<<bD, 256, 0, st>>>(D, nparts, part.p, x.p);
        count_launches(2);
    }
    // phi of source k: [D] rows (tube rows, then its own DOF rows; the rows past its DOFs are 0)
    std::vector<double> hx;
    CPM_TRY(x.download(hx, (size_t)D * K));
    for (int k = 0; k < ns; ++k) {
        const int64_t Dk = N + (int64_t)g->info.dof_set[k].size();
        for (int64_t r = 0; r < D; ++r) phi_out[(size_t)k * D + r] = r < Dk ? hx[(size_t)r * K + k] : 0.0;
    }
    return cleanup(0);
}

extern "C" int cpm_geodesic_batch_destroy(cpm_geodesic_batch_t g) {
    delete g;
    return 0;
}

// ---------------------------------------------------------------------------
// GeodesicDistanceNearest::ComputeDistance (problems/GeodesicDistanceNearest.cpp:11-53)
struct cpm_geodesic_nearest_s {
    cpm_tube_s *tube = nullptr;
    cpm_opset_t op_plain = nullptr, op_id = nullptr;
    int64_t N = 0;
    DBuf<int32_t> grp_of;
    std::vector<double> rhs_heat;  // Step1 right-hand side (:62-90)
    ~cpm_geodesic_nearest_s() {
        if (op_id) cpm_opset_destroy(op_id);
        if (op_plain) cpm_opset_destroy(op_plain);
    }
};

extern "C" int cpm_geodesic_nearest_create(cpm_tube_t t, int64_t n_ibc, const int64_t *ibc_rows, int64_t n_inside,
                                           const int64_t *inside_rows, const double *inside_dist,
                                           cpm_geodesic_nearest_t *out) {
    if (!t || !out || n_ibc < 0 || n_inside < 0 || (n_ibc > 0 && !ibc_rows) || (n_inside > 0 && (!inside_rows || !inside_dist)))
        return fail(CPM_ERR_INVALID_ARG, "geodesic_nearest_create: invalid arguments");
    *out = nullptr;
    const int64_t N = t->N;
    for (int64_t i = 0; i < n_ibc; ++i)
        if (ibc_rows[i] < 0 || ibc_rows[i] >= N) return fail(CPM_ERR_INVALID_ARG, "geodesic_nearest_create: constraint row outside the tube");
    for (int64_t i = 0; i < n_inside; ++i)
        if (inside_rows[i] < 0 || inside_rows[i] >= N)
            return fail(CPM_ERR_INVALID_ARG, "geodesic_nearest_create: inside row outside the tube");
    cpm_geodesic_nearest_s *g = new cpm_geodesic_nearest_s();
    g->tube = t;
    g->N = N;
    auto bail = [&](int rc) {
        delete g;
        return rc;
    };
    int rc = cpm_opset_create(t, 0, nullptr, &g->op_plain);
    if (!rc) rc = opset_tube_normals(g->op_plain);  // ComputeSurfaceNormals (:311-345)
    if (!rc) rc = cpm_opset_create_identity(t, n_ibc, ibc_rows, &g->op_id);
    if (!rc) rc = g->grp_of.alloc(N);
    if (rc) return bail(rc);
    cudaStream_t st = stream();
    DBuf<int32_t> err;
    if ((rc = err.alloc(1)) || (rc = err.zero())) return bail(rc);
    if (cudaMemsetAsync(g->grp_of.p, 0xff, N * sizeof(int32_t), st) != cudaSuccess)
        return bail(fail(CPM_ERR_CUDA, "geodesic_nearest_create: memset"));
    const cpm_opset_s *op = g->op_plain;
    if (op->n_grp > 0) {
        k_group_of_base<<<(unsigned)((op->n_grp + 255) / 256), 256, 0, st>>>(op->view<double>(), g->grp_of.p, err.p);
        count_launches(1);
    }
    std::vector<int32_t> he;
    if ((rc = err.download(he, 1))) return bail(rc);
    if (he[0]) return bail(fail(CPM_ERR_BASEPOINT_OUTSIDE_TUBE, "geodesic_nearest_create: a base point is not a tube node"));
    // Step1 right-hand side: SmoothH(t) = 0.5 tanh(-scale t) + 0.5, scale = atanh(1 - dx) / r;
    // constraint rows t = -|x - cp|, inside rows t = -dist (later entries win, as in the reference)
    std::vector<uint32_t> key;
    std::vector<double> cp;
    if ((rc = t->key.download(key, N)) || (rc = t->cp.download(cp, 3 * N))) return bail(rc);
    const double scale = std::atanh(1 - t->g.dx) / t->g.radius;
    auto smooth = [scale](double x) { return 0.5 * std::tanh(-scale * x) + 0.5; };
    g->rhs_heat.assign(N, 0.0);
    for (int64_t i = 0; i < n_ibc; ++i) {
        const int64_t r = ibc_rows[i];
        const int ijk[3] = {unpack_i(key[r]), unpack_j(key[r]), unpack_k(key[r])};
        double s = 0.0;
        for (int d = 0; d < 3; ++d) {
            const double e = (t->g.xstart + (double)ijk[d] * t->g.dx) - cp[3 * r + d];
            s += e * e;
        }
        g->rhs_heat[r] = smooth(-std::sqrt(s));
    }
    for (int64_t i = 0; i < n_inside; ++i) g->rhs_heat[inside_rows[i]] = smooth(-inside_dist[i]);
    *out = g;
    return 0;
}

extern "C" int cpm_geodesic_nearest_run(cpm_geodesic_nearest_t g, double dt, int32_t precision, double tol, int32_t heat_sweeps,
                                        double *phi_out, int32_t *iters_out) {
    if (!g || !phi_out || dt <= 0) return fail(CPM_ERR_INVALID_ARG, "geodesic_nearest_run: invalid arguments");
    const int64_t N = g->N;
    const double dx = g->tube->g.dx;
    const cpm_opset_s *pl = g->op_plain;
    auto plain = pl->view<double>();
    const int32_t *nbr6 = pl->nbr6.p;
    const uint8_t *ident = g->op_id->flags.p;
    const double Loff = plain.Loff, omega = 2.0 / 3.0;
    const int sweeps = heat_sweeps > 0 ? heat_sweeps : 2000;
    const double rtol = tol > 0 ? tol : 1e-10;
    DBuf<double> b, x, r, r0, p, v, s, tt, y, z, w, jac, part, dsc;
    for (DBuf<double> *q : {&b, &x, &r, &r0, &p, &v, &s, &tt, &y, &z, &w, &jac}) CPM_TRY(q->alloc(N));
    CPM_TRY(part.alloc(NEAREST_DOT_BLOCKS));
    CPM_TRY(dsc.alloc(1));
    cudaStream_t st = stream();
    const unsigned bN = (unsigned)((N + 255) / 256);
    auto dot = [&](const double *a, const double *c, double &out) -> int {
        k_dot_parts<<<NEAREST_DOT_BLOCKS, 256, 0, st>>>(N, a, c, part.p);
        k_sum_parts<<<1, 1, 0, st>>>(NEAREST_DOT_BLOCKS, part.p, dsc.p);
        count_launches(2);
        CPM_CUDA_TRY(cudaMemcpyAsync(&out, dsc.p, sizeof(double), cudaMemcpyDeviceToHost, st));
        CPM_CUDA_TRY(cudaStreamSynchronize(st));
        return 0;
    };
    // A^T v -> o
    auto multiply = [&](const double *in_v, double *o) {
        k_loff_sum<<<bN, 256, 0, st>>>(N, nbr6, Loff, in_v, w.p);
        k_heat_transposed<<<bN, 256, 0, st>>>(plain, g->grp_of.p, ident, dt, in_v, w.p, nullptr, 0.0, o);
        count_launches(2);
    };
    // damped Jacobi sweeps from o = 0 (src/GeneralizedBiCGStabSystem.h:350-385)
    auto precondition = [&](const double *in, double *o) -> int {
        CPM_CUDA_TRY(cudaMemsetAsync(o, 0, N * sizeof(double), st));
        double *cur = o, *nxt = jac.p;
        for (int it = 0; it < sweeps; ++it) {
            k_loff_sum<<<bN, 256, 0, st>>>(N, nbr6, Loff, cur, w.p);
            k_heat_transposed<<<bN, 256, 0, st>>>(plain, g->grp_of.p, ident, dt, cur, w.p, in, omega, nxt);
            std::swap(cur, nxt);
        }
        count_launches(2LL * sweeps);
        if (cur != o) CPM_CUDA_TRY(cudaMemcpyAsync(o, cur, N * sizeof(double), cudaMemcpyDeviceToDevice, st));
        CPM_CUDA_TRY(cudaGetLastError());
        return 0;
    };
    // Step1: BiCGStab (src/BiCGStab.h:30-108) on the transposed heat matrix, x0 = 0
    CPM_CUDA_TRY(cudaMemcpyAsync(b.p, g->rhs_heat.data(), N * 8, cudaMemcpyHostToDevice, st));
    CPM_TRY(x.zero());
    CPM_TRY(v.zero());
    CPM_TRY(p.zero());
    CPM_CUDA_TRY(cudaMemcpyAsync(r.p, b.p, N * 8, cudaMemcpyDeviceToDevice, st));
    CPM_CUDA_TRY(cudaMemcpyAsync(r0.p, b.p, N * 8, cudaMemcpyDeviceToDevice, st));
    double r0_sq = 0, rhs_sq = 0, rr = 0;
    CPM_TRY(dot(r0.p, r0.p, r0_sq));
    CPM_TRY(dot(b.p, b.p, rhs_sq));
    int iters = 0, restarts = 0;
    if (rhs_sq > 0.0) {
        double rho = 1.0, alpha = 1.0, om = 1.0;
        const double tol2 = rtol * rtol * rhs_sq, eps = 2.220446049250313e-16, eps2 = eps * eps;
        rr = r0_sq;
        while (rr > tol2 && iters < NEAREST_HEAT_MAX_ITERS) {
            const double rho_old = rho;
            CPM_TRY(dot(r0.p, r.p, rho));
            if (std::abs(rho) < eps2 * r0_sq) {  // restart from the true residual
                multiply(x.p, r0.p);
                k_sub<<<bN, 256, 0, st>>>(N, b.p, r0.p, r.p);
                count_launches(1);
                CPM_CUDA_TRY(cudaMemcpyAsync(r0.p, r.p, N * 8, cudaMemcpyDeviceToDevice, st));
                CPM_TRY(dot(r.p, r.p, r0_sq));
                rho = r0_sq;
                if (restarts++ == 0) iters = 0;
            }
            const double beta = (rho / rho_old) * (alpha / om);
            k_bicg_p<<<bN, 256, 0, st>>>(N, beta, om, r.p, v.p, p.p);
            count_launches(1);
            CPM_TRY(precondition(p.p, y.p));
            multiply(y.p, v.p);
            double r0v = 0;
            CPM_TRY(dot(r0.p, v.p, r0v));
            alpha = rho / r0v;
            k_bicg_s<<<bN, 256, 0, st>>>(N, alpha, r.p, v.p, s.p);
            count_launches(1);
            CPM_TRY(precondition(s.p, z.p));
            multiply(z.p, tt.p);
            double t2 = 0, ts = 0;
            CPM_TRY(dot(tt.p, tt.p, t2));
            if (t2 > 0.0) CPM_TRY(dot(tt.p, s.p, ts));
            om = t2 > 0.0 ? ts / t2 : 0.0;
            k_bicg_xr<<<bN, 256, 0, st>>>(N, alpha, om, y.p, z.p, s.p, tt.p, x.p, r.p);
            count_launches(1);
            ++iters;
            CPM_TRY(dot(r.p, r.p, rr));
        }
        if (!(rr <= tol2)) return fail(CPM_ERR_NOT_CONVERGED, "geodesic_nearest_run: heat step did not converge");
    }
    if (iters_out) iters_out[0] = iters;
    // u = -(E u) (:136 and :25)
    k_extend1<<<bN, 256, 0, st>>>(plain, x.p, y.p);
    k_negate<<<bN, 256, 0, st>>>(N, y.p, z.p);
    count_launches(2);
    double *u = z.p;
    // Steps 2 and 3 with the Poisson solve (m = 0, n = 1, diagonal preconditioner, :244-293)
    cpm_solve_opts o;
    memset(&o, 0, sizeof(o));
    o.tol = rtol;
    o.max_iters = 100000;
    o.precision = precision;
    o.precond = 1;
    cpm_solve_stats ss;
    cpm_solver_t pois = nullptr;
    CPM_TRY(cpm_solver_create(g->op_id, 0.0, 1.0, 1, &pois));
    auto done = [&](int rc2) {
        cpm_solver_destroy(pois);
        return rc2;
    };
    DBuf<double> gr, eg;
    int rc = gr.alloc(3 * N);
    if (!rc) rc = eg.alloc(3 * N);
    if (rc) return done(rc);
    const int nparts = 256;
    const int64_t n_id = g->op_id->n_ident;
    for (int round = 0; round < 3; ++round) {
        if (round > 0) {  // u = E phi (:36-41)
            k_extend1<<<bN, 256, 0, st>>>(plain, x.p, z.p);
            count_launches(1);
        }
        k_grad3<<<bN, 256, 0, st>>>(N, nbr6, dx, u, gr.p);
        k_extend3<<<(unsigned)((3 * N + 255) / 256), 256, 0, st>>>(plain, gr.p, eg.p);
        k_project_normalise<<<bN, 256, 0, st>>>(N, pl->normals.p, eg.p);
        k_divergence<<<bN, 256, 0, st>>>(N, N, nbr6, dx, eg.p, b.p);
        count_launches(4);
        if (n_id > 0) {
            k_zero_rows<<<(unsigned)((n_id + 255) / 256), 256, 0, st>>>(n_id, g->op_id->ident.p, b.p);
            count_launches(1);
        }
        if (cudaGetLastError() != cudaSuccess) return done(fail(CPM_ERR_CUDA, "geodesic_nearest_run: launch failed"));
        if ((rc = cpm_solve_device(pois, 1, b.p, x.p, &o, &ss))) return done(rc);
        if (iters_out) iters_out[1 + round] = ss.iterations;
        if (ss.fp64_fallback) o.precision = 0;
        k_block_min<<<nparts, 256, 0, st>>>(N, x.p, part.p);
        k_sub_min<<<bN, 256, 0, st>>>(N, nparts, part.p, x.p);
        count_launches(2);
    }
    if (cudaMemcpyAsync(phi_out, x.p, N * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return done(fail(CPM_ERR_CUDA, "geodesic_nearest_run: copy-out failed"));
    return done(0);
}

extern "C" int cpm_geodesic_nearest_destroy(cpm_geodesic_nearest_t g) {
    delete g;
    return 0;
}
