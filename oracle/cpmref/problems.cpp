// ORACLE — test infrastructure only. Not part of the product library.
#include "problems.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <stdexcept>

namespace cpmref {

Problem::Problem(const SurfaceSpec &surface, const std::vector<SurfaceSpec> &ibcs, size_t p, double dx) : tube(surface, p, dx) {
    Assemble(ibcs);
}

void Problem::Assemble(const std::vector<SurfaceSpec> &ibcs) {
    SetupMatrices(tube, E, L);
    const size_t N = tube.nNodes();
    if (ibcs.empty()) {
        // Poisson::Initialize without boundaries (problems/Poisson.cpp:229-236).
        has_ibc = false;
        Lfull = L;
        Efull = E;
        identity_rows.assign(N, false);
        row_kind.assign(N, ROW_TUBE);
        row_ibc.assign(N, -1);
        row_point = tube.cpx();
        return;
    }
    has_ibc = true;
    ibc.Initialize(tube, ibcs);
    // PoissonWithIBC::Initialize (problems/PoissonWithIBC.cpp:162-192).
    Lfull = AddIBCFiniteDifference(L, tube, ibc);
    Efull = AddIBCExtension(E, tube, ibc);
    identity_rows = IBCIdentityRows(tube, ibc);
    size_t Dn = Lfull.rows;
    row_kind.assign(Dn, ROW_OTHER);
    row_ibc.assign(Dn, -1);
    row_point.assign(Dn, V3{0, 0, 0});
    for (size_t i = 0; i < N; ++i) {
        row_kind[i] = ROW_TUBE;
        row_point[i] = tube.cpx()[i];
    }
    // PoissonWithIBC::GetRHS (problems/PoissonWithIBC.cpp:92-133).
    for (size_t c = 0; c < ibc.NumIBCs(); ++c)
        for (size_t i = 0; i < ibc.DOFSubset()[c].size(); ++i) {
            const IBCMeta &mc = ibc.meta(c);
            size_t bc = mc.is_oriented ? ibc.DOFSubset()[c].which_side()[i] - 1 : 0;
            if (mc.boundary_type[bc] == 1 || (mc.boundary_type[bc] == 0 && mc.boundary_order == 2)) {
                size_t r = i + ibc.IBCColumnStartIndex(c);
                row_kind[r] = ROW_IBC_F;
                row_ibc[r] = (int)c;
                row_point[r] = ibc.DOFSubset()[c].cpx()[i];
            }
        }
    for (size_t c = 0; c < ibc.NumIBCs(); ++c)
        for (size_t i = 0; i < ibc.DOFSubset()[c].size(); ++i) {
            const IBCMeta &mc = ibc.meta(c);
            size_t bc = mc.is_oriented ? ibc.DOFSubset()[c].which_side()[i] - 1 : 0;
            if (mc.boundary_type[bc] == 0) {
                size_t r = DirichletValueRow(ibc, c, i);
                row_kind[r] = ROW_DIRICHLET;
                row_ibc[r] = (int)c;
                row_point[r] = ibc.DOFSubset()[c].cpx()[i];
            }
        }
}

SpMat Problem::PlotMatrix() const {
    SpMat plotE;
    GetPlotInterpMatrix(tube, plotE);
    if (!has_ibc) return plotE;
    return AddIBCPlotInterpolation(plotE, tube, ibc);
}

// GeodesicDistance::ComputeDistance (problems/GeodesicDistance.cpp:11-69) with
// Step1 (:75-173), Step2 (:179-311), ComputeDivergence (:317-327), Step3 (:330-413).
std::vector<double> Problem::GeodesicDistance(double dt, int step1_jacobi_iters, std::vector<int> *iters) const {
    const size_t N = tube.nNodes();
    const size_t Dn = Lfull.rows;
    // Step 1: heat flow from the IBC.
    double extent = tube.TubeRadius();
    double tol = tube.dx();
    double scale = std::atanh(1 - tol) / extent;
    auto SmoothH = [scale](double t) { return 0.5 * std::tanh(-scale * t) + 0.5; };
    std::vector<double> rhs(Dn, 0.0);
    for (size_t c = 0; c < ibc.NumIBCs(); ++c)
        for (size_t i = 0; i < ibc.DOFSubset()[c].size(); ++i) {
            const IBCMeta &mc = ibc.meta(c);
            size_t bc = mc.is_oriented ? ibc.DOFSubset()[c].which_side()[i] - 1 : 0;
            if (mc.boundary_type[bc] == 0) rhs[DirichletValueRow(ibc, c, i)] = SmoothH(-Norm(ibc.DOFSubset()[c].cp_diff()[i]));
        }
    for (size_t c = 0; c < ibc.NumIBCs(); ++c)
        for (size_t i = 0; i < ibc.DOFSubset()[c].size(); ++i)
            rhs[ibc.DOFSubset()[c].SetIndexFromSubsetIndex()[i]] = SmoothH(Norm(ibc.DOFSubset()[c].cp_diff()[i]));
    Solver sv1;
    if (step1_jacobi_iters > 0) {
        sv1.Init(1.0, -dt, Lfull, Efull, Preconditioner::jacobi, identity_rows);
        sv1.SetPrecond(step1_jacobi_iters);
    } else {
        sv1.Init(1.0, -dt, Lfull, Efull, Preconditioner::diagonal, identity_rows);
    }
    std::vector<double> ufull = sv1.Solve(rhs);
    if (iters) iters->push_back(sv1.stats().iterations);
    std::vector<double> u(N);
    for (size_t i = 0; i < N; ++i) u[i] = -ufull[i];

    std::vector<SpMat> Dc;
    BuildGradientMatrices(tube, Dc);
    const std::vector<V3> &normals = ibc.TaggingSubset()[0].surface_normals_on_tube();

    auto step2_div = [&](const std::vector<double> &uu) {
        std::vector<double> g[3], tmp;
        for (int d = 0; d < 3; ++d) {
            Dc[d].Multiply(uu, tmp);
            E.Multiply(tmp, g[d]);
        }
        for (size_t i = 0; i < normals.size(); ++i) {
            V3 gr{g[0][i], g[1][i], g[2][i]};
            gr = Sub(gr, Scale(Dot(gr, normals[i]), normals[i]));
            for (int d = 0; d < 3; ++d) g[d][i] = gr[d];
        }
        for (size_t i = 0; i < N; ++i) {
            double gn = 0.0;
            for (int d = 0; d < 3; ++d) gn += g[d][i] * g[d][i];
            gn = std::sqrt(gn);
            if (gn != 0.0)
                for (int d = 0; d < 3; ++d) g[d][i] /= gn;
        }
        std::vector<double> div(N, 0.0);
        for (int d = 0; d < 3; ++d) {
            Dc[d].Multiply(g[d], tmp);
            for (size_t i = 0; i < N; ++i) div[i] = div[i] + tmp[i];
        }
        return div;
    };
    auto step3 = [&](const std::vector<double> &div) {
        std::vector<double> divfull(Dn, 0.0);
        for (size_t i = 0; i < N; ++i) divfull[i] = div[i];
        Solver sv;
        sv.Init(0.0, 1.0, Lfull, Efull, Preconditioner::diagonal, identity_rows);
        std::vector<double> phi = sv.Solve(divfull);
        if (iters) iters->push_back(sv.stats().iterations);
        double mn = std::numeric_limits<double>::max();
        for (double v : phi) mn = std::min(mn, v);
        for (double &v : phi) v -= mn;
        return phi;
    };
    std::vector<double> phi = step3(step2_div(u));
    for (int k = 0; k < 2; ++k) {
        for (size_t i = 0; i < N; ++i) u[i] = phi[i];
        std::vector<double> eu;
        E.Multiply(u, eu);
        phi = step3(step2_div(eu));
    }
    return phi;
}

// Dense LU with partial pivoting, then forward and back substitution: the exact
// solve that stands in for Eigen::SparseLU (problems/GeodesicDistanceNearest.cpp:123-133).
static std::vector<double> DenseSolve(const SpMat &A, const std::vector<double> &b) {
    const size_t n = A.rows;
    if (n > 8000) throw std::runtime_error("oracle: dense heat solve is for small tubes only");
    std::vector<double> a(n * n, 0.0), x(b);
    for (size_t i = 0; i < n; ++i)
        for (size_t e = A.ptr[i]; e < A.ptr[i + 1]; ++e) a[i * n + A.idx[e]] = A.val[e];
    for (size_t k = 0; k < n; ++k) {
        size_t piv = k;
        for (size_t i = k + 1; i < n; ++i)
            if (std::abs(a[i * n + k]) > std::abs(a[piv * n + k])) piv = i;
        if (a[piv * n + k] == 0.0) throw std::runtime_error("oracle: singular heat matrix");
        if (piv != k) {
            for (size_t j = 0; j < n; ++j) std::swap(a[k * n + j], a[piv * n + j]);
            std::swap(x[k], x[piv]);
        }
        const double d = a[k * n + k];
#pragma omp parallel for schedule(static)
        for (long long ii = (long long)k + 1; ii < (long long)n; ++ii) {
            double *ri = &a[(size_t)ii * n];
            const double l = ri[k] / d;
            if (l == 0.0) continue;
            ri[k] = l;
            const double *rk = &a[k * n];
            for (size_t j = k + 1; j < n; ++j) ri[j] -= l * rk[j];
        }
        for (size_t i = k + 1; i < n; ++i) x[i] -= a[i * n + k] * x[k];
    }
    for (size_t kk = n; kk-- > 0;) {
        double s = x[kk];
        for (size_t j = kk + 1; j < n; ++j) s -= a[kk * n + j] * x[j];
        x[kk] = s / a[kk * n + kk];
    }
    return x;
}

// GeodesicDistanceNearest::Step1 (problems/GeodesicDistanceNearest.cpp:60-133): the smoothed
// sources and the solve of the transposed implicit-Euler matrix with identity rows.
std::vector<double> Problem::HeatNearest(const std::vector<size_t> &ibc_idx, const std::vector<size_t> &inside_idx,
                                         const std::vector<double> &inside_dist, double dt, int step1_jacobi_iters,
                                         int *iters) const {
    if (has_ibc) throw std::runtime_error("oracle: GeodesicDistanceNearest runs on a problem without IBCs");
    const size_t N = tube.nNodes();
    std::vector<bool> ident(N, false);
    for (size_t i : ibc_idx) ident[i] = true;
    // Step 1: smoothed heat sources (:62-90)
    const double extent = tube.TubeRadius(), tol = tube.dx();
    const double scale = std::atanh(1 - tol) / extent;
    auto SmoothH = [scale](double t) { return 0.5 * std::tanh(-scale * t) + 0.5; };
    std::vector<double> rhs(N, 0.0);
    for (size_t i : ibc_idx) rhs[i] = SmoothH(-Distance(tube.x()[i], tube.cpx()[i]));
    for (size_t i = 0; i < inside_idx.size(); ++i) rhs[inside_idx[i]] = SmoothH(-inside_dist[i]);
    // Afull = I - dt (diag(L) + (L - diag(L)) E) (Helpers::ImplicitEulerMatrix, src/Helpers.cpp:292-299;
    // LaplacianSharp :107-115), transposed, identity rows set (:92-121)
    std::vector<Triplet> tr;
    std::vector<double> acc(N, 0.0);
    std::vector<char> seen(N, 0);
    std::vector<size_t> touched;
    for (size_t q = 0; q < N; ++q) {
        touched.clear();
        double lqq = 0.0;
        for (size_t e = L.ptr[q]; e < L.ptr[q + 1]; ++e) {
            const size_t c = L.idx[e];
            if (c == q) {
                lqq = L.val[e];
                continue;
            }
            for (size_t f = E.ptr[c]; f < E.ptr[c + 1]; ++f) {
                const size_t k = E.idx[f];
                if (!seen[k]) {
                    seen[k] = 1;
                    touched.push_back(k);
                }
                acc[k] += L.val[e] * E.val[f];
            }
        }
        if (!seen[q]) {
            seen[q] = 1;
            touched.push_back(q);
        }
        acc[q] += lqq;
        for (size_t k : touched) {
            const double a = (k == q ? 1.0 : 0.0) - dt * acc[k];
            tr.push_back({k, q, a});  // transposed: Ar(k, q) = Afull(q, k)
            acc[k] = 0.0;
            seen[k] = 0;
        }
    }
    std::vector<Triplet> tr2;
    tr2.reserve(tr.size());
    for (const auto &t : tr)
        if (!ident[t.row]) tr2.push_back(t);
    for (size_t k = 0; k < N; ++k)
        if (ident[k]) tr2.push_back({k, k, 1.0});
    SpMat Ar;
    Ar.FromTriplets(N, N, tr2);
    std::vector<double> u;
    if (step1_jacobi_iters <= 0) {
        u = DenseSolve(Ar, rhs);
        if (iters) *iters = 0;
    } else {
        // the device's substitute for the direct solve: BiCGStab preconditioned by damped
        // Jacobi sweeps with the reference's matrix-free diagonal m + n L_kk = 1 - dt L_kk
        // (src/GeneralizedBiCGStabSystem.h:281-385)
        std::vector<double> diag(N);
        for (size_t k = 0; k < N; ++k) diag[k] = ident[k] ? 1.0 : 1.0 + L.Coeff(k, k) * (-dt);
        auto mul = [&](const std::vector<double> &a, std::vector<double> &o) { Ar.Multiply(a, o); };
        auto prec = [&](const std::vector<double> &in, std::vector<double> &out) {
            out.assign(N, 0.0);
            std::vector<double> tmp, res(N);
            const double omega = 2.0 / 3.0;
            for (int it = 0; it < step1_jacobi_iters; ++it) {
                Ar.Multiply(out, tmp);
                for (size_t q = 0; q < N; ++q) res[q] = (in[q] - tmp[q]) / diag[q];
                for (size_t q = 0; q < N; ++q) out[q] += omega * res[q];
            }
        };
        u.assign(N, 0.0);
        SolveStats st = BiCGStabSolveOp(mul, prec, u, rhs, 1e-10, 100000);
        if (iters) *iters = st.iterations;
    }
    return u;
}

// GeodesicDistanceNearest::ComputeDistance (problems/GeodesicDistanceNearest.cpp:11-53) with
// Step1 (:60-147), Step2 (:154-236), ComputeDivergence (:298-308), Step3 (:244-293).
std::vector<double> Problem::GeodesicDistanceNearest(const std::vector<size_t> &ibc_idx, const std::vector<size_t> &inside_idx,
                                                     const std::vector<double> &inside_dist, double dt,
                                                     int step1_jacobi_iters, std::vector<int> *iters) const {
    const size_t N = tube.nNodes();
    std::vector<bool> ident(N, false);
    for (size_t i : ibc_idx) ident[i] = true;
    int heat_iters = 0;
    std::vector<double> u = HeatNearest(ibc_idx, inside_idx, inside_dist, dt, step1_jacobi_iters, &heat_iters);
    if (iters) iters->push_back(heat_iters);
    std::vector<double> eu;
    E.Multiply(u, eu);  // u = m_E * u (:136)
    for (size_t i = 0; i < N; ++i) u[i] = -eu[i];  // u = -Step1 (:25)

    std::vector<SpMat> Dc;
    BuildGradientMatrices(tube, Dc);
    const std::vector<V3> normals = NormalsFromJcp(tube);
    auto step2_div = [&](const std::vector<double> &uu) {
        std::vector<double> g[3], tmp;
        for (int d = 0; d < 3; ++d) {
            Dc[d].Multiply(uu, tmp);
            E.Multiply(tmp, g[d]);
        }
        for (size_t i = 0; i < N; ++i) {
            V3 gr{g[0][i], g[1][i], g[2][i]};
            gr = Sub(gr, Scale(Dot(gr, normals[i]), normals[i]));
            double gn = 0.0;
            for (int d = 0; d < 3; ++d) gn += gr[d] * gr[d];
            gn = std::sqrt(gn);
            for (int d = 0; d < 3; ++d) g[d][i] = gn != 0.0 ? gr[d] / gn : gr[d];
        }
        std::vector<double> div(N, 0.0);
        for (int d = 0; d < 3; ++d) {
            Dc[d].Multiply(g[d], tmp);
            for (size_t i = 0; i < N; ++i) div[i] = div[i] + tmp[i];
        }
        return div;
    };
    auto step3 = [&](std::vector<double> div) {
        for (size_t i : ibc_idx) div[i] = 0.0;
        Solver sv;
        sv.Init(0.0, 1.0, L, E, Preconditioner::diagonal, ident);
        std::vector<double> phi = sv.Solve(div);
        if (iters) iters->push_back(sv.stats().iterations);
        double mn = std::numeric_limits<double>::max();
        for (double v : phi) mn = std::min(mn, v);
        for (double &v : phi) v -= mn;
        return phi;
    };
    std::vector<double> phi = step3(step2_div(u));
    for (int k = 0; k < 2; ++k) {
        E.Multiply(phi, eu);
        phi = step3(step2_div(eu));
    }
    return phi;
}

}  // namespace cpmref
