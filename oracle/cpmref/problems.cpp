// ORACLE — test infrastructure only. Not part of the product library.
#include "problems.h"

#include <cmath>
#include <limits>

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

}  // namespace cpmref
