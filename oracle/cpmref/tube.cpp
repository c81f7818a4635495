// ORACLE — test infrastructure only. Not part of the product library.
#include "tube.h"

#include <cmath>
#include <stdexcept>

namespace cpmref {

Tube::Tube(const SurfaceSpec &spec, size_t interp_deg, double dx) {
    Setup(spec, interp_deg, dx);
    const Surface &s = m_surface;
    BuildTube([&s](size_t, const V3 &x, V3 &cp, double &dist, size_t &bdy) { s.ClosestPoint(x, cp, dist, bdy); });
}

// Tube::ConstructTube + ComputeTubeRadius + grid sizing (src/Tube.cpp:115-157).
void Tube::Setup(const SurfaceSpec &spec, size_t interp_deg, double dx) {
    m_surface = Surface(spec);
    m_p = interp_deg;
    m_grid.dim = 3;
    m_grid.dx = dx;
    const size_t order = 2;
    m_radius_factor = 1.0001 * std::sqrt((m_grid.dim - 1) * std::pow(0.5 * (m_p + 1), 2) + std::pow(0.5 * (order + m_p + 1), 2));
    m_radius = m_radius_factor * dx;

    const size_t pad = 5;
    const double *bb = m_surface.bbox();
    size_t spacings = (size_t)std::ceil((bb[1] - bb[0]) / dx);
    size_t n = (size_t)std::ceil(std::log2((double)(spacings + 2 * pad)));
    size_t diff = (size_t)std::ceil(0.5 * (std::pow(2, n) - spacings - 2 * pad));
    m_grid.xstart = bb[0] - (pad + diff) * dx;
    m_grid.n = n;
    m_grid.N1d = (size_t)(std::pow(2.0, n) + 1);
    m_grid.N = (size_t)std::pow((double)m_grid.N1d, 3);
}

// Tube::SetNeighbours (src/Tube.cpp:677-693).
void Tube::SetNeighbours() {
    m_nbr.assign(6 * m_num, -1);
    for (size_t i = 0; i < m_num; ++i) {
        size_t t[3];
        m_grid.Triplet(m_rec[i], t);
        for (int d = 0; d < 3; ++d)
            for (int si = 0; si < 2; ++si) {
                size_t nt[3] = {t[0], t[1], t[2]};
                nt[d] += (si == 0) ? 1 : (size_t)-1;
                int64_t m = m_map[m_grid.Linear(nt[0], nt[1], nt[2])];
                if (m >= 0 && (size_t)m < m_num) m_nbr[6 * i + 2 * d + si] = m;
            }
    }
}

// InterpBasePointTriplet (src/Tube.cpp:502-531): floor for odd p, round for even p,
// then shift by p/2 (even) or (p-1)/2 (odd) towards -1.
void Tube::BasePointTriplet(const V3 &xq, size_t t[3]) const {
    for (int d = 0; d < 3; ++d) {
        if (m_p % 2 == 0)
            t[d] = (size_t)std::round((xq[d] - m_grid.xstart) / m_grid.dx);
        else
            t[d] = (size_t)std::floor((xq[d] - m_grid.xstart) / m_grid.dx);
    }
    size_t shifts = (m_p % 2 == 0) ? m_p / 2 : (m_p - 1) / 2;
    for (int d = 0; d < 3; ++d) t[d] -= shifts;
}

std::vector<size_t> Tube::ComputeBasePoints(const std::vector<V3> &xq) const {
    std::vector<size_t> out(xq.size());
    for (size_t i = 0; i < xq.size(); ++i) {
        size_t t[3];
        BasePointTriplet(xq[i], t);
        for (int d = 0; d < 3; ++d)
            if (t[d] >= m_grid.N1d)
                throw std::runtime_error("Tube::ComputeBasePoints - Interpolation base point is not within the tube.");
        int64_t m = m_map[m_grid.Linear(t[0], t[1], t[2])];
        if (m < 0 || (size_t)m >= m_num)
            throw std::runtime_error("Tube::ComputeBasePoints - Interpolation base point is not within the tube.");
        out[i] = (size_t)m;
    }
    return out;
}

int64_t Tube::NearestTubeIndex(const V3 &xq) const {
    size_t t[3];
    for (int d = 0; d < 3; ++d) t[d] = (size_t)std::round((xq[d] - m_grid.xstart) / m_grid.dx);
    return m_map[m_grid.Linear(t[0], t[1], t[2])];
}

// ---------------------------------------------------------------------------
// Interpolation (src/Interpolation.cpp:8-225)

Interpolation::Interpolation(const Tube &t) {
    m_xq = t.cpx();
    m_Nq = t.nNodes();
    m_bpt = t.bpt();
    m_stencil = (int)t.p() + 1;
    UniformGridWeights1D();
    BuildWeights(t);
}

Interpolation::Interpolation(const Tube &t, const std::vector<V3> &xquery) {
    m_xq = xquery;
    m_Nq = m_xq.size();
    m_bpt = t.ComputeBasePoints(m_xq);
    m_stencil = (int)t.p() + 1;
    UniformGridWeights1D();
    BuildWeights(t);
}

// UniformGridWeights1D (src/Interpolation.cpp:128-159): signed binomials.
void Interpolation::UniformGridWeights1D() {
    static const double tab[6][5] = {{1}, {1, -1}, {1, -2, 1}, {1, -3, 3, -1}, {1, -4, 6, -4, 1}};
    m_uniform.assign(tab[m_stencil - 1], tab[m_stencil - 1] + m_stencil);
}

// BuildInterpolationWeights1D (src/Interpolation.cpp:162-200): barycentric
// Lagrange weights; an exact node (|xq - x_j| < 1e-17) gets weight 1.
void Interpolation::Weights1D(const double *x, double xq, double *w) const {
    bool exact = false;
    int ip = 0;
    for (int j = 0; j < m_stencil; ++j)
        if (std::abs(xq - x[j]) < 1e-17) {
            exact = true;
            ip = j;
        }
    if (exact) {
        for (int j = 0; j < m_stencil; ++j) w[j] = 0.0;
        w[ip] = 1.0;
    } else {
        double sum = 0.0;
        for (int j = 0; j < m_stencil; ++j) {
            w[j] = m_uniform[j] / (xq - x[j]);
            sum += w[j];
        }
        for (int j = 0; j < m_stencil; ++j) w[j] /= sum;
    }
}

// BuildInterpolationWeights (src/Interpolation.cpp:204-225): stencil coordinates
// are read by walking +d neighbours from the base point.
void Interpolation::BuildWeights(const Tube &t) {
    m_w.assign(3, std::vector<std::vector<double>>(m_Nq, std::vector<double>(m_stencil)));
    std::vector<double> x(m_stencil);
    for (int d = 0; d < 3; ++d) {
        for (size_t q = 0; q < m_Nq; ++q) {
            int64_t index = (int64_t)m_bpt[q];
            x[0] = t.x()[m_bpt[q]][d];
            for (int i = 1; i < m_stencil; ++i) {
                int64_t nb = t.neighbour(index, 2 * d);
                if (nb < 0) throw std::runtime_error("Interpolation: stencil leaves the tube");
                x[i] = t.x()[nb][d];
                index = nb;
            }
            Weights1D(x.data(), m_xq[q][d], m_w[d][q].data());
        }
    }
}

void Interpolation::BuildInterpolationMatrix(const Tube &t, SpMat &E) const {
    std::vector<int64_t> ident(t.nNodes());
    for (size_t i = 0; i < t.nNodes(); ++i) ident[i] = (int64_t)i;
    BuildInterpolationMatrix(t, ident, E);
}

// BuildInterpolationMatrix, 3-D branch (src/Interpolation.cpp:52-121): row q has
// entries at base+(i,j,k) walked +x outer, +y, +z inner, valued w2[k]*w1[j]*w0[i].
void Interpolation::BuildInterpolationMatrix(const Tube &t, const std::vector<int64_t> &subset_idx_from_set_idx, SpMat &E) const {
    std::vector<Triplet> coeffs;
    coeffs.reserve(m_Nq * (size_t)m_stencil * m_stencil * m_stencil);
    for (size_t q = 0; q < m_Nq; ++q) {
        int64_t xindex = (int64_t)m_bpt[q], yindex = xindex, zindex = xindex;
        for (int i = 0; i < m_stencil; ++i) {
            for (int j = 0; j < m_stencil; ++j) {
                for (int k = 0; k < m_stencil; ++k) {
                    if (zindex < 0) throw std::runtime_error("Interpolation: stencil leaves the tube");
                    int64_t sub = subset_idx_from_set_idx[zindex];
                    if (sub >= 0) coeffs.push_back({q, (size_t)sub, m_w[2][q][k] * m_w[1][q][j] * m_w[0][q][i]});
                    zindex = t.neighbour(zindex, 4);
                }
                zindex = t.neighbour(yindex, 2);
                yindex = zindex;
            }
            zindex = t.neighbour(xindex, 0);
            yindex = zindex;
            xindex = zindex;
        }
    }
    size_t cols = 0;
    for (int64_t v : subset_idx_from_set_idx)
        if (v >= 0) cols = std::max(cols, (size_t)v + 1);
    if (E.cols > cols) cols = E.cols;
    E.FromTriplets(m_Nq, cols, coeffs);
}

// ---------------------------------------------------------------------------
// FDMatrices (src/FDMatrices.cpp:11-92)

void BuildLaplacianMatrix(const Tube &t, SpMat &L) {
    std::vector<size_t> s2(t.nNodes());
    std::vector<int64_t> s1(t.nNodes());
    for (size_t i = 0; i < t.nNodes(); ++i) {
        s1[i] = (int64_t)i;
        s2[i] = i;
    }
    BuildLaplacianMatrix(t, s2, s1, L);
}

// Diagonal -2*dim, each existing in-subset neighbour +1, then L /= dx*dx.
void BuildLaplacianMatrix(const Tube &t, const std::vector<size_t> &set_from_subset, const std::vector<int64_t> &subset_from_set, SpMat &L) {
    std::vector<Triplet> c;
    c.reserve(set_from_subset.size() * 7);
    for (size_t row = 0; row < set_from_subset.size(); ++row) {
        c.push_back({row, row, -2.0 * (double)t.dim()});
        size_t s = set_from_subset[row];
        for (size_t nbr = 0; nbr < 2 * t.dim(); ++nbr) {
            int64_t ni = t.neighbour(s, nbr);
            if (ni >= 0) {
                int64_t sub = subset_from_set[ni];
                if (sub >= 0) c.push_back({row, (size_t)sub, 1.0});
            }
        }
    }
    L.FromTriplets(set_from_subset.size(), set_from_subset.size(), c);
    L.Scale(t.dx() * t.dx());
}

void BuildGradientMatrices(const Tube &t, std::vector<SpMat> &Dc) {
    std::vector<size_t> s2(t.nNodes());
    std::vector<int64_t> s1(t.nNodes());
    for (size_t i = 0; i < t.nNodes(); ++i) {
        s1[i] = (int64_t)i;
        s2[i] = i;
    }
    BuildGradientMatrices(t, s2, s1, Dc);
}

// Central differences: +/-0.5 at the +/-e_d neighbours (sign pow(-1, nbr)), then /= dx.
void BuildGradientMatrices(const Tube &t, const std::vector<size_t> &set_from_subset, const std::vector<int64_t> &subset_from_set, std::vector<SpMat> &Dc) {
    std::vector<std::vector<Triplet>> c(3);
    for (size_t row = 0; row < set_from_subset.size(); ++row) {
        size_t s = set_from_subset[row];
        for (size_t nbr = 0; nbr < 6; ++nbr) {
            int64_t ni = t.neighbour(s, nbr);
            if (ni >= 0) {
                int64_t sub = subset_from_set[ni];
                if (sub >= 0) c[nbr / 2].push_back({row, (size_t)sub, ((nbr % 2) ? -1.0 : 1.0) * 0.5});
            }
        }
    }
    Dc.resize(3);
    for (int d = 0; d < 3; ++d) {
        Dc[d].FromTriplets(set_from_subset.size(), set_from_subset.size(), c[d]);
        Dc[d].Scale(t.dx());
    }
}

void SetupMatrices(const Tube &t, SpMat &E, SpMat &L) {
    BuildLaplacianMatrix(t, L);
    Interpolation interp(t);
    E.Resize(t.nNodes(), t.nNodes());
    interp.BuildInterpolationMatrix(t, E);
}

void GetPlotInterpMatrix(const Tube &t, SpMat &plotE) {
    plotE.Resize(t.surface().xp().size(), t.nNodes());
    Interpolation pi(t, t.surface().xp());
    pi.BuildInterpolationMatrix(t, plotE);
}

}  // namespace cpmref
