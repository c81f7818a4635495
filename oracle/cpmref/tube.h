// ORACLE — test infrastructure only. Not part of the product library.
//
// Tube (computational band), Interpolation (tricubic closest-point extension)
// and FDMatrices (Laplacian, central gradients), restated from:
//   src/Grid.cpp:28-156, src/Node.h:7-24
//   src/Tube.cpp:115-157 (radius, grid sizing), :295-461 (dense BFS build),
//               :464-531 (base points), :540-605 (seed, AddTubeNode), :677-693 (neighbours)
//   src/Interpolation.cpp:8-225
//   src/FDMatrices.cpp:25-92
// Tube node order is the reference's BFS discovery order.
#pragma once

#include <cstdint>
#include <vector>

#include "sparse.h"
#include "surface.h"

namespace cpmref {

struct Grid {
    size_t dim = 3;
    double dx = 0;
    double xstart = 0;  // the reference stores one xstart per dimension, all equal
    size_t n = 0, N1d = 0, N = 0;

    // CoordinateFromTriplet (src/Grid.cpp:28-39): xstart + idx*dx.
    double Coord(size_t idx) const { return xstart + idx * dx; }
    // LinearIndexFromTriplet (src/Grid.cpp:123-144): i*N1d^2 + j*N1d + k.
    size_t Linear(size_t i, size_t j, size_t k) const { return i * N1d * N1d + j * N1d + k; }
    void Triplet(size_t index, size_t t[3]) const {
        t[2] = (index % (N1d * N1d)) % N1d;
        t[1] = ((index - t[2]) / N1d) % N1d;
        t[0] = (index - t[2] - t[1] * N1d) / (N1d * N1d);
    }
};

class Tube {
  public:
    Tube() = default;
    // Tube(SurfaceSpecifier&, p, dx) (src/Tube.cpp:46-55 -> :88-95 -> :115-157 -> :295-461)
    Tube(const SurfaceSpec &spec, size_t interp_deg, double dx);
    // Variant used by parity tests: same BFS, but the closest point of every
    // visited grid node is read from a caller-supplied function instead of the surface.
    template <class CPF>
    void BuildWith(const SurfaceSpec &spec, size_t interp_deg, double dx, CPF cpf);

    size_t dim() const { return 3; }
    size_t p() const { return m_p; }
    size_t nNodes() const { return m_num; }
    double dx() const { return m_grid.dx; }
    size_t N1d() const { return m_grid.N1d; }
    size_t n() const { return m_grid.n; }
    double xstart() const { return m_grid.xstart; }
    double TubeRadius() const { return m_radius; }
    double TubeRadiusFactor() const { return m_radius_factor; }
    const Grid &grid() const { return m_grid; }
    const Surface &surface() const { return m_surface; }

    const std::vector<V3> &x() const { return m_x; }
    const std::vector<V3> &cpx() const { return m_cpx; }
    const std::vector<double> &dist() const { return m_dist; }
    const std::vector<size_t> &bdy() const { return m_bdy; }
    const std::vector<size_t> &bpt() const { return m_bpt; }
    const std::vector<size_t> &recIndex() const { return m_rec; }
    // neighbour(i, nbr): tube index or -1, order +x,-x,+y,-y,+z,-z (src/Node.h:23)
    int64_t neighbour(int64_t i, size_t nbr) const { return i < 0 ? -1 : m_nbr[6 * (size_t)i + nbr]; }
    // TubeIndexFromRecIndex (src/Tube.h:79-103) over the dense map.
    int64_t TubeIndexFromRecIndex(size_t rec) const { return m_map[rec]; }
    // NearestTubeIndex (src/Tube.h:116-121): round((xq-xstart)/dx) per dimension.
    int64_t NearestTubeIndex(const V3 &xq) const;
    // ComputeBasePoints (src/Tube.cpp:464-483); throws like the reference.
    std::vector<size_t> ComputeBasePoints(const std::vector<V3> &xq) const;

    void ClosestPoint(const V3 &x, V3 &cp) const { m_surface.ClosestPoint(x, cp); }
    // Number of grid nodes whose closest point the BFS evaluated (tube + outer shell).
    size_t nVisited() const { return m_visited; }

  private:
    Surface m_surface;
    Grid m_grid;
    size_t m_p = 3, m_num = 0, m_visited = 0;
    double m_radius = 0, m_radius_factor = 0;
    std::vector<V3> m_x, m_cpx;
    std::vector<double> m_dist;
    std::vector<size_t> m_bdy, m_bpt, m_rec;
    std::vector<int64_t> m_nbr;
    std::vector<int64_t> m_map;

    void Setup(const SurfaceSpec &spec, size_t interp_deg, double dx);
    template <class CPF>
    void BuildTube(CPF cpf);
    void SetNeighbours();
    void BasePointTriplet(const V3 &xq, size_t t[3]) const;
};

// Interpolation (src/Interpolation.cpp:8-225).
class Interpolation {
  public:
    explicit Interpolation(const Tube &t);                          // query points = tube cps
    Interpolation(const Tube &t, const std::vector<V3> &xquery);    // arbitrary query points
    void BuildInterpolationMatrix(const Tube &t, SpMat &E) const;
    void BuildInterpolationMatrix(const Tube &t, const std::vector<int64_t> &subset_idx_from_set_idx, SpMat &E) const;
    // w[d][q][j]
    const std::vector<std::vector<std::vector<double>>> &weights() const { return m_w; }
    const std::vector<size_t> &basePoints() const { return m_bpt; }

  private:
    size_t m_Nq = 0;
    int m_stencil = 4;
    std::vector<V3> m_xq;
    std::vector<size_t> m_bpt;
    std::vector<double> m_uniform;
    std::vector<std::vector<std::vector<double>>> m_w;
    void UniformGridWeights1D();
    void Weights1D(const double *x, double xq, double *w) const;
    void BuildWeights(const Tube &t);
};

// FDMatrices (src/FDMatrices.cpp:11-92).
void BuildLaplacianMatrix(const Tube &t, SpMat &L);
void BuildLaplacianMatrix(const Tube &t, const std::vector<size_t> &set_from_subset, const std::vector<int64_t> &subset_from_set, SpMat &L);
void BuildGradientMatrices(const Tube &t, std::vector<SpMat> &Dc);
void BuildGradientMatrices(const Tube &t, const std::vector<size_t> &set_from_subset, const std::vector<int64_t> &subset_from_set, std::vector<SpMat> &Dc);

// Helpers::SetupMatrices (src/Helpers.cpp:86-93) and GetPlotInterpMatrix (:97-103).
void SetupMatrices(const Tube &t, SpMat &E, SpMat &L);
void GetPlotInterpMatrix(const Tube &t, SpMat &plotE);

}  // namespace cpmref

#include "tube_impl.h"
