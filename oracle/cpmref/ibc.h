// ORACLE — test infrastructure only. Not part of the product library.
//
// Interior boundary conditions, restated from:
//   IBCSubset                src/IBCSubset.cpp:12-268
//   IBCDOFSubset             src/IBCDOFSubset.cpp:10-227
//   IBCSubsets               src/IBCSubsets.cpp:11-116
//   Geometry (Jcp frames)    src/Geometry.cpp:27-266
//   IBCMatrixManipulations   src/IBCMatrixManipulations.cpp:12-463
// The 3x3 symmetric eigenproblem of Geometry::EigenDecomposition (Eigen's
// SelfAdjointEigenSolver in the reference) is solved by the cyclic Jacobi method
// (Golub & Van Loan, Matrix Computations, 4th ed., section 8.5); eigenvalues are
// returned ascending like Eigen's.  Eigenvector signs are arbitrary in both, and
// only sign-invariant quantities reach the solve.
#pragma once

#include <vector>

#include "tube.h"

namespace cpmref {

struct Eig3 {
    double val[3];     // ascending
    double vec[3][3];  // vec[row][col]: column c is the eigenvector of val[c]
};
Eig3 SymmetricEigen3(const double A[3][3]);

class IBCSubset {
  public:
    // normals_on_tube: eigenvector 0 of the whole-tube Jcp (computed once by
    // IBCSubsets; the reference recomputes the identical quantity per IBC).
    void ComputeSubset(const Surface &ibc, const Tube &t, const std::vector<V3> &normals_on_tube);
    size_t size() const { return m_set_from_subset.size(); }
    const std::vector<size_t> &SetIndexFromSubsetIndex() const { return m_set_from_subset; }
    const std::vector<int64_t> &SubsetIndexFromSetIndex() const { return m_subset_from_set; }
    const std::vector<V3> &cpx() const { return m_cpx_c; }
    const std::vector<V3> &cp_diff() const { return m_cp_diff; }
    const std::vector<double> &dist() const { return m_dist_c; }
    const std::vector<size_t> &bdy() const { return m_bdy; }
    const std::vector<V3> &surface_normals_on_tube() const { return m_normals_tube; }
    const std::vector<V3> &surface_normals() const { return m_normals; }
    const std::vector<V3> &tangents() const { return m_tangents; }
    const std::vector<V3> &binormals() const { return m_binormals; }
    const std::vector<V3> &directions() const { return m_directions; }
    const IBCMeta &meta() const { return m_meta; }

  private:
    IBCMeta m_meta;
    std::vector<V3> m_cpx_c, m_cp_diff, m_normals_tube, m_normals, m_tangents, m_binormals, m_directions;
    std::vector<double> m_dist_c;
    std::vector<size_t> m_bdy;
    std::vector<int64_t> m_subset_from_set;
    std::vector<size_t> m_set_from_subset;
    void ComputeSubsetNearIBC(const Surface &ibc, const Tube &t);
    void ComputeCPdiff(const Surface &ibc, const Tube &t);
    void ComputeFrameBasedDirections(const Tube &t, const std::vector<V3> &normals_on_tube);
};

class IBCDOFSubset {
  public:
    void ComputeDOFSubset(const Surface &ibc, const IBCSubset &sub, const Tube &t);
    size_t size() const { return m_set_from_subset.size(); }
    const std::vector<size_t> &SetIndexFromSubsetIndex() const { return m_set_from_subset; }
    const std::vector<int64_t> &SubsetIndexFromSetIndex() const { return m_subset_from_set; }
    const std::vector<size_t> &DirichletSetIndexFromSubsetIndex() const { return m_dir_set_from_subset; }
    const std::vector<int64_t> &DirichletSubsetIndexFromSetIndex() const { return m_dir_subset_from_set; }
    const std::vector<V3> &cpx() const { return m_cpx_c; }
    const std::vector<V3> &cpbar() const { return m_cp_bar; }
    const std::vector<V3> &cp_diff() const { return m_cp_diff; }
    const std::vector<double> &dist() const { return m_dist_c; }
    const std::vector<size_t> &bdy() const { return m_bdy; }
    const std::vector<size_t> &which_side() const { return m_which_side; }
    const std::vector<V3> &directions() const { return m_directions; }
    const SpMat &cpExtensionMatrix() const { return m_E; }
    const IBCMeta &meta() const { return m_meta; }

  private:
    IBCMeta m_meta;
    std::vector<V3> m_cp_bar, m_cpx_c, m_cp_diff, m_normals, m_tangents, m_binormals, m_directions;
    std::vector<double> m_dist_c;
    std::vector<size_t> m_bdy, m_which_side;
    std::vector<int64_t> m_subset_from_set, m_dir_subset_from_set;
    std::vector<size_t> m_set_from_subset, m_dir_set_from_subset;
    SpMat m_E;
    void OrientSubset(const Surface &ibc, const Tube &t);
};

class IBCSubsets {
  public:
    void Initialize(const Tube &t, const std::vector<SurfaceSpec> &specs);
    const IBCMeta &meta(size_t c) const { return m_dof[c].meta(); }
    size_t TotalIBCDOFs() const { return m_total; }
    size_t NumIBCs() const { return m_num; }
    size_t IBCColumnStartIndex(size_t c) const { return m_start[c]; }
    size_t DirichletIBCColumnStartIndex(size_t c) const { return m_dstart[c]; }
    size_t IdentityRowsStart() const { return m_id_start; }
    size_t Num2ndOrderDirichletRows() const { return m_num2; }
    const std::vector<IBCSubset> &TaggingSubset() const { return m_tag; }
    const std::vector<IBCDOFSubset> &DOFSubset() const { return m_dof; }
    const Surface &surface(size_t c) const { return m_surf[c]; }
    void ClosestPoint(size_t c, const V3 &x, V3 &cp, double &d, size_t &b) const { m_surf[c].ClosestPoint(x, cp, d, b); }

  private:
    size_t m_num = 0, m_total = 0, m_id_start = 0, m_num2 = 0;
    std::vector<Surface> m_surf;
    std::vector<IBCSubset> m_tag;
    std::vector<IBCDOFSubset> m_dof;
    std::vector<size_t> m_start, m_dstart;
};

// IBCMatrixManipulations (src/IBCMatrixManipulations.cpp).
// TagStencils returns one tag (1 or 2) per stored entry of A, in A's storage order
// (the reference returns a matrix with A's pattern and reads it with coeffRef).
std::vector<uint8_t> TagStencils(const SpMat &A, const Tube &t, const IBCSubsets &ibc, const std::vector<V3> &director_directions,
                                 const std::vector<int64_t> &director_subset_from_set, size_t c, double flip_scale = 1.0);
SpMat AddIBCFiniteDifference(const SpMat &L, const Tube &t, const IBCSubsets &ibc);
SpMat AddIBCExtension(const SpMat &E, const Tube &t, const IBCSubsets &ibc);
SpMat AddIBCPlotInterpolation(const SpMat &plotE, const Tube &t, const IBCSubsets &ibc);

// Geometry helpers (src/Geometry.cpp).
void EigenDecompositionOfJcp(const Tube &t, const std::vector<V3> &subset_cpx, const std::vector<size_t> &set_from_subset,
                             const std::vector<int64_t> &subset_from_set, std::vector<Eig3> &out);
void InterpolateUnorientedVectorFromNeighbours(const Tube &t, std::vector<V3> &vecs, const std::vector<size_t> &set_from_subset,
                                               const std::vector<int64_t> &subset_from_set, size_t i, double zero_tol);
std::vector<V3> InterpolateUnorientedVectors(const Tube &t, const std::vector<int64_t> &subset_from_set, size_t subset_size,
                                             const std::vector<V3> &vecs, const std::vector<V3> &xq, bool normalize = true);

// Whole-tube surface normals: eigenvector 0 of the symmetrised Jcp
// (GeodesicDistanceNearest::ComputeSurfaceNormals, problems/GeodesicDistanceNearest.cpp:311-345).
std::vector<V3> NormalsFromJcp(const Tube &t);

// Identity-row vector shared by PoissonWithIBC / GeodesicDistance (problems/PoissonWithIBC.cpp:173-191).
std::vector<bool> IBCIdentityRows(const Tube &t, const IBCSubsets &ibc);
// Row index holding the Dirichlet value of DOF i of IBC c.
size_t DirichletValueRow(const IBCSubsets &ibc, size_t c, size_t i);

}  // namespace cpmref
