// ORACLE — test infrastructure only. Not part of the product library.
//
// Problem assembly restated from the reference's problems/:
//   Poisson (no boundary)   problems/Poisson.cpp:12-18, 164-238 (bdy_order 0 branch)
//   PoissonWithIBC          problems/PoissonWithIBC.cpp:8-47, 50-133, 162-192
//   HeatWithIBC             problems/HeatWithIBC.cpp:50-103, 135-169
//   GeodesicDistance        problems/GeodesicDistance.cpp:11-413
//   GeodesicDistanceNearest problems/GeodesicDistanceNearest.cpp:11-345
#pragma once

#include <functional>
#include <memory>
#include <vector>

#include "ibc.h"
#include "solver.h"

namespace cpmref {

// Row kinds of the assembled system, used to build right-hand sides:
//   0 tube row (f at the tube closest point)
//   1 IBC DOF row whose right-hand side is f at the DOF's IBC closest point
//     (2nd-order Dirichlet or Neumann, problems/PoissonWithIBC.cpp:99-108)
//   2 Dirichlet value row (identity row carrying the IBC value)
enum RowKind { ROW_TUBE = 0, ROW_IBC_F = 1, ROW_DIRICHLET = 2, ROW_OTHER = 3 };

class Problem {
  public:
    Problem(const SurfaceSpec &surface, const std::vector<SurfaceSpec> &ibcs, size_t p, double dx);
    // Tube from caller-supplied closest points (parity tests: "given the same closest points").
    template <class CPF>
    Problem(const SurfaceSpec &surface, size_t p, double dx, CPF cpf, bool) {
        tube.BuildWith(surface, p, dx, cpf);
        Assemble({});
    }

    Tube tube;
    IBCSubsets ibc;
    bool has_ibc = false;
    SpMat L, E, Lfull, Efull;
    std::vector<bool> identity_rows;
    std::vector<int> row_kind;     // RowKind per system row
    std::vector<int> row_ibc;      // IBC index for kinds 1, 2 (else -1)
    std::vector<V3> row_point;     // evaluation point per row
    size_t D() const { return Lfull.rows; }

    // plot interpolation (with IBC columns when IBCs are present)
    SpMat PlotMatrix() const;

    // GeodesicDistance::ComputeDistance; returns phi on the system rows (not plotted).
    // step1_jacobi_iters = 0 selects the diagonal preconditioner for the heat solve.
    std::vector<double> GeodesicDistance(double dt, int step1_jacobi_iters, std::vector<int> *iters = nullptr) const;

    // GeodesicDistanceNearest::ComputeDistance (problems/GeodesicDistanceNearest.cpp:11-53) on a
    // problem without IBCs: identity rows at ibc_idx (the constraint rows of every curve, in
    // order), smoothed heat sources at inside_idx with distances inside_dist.  Returns phi on
    // the tube rows (the reference returns plotE * phi).  The heat step solves the transposed
    // implicit-Euler matrix (:103-133); step1_jacobi_iters = 0 solves it directly (dense LU with
    // partial pivoting, standing in for the reference's SparseLU, small tubes only), > 0 by
    // BiCGStab with that many damped Jacobi sweeps per preconditioner call.
    std::vector<double> GeodesicDistanceNearest(const std::vector<size_t> &ibc_idx, const std::vector<size_t> &inside_idx,
                                                const std::vector<double> &inside_dist, double dt, int step1_jacobi_iters,
                                                std::vector<int> *iters = nullptr) const;
    // Its heat step alone (:60-133): the solution of the transposed implicit-Euler system, before
    // the extension u = E u (:136).
    std::vector<double> HeatNearest(const std::vector<size_t> &ibc_idx, const std::vector<size_t> &inside_idx,
                                    const std::vector<double> &inside_dist, double dt, int step1_jacobi_iters,
                                    int *iters = nullptr) const;

    // (Re)assemble L, E and, with IBCs, the rewritten Lfull/Efull on the current tube.
    void Assemble(const std::vector<SurfaceSpec> &ibcs);
};

}  // namespace cpmref
