// ORACLE — test infrastructure only. Not part of the product library.
//
// The reference's custom ("partially matrix-free") BiCGStab solve path:
//   GeneralizedBiCGStabSystem   src/GeneralizedBiCGStabSystem.h:37-385
//   BiCGStab::Solve             src/BiCGStab.h:30-108
//   BiCGStabVector ops          src/BiCGStabVector.h:23-72 (OpenMP-parallel, as in the reference)
//   Solver Init/Solve/Multiply  src/Solver.cpp:8-138
// The sparse products run serially (the reference's OPENMP macro is never
// defined; tests may put their rows on OpenMP threads, ParallelRows() in
// sparse.h, which changes no result); vector updates run OpenMP-parallel; dot products are serial sums
// (the reference uses Eigen's dot, whose vectorised summation order is not
// pinned by any version in the reference tree).
#pragma once

#include <functional>
#include <vector>

#include "sparse.h"

namespace cpmref {

enum class Preconditioner { identity = 0, diagonal = 1, jacobi = 2 };

class GeneralizedSystem {
  public:
    double m = 0, n = 0;
    Preconditioner precond = Preconditioner::diagonal;
    SpMat L, E;
    int precond_iters = 0;
    int nD = 0;
    size_t dofs = 0;
    std::vector<bool> identity_rows;

    void SetComponents(double m_in, double n_in, const SpMat &L_in, const SpMat &E_in, Preconditioner p,
                       const std::vector<bool> &identity_rows_in, int nD_in = 0);
    // Multiply (src/GeneralizedBiCGStabSystem.h:191-233)
    void Multiply(const std::vector<double> &x, std::vector<double> &result) const { Multiply(x, result, m, n); }
    void Multiply(const std::vector<double> &x, std::vector<double> &result, double m_in, double n_in) const;
    // Interpolation step of Multiply: t = E~ x (identity rows copy x) (:235-261)
    void Interp(const std::vector<double> &x, std::vector<double> &t) const;
    void Precondition(const std::vector<double> &x, std::vector<double> &result) const;
    void DiagonalInverse(const std::vector<double> &in, std::vector<double> &out) const;
};

struct SolveStats {
    int iterations = 0;
    int restarts = 0;
    double final_rel_residual2 = 0;  // ||r||^2 / ||b||^2 on the recursive residual
    bool converged = false;
};

// BiCGStab::Solve (src/BiCGStab.h:30-108) over any operator and preconditioner
// (the algorithm is a template over the system in the reference).
using LinOp = std::function<void(const std::vector<double> &, std::vector<double> &)>;
SolveStats BiCGStabSolveOp(const LinOp &multiply, const LinOp &precondition, std::vector<double> &x,
                           const std::vector<double> &b, double tolerance, int max_iterations);

// BiCGStab::Solve (src/BiCGStab.h:30-108) with x0 = 0 as Solver::Solve uses it.
SolveStats BiCGStabSolve(const GeneralizedSystem &sys, std::vector<double> &x, const std::vector<double> &b,
                         double tolerance, int max_iterations);

class Solver {
  public:
    void Init(double m, double n, const SpMat &L, const SpMat &E, Preconditioner precond,
              const std::vector<bool> &identity_rows, int nD = 0);
    void SetPrecond(int iters) { m_sys.precond_iters = iters; }
    // tol 1e-10, max 100000 iterations, x0 = 0 (src/Solver.cpp:69-114)
    std::vector<double> Solve(const std::vector<double> &rhs, double tol = 1e-10, int max_iters = 100000);
    void Multiply(const std::vector<double> &x, std::vector<double> &b, double m, double n) const { m_sys.Multiply(x, b, m, n); }
    const GeneralizedSystem &system() const { return m_sys; }
    const SolveStats &stats() const { return m_stats; }

  private:
    GeneralizedSystem m_sys;
    SolveStats m_stats;
};

// Dot products used by the restated BiCGStab.
double DotSerial(const std::vector<double> &a, const std::vector<double> &b);

}  // namespace cpmref
