// ORACLE — test infrastructure only. Not part of the product library.
#include "solver.h"

#include <cmath>
#include <limits>

namespace cpmref {

double DotSerial(const std::vector<double> &a, const std::vector<double> &b) {
    double s = 0.0;
    for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
    return s;
}

// SetComponents (src/GeneralizedBiCGStabSystem.h:37-53).
void GeneralizedSystem::SetComponents(double m_in, double n_in, const SpMat &L_in, const SpMat &E_in, Preconditioner p,
                                      const std::vector<bool> &identity_rows_in, int nD_in) {
    m = m_in;
    n = n_in;
    L = L_in;
    E = E_in;
    precond = p;
    identity_rows = identity_rows_in;
    nD = nD_in;
    dofs = L.rows - nD;
}

// Interpolation (src/GeneralizedBiCGStabSystem.h:235-261): rows of E in order;
// identity rows copy x; other rows sum val*x[col] in ascending column order.
void GeneralizedSystem::Interp(const std::vector<double> &x, std::vector<double> &t) const {
    t.assign(dofs + nD, 0.0);
#pragma omp parallel for schedule(static) if (ParallelRows())
    for (long long kk = 0; kk < (long long)E.rows; ++kk) {
        const size_t k = (size_t)kk;
        if (identity_rows[k]) {
            t[k] = x[k];
        } else {
            double acc = 0.0;
            for (size_t e = E.ptr[k]; e < E.ptr[k + 1]; ++e) acc += E.val[e] * x[E.idx[e]];
            t[k] = acc;
        }
    }
}

// Multiply (src/GeneralizedBiCGStabSystem.h:191-233): t = E~x; result = offdiag(L) t;
// tmp = diag(L) x; finalise m*x + n*(tmp + result); identity rows -> x; nD rows -> (m-n)x.
void GeneralizedSystem::Multiply(const std::vector<double> &x, std::vector<double> &result, double m_in, double n_in) const {
    std::vector<double> t;
    Interp(x, t);
    result.assign(x.size(), 0.0);
    // LnodiagTimesX (:93-115)
#pragma omp parallel for schedule(static) if (ParallelRows())
    for (long long kk = 0; kk < (long long)L.rows; ++kk) {
        const size_t k = (size_t)kk;
        double acc = 0.0;
        for (size_t e = L.ptr[k]; e < L.ptr[k + 1]; ++e)
            if (L.idx[e] != k) acc += L.val[e] * t[L.idx[e]];
        result[k] = acc;
    }
    // LdiagTimesX (:65-91)
    std::vector<double> tmp(dofs + nD, 0.0);
#pragma omp parallel for schedule(static) if (ParallelRows())
    for (long long kk = 0; kk < (long long)dofs; ++kk) {
        const size_t k = (size_t)kk;
        for (size_t e = L.ptr[k]; e < L.ptr[k + 1]; ++e)
            if (L.idx[e] == k) tmp[k] += L.val[e] * x[k];
    }
    for (int i = 0; i < nD; ++i) tmp[dofs + i] = (m_in - n_in) * x[dofs + i];
    // FinalizeMultiplication (:166-189)
#pragma omp parallel for schedule(static) if (ParallelRows())
    for (long long qq = 0; qq < (long long)dofs; ++qq) {
        const size_t q = (size_t)qq;
        if (identity_rows[q])
            result[q] = x[q];
        else
            result[q] = m_in * x[q] + n_in * (tmp[q] + result[q]);
    }
    for (int i = 0; i < nD; ++i) result[dofs + i] = (m_in - n_in) * x[dofs + i];
}

// Diagonal_Inverse, non-"computed" branch (src/GeneralizedBiCGStabSystem.h:281-340):
// out = in / (m + L_kk*n) with L_kk the first diagonal entry of row k.
void GeneralizedSystem::DiagonalInverse(const std::vector<double> &in, std::vector<double> &out) const {
    out.resize(in.size());
#pragma omp parallel for schedule(static)
    for (long long kk = 0; kk < (long long)L.rows; ++kk) {
        size_t k = (size_t)kk;
        if (identity_rows[k]) {
            out[k] = in[k];
            continue;
        }
        bool found = false;
        for (size_t e = L.ptr[k]; e < L.ptr[k + 1]; ++e) {
            if (L.idx[e] == k) {
                double v = m + L.val[e] * n;
                out[k] = in[k] / v;
                found = true;
                break;
            }
        }
        if (!found) out[k] = in[k];
    }
    for (int i = 0; i < nD; ++i) out[dofs + i] = in[dofs + i] / (m - n);
}

// Precondition (src/GeneralizedBiCGStabSystem.h:350-385). The Jacobi branch
// allocates its scratch as dofs+2 in the reference (:362-363), which only works
// through Eigen's release-mode resizing; the restatement sizes it dofs.
void GeneralizedSystem::Precondition(const std::vector<double> &x, std::vector<double> &result) const {
    if (precond == Preconditioner::diagonal) {
        DiagonalInverse(x, result);
    } else if (precond == Preconditioner::jacobi) {
        result.assign(x.size(), 0.0);
        std::vector<double> tmp, res(x.size());
        const double omega = 2.0 / 3.0;
        for (int i = 0; i < precond_iters; ++i) {
            Multiply(result, tmp);
            for (size_t q = 0; q < x.size(); ++q) res[q] = x[q] - tmp[q];
            DiagonalInverse(res, res);
            for (size_t q = 0; q < dofs; ++q) result[q] += omega * res[q];
        }
    } else {
        result = x;
    }
}

// BiCGStab::Solve (src/BiCGStab.h:30-108).
SolveStats BiCGStabSolve(const GeneralizedSystem &sys, std::vector<double> &x, const std::vector<double> &b,
                         double tolerance, int max_iterations) {
    return BiCGStabSolveOp([&](const std::vector<double> &a, std::vector<double> &o) { sys.Multiply(a, o); },
                           [&](const std::vector<double> &a, std::vector<double> &o) { sys.Precondition(a, o); }, x, b,
                           tolerance, max_iterations);
}

SolveStats BiCGStabSolveOp(const LinOp &multiply, const LinOp &precondition, std::vector<double> &x,
                           const std::vector<double> &b, double tolerance, int max_iterations) {
    SolveStats st;
    const size_t N = b.size();
    std::vector<double> r(N), r0(N, 0.0), v(N, 0.0), p(N, 0.0), s(N), t(N), y(N), z(N);
    r = b;
    multiply(x, r0);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)N; ++i) r[i] -= r0[i];
    r0 = r;
    double r0_sqnorm = DotSerial(r0, r0);
    double rhs_sqnorm = DotSerial(b, b);
    if (rhs_sqnorm == 0.0) {
        x.assign(N, 0.0);
        st.converged = true;
        return st;
    }
    double rho = 1.0, alpha = 1.0, w = 1.0;
    double tol2 = tolerance * tolerance * rhs_sqnorm;
    const double eps = std::numeric_limits<double>::epsilon();
    double eps2 = eps * eps;
    int iters = 0, restarts = 0;
    double rr = DotSerial(r, r);
    while (rr > tol2 && iters < max_iterations) {
        double rho_old = rho;
        rho = DotSerial(r0, r);
        if (std::abs(rho) < eps2 * r0_sqnorm) {
            r = b;
            multiply(x, r0);
#pragma omp parallel for schedule(static)
            for (long long i = 0; i < (long long)N; ++i) r[i] -= r0[i];
            r0 = r;
            rho = r0_sqnorm = DotSerial(r, r);
            if (restarts++ == 0) iters = 0;
        }
        double beta = (rho / rho_old) * (alpha / w);
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < (long long)N; ++i) {
            double pi = -w * v[i] + p[i];
            pi *= beta;
            p[i] = pi + r[i];
        }
        precondition(p, y);
        multiply(y, v);
        alpha = rho / DotSerial(r0, v);
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < (long long)N; ++i) s[i] = -alpha * v[i] + r[i];
        precondition(s, z);
        multiply(z, t);
        double val = DotSerial(t, t);
        w = (val > 0.0) ? DotSerial(t, s) / val : 0.0;
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < (long long)N; ++i) {
            double xi = alpha * y[i] + x[i];
            x[i] = w * z[i] + xi;
            r[i] = -w * t[i] + s[i];
        }
        ++iters;
        rr = DotSerial(r, r);
    }
    st.iterations = iters;
    st.restarts = restarts;
    st.final_rel_residual2 = rr / rhs_sqnorm;
    st.converged = rr <= tol2;
    return st;
}

// Solver::Init / Solve, CUSTOM_SOLVER branch (src/Solver.cpp:8-68, 69-114).
void Solver::Init(double m, double n, const SpMat &L, const SpMat &E, Preconditioner precond,
                  const std::vector<bool> &identity_rows, int nD) {
    m_sys.SetComponents(m, n, L, E, precond, identity_rows, nD);
}

std::vector<double> Solver::Solve(const std::vector<double> &rhs, double tol, int max_iters) {
    std::vector<double> u(rhs.size(), 0.0);
    m_stats = BiCGStabSolve(m_sys, u, rhs, tol, max_iters);
    return u;
}

}  // namespace cpmref
