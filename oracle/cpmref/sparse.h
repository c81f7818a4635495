// ORACLE — test infrastructure only. Not part of the product library.
//
// Row-major CSR matrix with the semantics the reference gets from
// Eigen::SparseMatrix<double, RowMajor> (src/Scalar.h:29-33):
//   * FromTriplets sums duplicate (row, col) entries and stores the columns of
//     every row in ascending order (Eigen setFromTriplets);
//   * iteration over a row visits columns in ascending order, which fixes the
//     summation order of every sparse product in the reference's custom solver.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace cpmref {

struct Triplet {
    size_t row, col;
    double val;
};

// Row loops of the sparse products run serially, as the reference's do (its OPENMP macro
// is never defined); tests may run them on OpenMP threads, which changes no result (each
// row is summed by one thread in its own order).  The CPU baseline keeps them serial.
inline bool &ParallelRows() {
    static bool on = false;
    return on;
}

struct SpMat {
    size_t rows = 0, cols = 0;
    std::vector<size_t> ptr{0};
    std::vector<size_t> idx;
    std::vector<double> val;

    void Resize(size_t r, size_t c) {
        rows = r;
        cols = c;
        ptr.assign(r + 1, 0);
        idx.clear();
        val.clear();
    }

    size_t nnz() const { return idx.size(); }

    void FromTriplets(size_t r, size_t c, const std::vector<Triplet> &t) {
        rows = r;
        cols = c;
        std::vector<size_t> count(r + 1, 0);
        for (const auto &e : t) count[e.row + 1]++;
        for (size_t i = 0; i < r; ++i) count[i + 1] += count[i];
        std::vector<size_t> ci(t.size());
        std::vector<double> cv(t.size());
        std::vector<size_t> pos(count.begin(), count.end() - 1);
        for (const auto &e : t) {  // stable: insertion order kept per row
            size_t p = pos[e.row]++;
            ci[p] = e.col;
            cv[p] = e.val;
        }
        ptr.assign(r + 1, 0);
        idx.clear();
        val.clear();
        idx.reserve(t.size());
        val.reserve(t.size());
        std::vector<size_t> order;
        for (size_t i = 0; i < r; ++i) {
            size_t b = count[i], e = count[i + 1];
            order.resize(e - b);
            for (size_t k = 0; k < e - b; ++k) order[k] = b + k;
            std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t bb) { return ci[a] < ci[bb]; });
            for (size_t k = 0; k < order.size(); ++k) {
                size_t o = order[k];
                if (!idx.empty() && idx.size() > ptr[i] && idx.back() == ci[o]) {
                    val.back() += cv[o];  // duplicates summed in insertion order
                } else {
                    idx.push_back(ci[o]);
                    val.push_back(cv[o]);
                }
            }
            ptr[i + 1] = idx.size();
        }
    }

    // Lookup of a stored coefficient (0 if absent): the read-only use of coeffRef.
    double Coeff(size_t r, size_t c) const {
        auto b = idx.begin() + ptr[r], e = idx.begin() + ptr[r + 1];
        auto it = std::lower_bound(b, e, c);
        if (it != e && *it == c) return val[it - idx.begin()];
        return 0.0;
    }

    // y = A x, each row summed from 0 in ascending column order (rows on OpenMP threads
    // when ParallelRows() is set: every row's sum is unchanged).
    void Multiply(const std::vector<double> &x, std::vector<double> &y) const {
        y.assign(rows, 0.0);
#pragma omp parallel for schedule(static) if (ParallelRows())
        for (long long ii = 0; ii < (long long)rows; ++ii) {
            const size_t i = (size_t)ii;
            double s = 0.0;
            for (size_t k = ptr[i]; k < ptr[i + 1]; ++k) s += val[k] * x[idx[k]];
            y[i] = s;
        }
    }

    void Scale(double inv_div) {  // A /= s, as Eigen's operator/= (a division per value)
        for (auto &v : val) v = v / inv_div;
    }
};

}  // namespace cpmref
