// Symmetric 3x3 eigen-decomposition by the cyclic Jacobi method (Golub & Van
// Loan, Matrix Computations, 4th ed., 8.5.2), host and device.  Eigenvalues
// ascending; vec[r][c] is component r of the eigenvector of val[c].  Used for
// the closest-point Jacobian frames of Geometry::EigenDecomposition
// (src/Geometry.cpp:72-98), where only sign-invariant quantities are consumed.
#pragma once

#include <math.h>

namespace cpm {

struct Eig3 {
    double val[3];
    double vec[3][3];
};

__host__ __device__ inline Eig3 sym_eig3(const double Ain[3][3]) {
    double a[3][3], v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a[i][j] = Ain[i][j];
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
        double scale = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2] + 2 * off;
        if (off == 0.0 || off <= 1e-36 * scale) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                double apq = a[p][q];
                if (apq == 0.0) continue;
                double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; ++k) {
                    double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - s * akq;
                    a[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {
                    double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - s * aqk;
                    a[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = c * vkp - s * vkq;
                    v[k][q] = s * vkp + c * vkq;
                }
            }
    }
    int o[3] = {0, 1, 2};
    double d[3] = {a[0][0], a[1][1], a[2][2]};
    for (int i = 0; i < 3; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (d[o[j]] < d[o[i]]) {
                int tmp = o[i];
                o[i] = o[j];
                o[j] = tmp;
            }
    Eig3 e;
    for (int c = 0; c < 3; ++c) {
        e.val[c] = d[o[c]];
        for (int r = 0; r < 3; ++r) e.vec[r][c] = v[r][o[c]];
    }
    return e;
}

}  // namespace cpm
