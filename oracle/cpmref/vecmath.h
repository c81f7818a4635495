// ORACLE — test infrastructure only. Not part of the product library.
//
// Small fixed-size vector helpers that reproduce the exact floating-point
// operation order of the reference's std::vector<Scalar> helpers
// (src/VectorMath.cpp:10-250). Every function below names the reference
// function whose arithmetic it restates.  Built with -ffp-contract=off so
// that no multiply-add is fused on any host (x86 or Arm).
#pragma once

#include <array>
#include <cmath>
#include <cstddef>
#include <vector>

namespace cpmref {

using Scalar = double;
using V3 = std::array<double, 3>;

// DotProduct (src/VectorMath.cpp:10-21): 0.0 + u0*v0 + u1*v1 + u2*v2, left to right.
inline double Dot(const V3 &u, const V3 &v) {
    double s = 0.0;
    for (int d = 0; d < 3; ++d) s += u[d] * v[d];
    return s;
}

// Norm (src/VectorMath.cpp:24-28) = sqrt(DotProduct(u, u)).
inline double Norm(const V3 &u) { return std::sqrt(Dot(u, u)); }

// CrossProduct (src/VectorMath.cpp:63-74).
inline V3 Cross(const V3 &u, const V3 &v) {
    return V3{u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
}

// Distance (src/VectorMath.cpp:78-89): 0.0 + (u0-v0)^2 + ..., pow(.,2) == x*x.
inline double Distance(const V3 &u, const V3 &v) {
    double s = 0.0;
    for (int d = 0; d < 3; ++d) {
        double t = u[d] - v[d];
        s += t * t;
    }
    return std::sqrt(s);
}

inline V3 Add(const V3 &u, const V3 &v) { return V3{u[0] + v[0], u[1] + v[1], u[2] + v[2]}; }
inline V3 Sub(const V3 &u, const V3 &v) { return V3{u[0] - v[0], u[1] - v[1], u[2] - v[2]}; }
// operator*(Scalar, vector) (src/VectorMath.cpp:215-224): scale * u[d].
inline V3 Scale(double a, const V3 &u) { return V3{a * u[0], a * u[1], a * u[2]}; }
// operator/(vector, Scalar) (src/VectorMath.cpp:227-236): u[d] / scale.
inline V3 Div(const V3 &u, double a) { return V3{u[0] / a, u[1] / a, u[2] / a}; }

// Normalize (src/VectorMath.cpp:36-53): divide by the norm if norm > zero_tol, else zero.
inline void Normalize(V3 &u, double zero_tol) {
    double n = Norm(u);
    if (n > zero_tol) {
        for (int d = 0; d < 3; ++d) u[d] /= n;
    } else {
        u = V3{0.0, 0.0, 0.0};
    }
}

}  // namespace cpmref
