// ORACLE — test infrastructure only. Not part of the product library.
//
// Surfaces and their closest-point functions, restated from the reference's
// Surface / SurfaceSpecifier classes for the surface kinds on the solve path:
//   Sphere    src/Surface.cpp:710-741      defaults src/SurfaceSpecifier.cpp:120-126
//   Torus     src/Surface.cpp:800-838      defaults src/SurfaceSpecifier.cpp:127-134
//   Circle3D  src/Surface.cpp:464-504      defaults src/SurfaceSpecifier.cpp:90-103
//   Point     src/Surface.cpp:840-848
//   Triangulation / Polyline: the reference queries fcpw (float BVH, not in the
//   reference tree, src/Surface.cpp:1751-1780).  The oracle instead computes the
//   exact FP64 point-triangle / point-segment closest point (Ericson, "Real-Time
//   Collision Detection", 2005, section 5.1.5 and 5.1.2) by brute force over a
//   uniform-grid candidate search.  Mesh-CP parity with fcpw is therefore unpinned.
#pragma once

#include <string>
#include <vector>

#include "vecmath.h"

namespace cpmref {

enum class SurfaceKind { Sphere = 0, Torus = 1, Circle3D = 2, Point = 3, Triangulation = 4, Polyline = 5 };

// IBCMetaData (src/IBCMetaData.h:9-24).
struct IBCMeta {
    bool is_oriented = false;
    std::vector<double> point_on_side1;
    size_t boundary_type[2] = {0, 0};
    size_t boundary_order = 1;
    double on_ibc_tolerance = 0.0;
    bool use_cp_diff_directions = false;
    bool use_Jcp_surface_normals = true;
    double ibc_DOFSubset_radius_scale = 1.0;
};

struct SurfaceSpec {
    SurfaceKind kind = SurfaceKind::Sphere;
    std::vector<double> params;
    double bbox[2] = {-1.0, 1.0};
    IBCMeta meta;
    // Triangulation: vertices + triangles; Polyline: vertices + segments (pairs).
    std::vector<V3> vertices;
    std::vector<std::array<size_t, 3>> faces;
    std::vector<std::array<size_t, 2>> segments;
};

// SurfaceSpecifier::SetSurface(string) defaults (src/SurfaceSpecifier.cpp:65-242).
SurfaceSpec DefaultSpec(SurfaceKind kind);

class MeshGrid;  // uniform-grid candidate search over mesh primitives

class Surface {
  public:
    Surface() = default;
    explicit Surface(const SurfaceSpec &spec);
    ~Surface();
    Surface(const Surface &) = delete;
    Surface &operator=(const Surface &) = delete;
    Surface(Surface &&) noexcept;
    Surface &operator=(Surface &&) noexcept;

    void ClosestPoint(const V3 &x, V3 &cpx, double &dist, size_t &bdy) const;
    void ClosestPoint(const V3 &x, V3 &cpx) const {
        double d;
        size_t b;
        ClosestPoint(x, cpx, d, b);
    }

    const SurfaceSpec &spec() const { return m_spec; }
    SurfaceKind kind() const { return m_spec.kind; }
    const std::vector<double> &params() const { return m_spec.params; }
    const std::vector<V3> &xp() const { return m_xp; }
    const std::vector<double> &thetap() const { return m_thetap; }
    const std::vector<double> &phip() const { return m_phip; }
    const double *bbox() const { return m_spec.bbox; }

  private:
    SurfaceSpec m_spec;
    std::vector<V3> m_xp;
    std::vector<double> m_thetap, m_phip;
    MeshGrid *m_grid = nullptr;

    void Parameterize();
    void cpSphere(const V3 &x, V3 &cpx, double &dist) const;
    void cpTorus(const V3 &x, V3 &cpx, double &dist) const;
    void cpCircle3D(const V3 &x, V3 &cpx, double &dist) const;
    void cpPoint(const V3 &x, V3 &cpx, double &dist) const;
    void cpMesh(const V3 &x, V3 &cpx, double &dist, size_t &bdy) const;
};

// Ericson 5.1.5: closest point on triangle abc to p (exact FP64 arithmetic).
V3 ClosestPtPointTriangle(const V3 &p, const V3 &a, const V3 &b, const V3 &c);
// Ericson 5.1.2: closest point on segment ab to p.
V3 ClosestPtPointSegment(const V3 &p, const V3 &a, const V3 &b);

// ComputeOrthogonalBasis (src/Surface.cpp:443-461).
void ComputeOrthogonalBasis(const V3 &n, V3 &t1, V3 &t2);

}  // namespace cpmref
