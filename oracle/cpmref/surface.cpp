// ORACLE — test infrastructure only. Not part of the product library.
// Restates the reference's closest-point functions (file:line cited per function).
#include "surface.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <stdexcept>

namespace cpmref {

SurfaceSpec DefaultSpec(SurfaceKind kind) {
    SurfaceSpec s;
    s.kind = kind;
    switch (kind) {
        case SurfaceKind::Sphere:  // src/SurfaceSpecifier.cpp:120-126
            s.params = {1.0};
            s.bbox[0] = -1.0;
            s.bbox[1] = 1.0;
            break;
        case SurfaceKind::Torus:  // src/SurfaceSpecifier.cpp:127-134
            s.params = {2.0, 1.0};
            s.bbox[0] = -3.0;
            s.bbox[1] = 3.0;
            break;
        case SurfaceKind::Circle3D:  // src/SurfaceSpecifier.cpp:90-103
            s.params = {1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0};
            s.bbox[0] = -1.0;
            s.bbox[1] = 1.0;
            break;
        default:
            break;
    }
    return s;
}

// ---------------------------------------------------------------------------
// Uniform-grid candidate search for mesh primitives (oracle-side acceleration;
// the answer is the exact minimum over all primitives, not an approximation).
class MeshGrid {
  public:
    MeshGrid(const SurfaceSpec &spec) : m_spec(spec) {
        m_is_tri = spec.kind == SurfaceKind::Triangulation;
        size_t np = m_is_tri ? spec.faces.size() : spec.segments.size();
        V3 lo{1e300, 1e300, 1e300}, hi{-1e300, -1e300, -1e300};
        for (const V3 &v : spec.vertices)
            for (int d = 0; d < 3; ++d) {
                lo[d] = std::min(lo[d], v[d]);
                hi[d] = std::max(hi[d], v[d]);
            }
        double ext = 0.0;
        for (int d = 0; d < 3; ++d) ext = std::max(ext, hi[d] - lo[d]);
        double margin = 0.05 * ext + 1e-9;
        for (int d = 0; d < 3; ++d) {
            m_lo[d] = lo[d] - margin;
            m_hi[d] = hi[d] + margin;
        }
        // about 2 primitives per occupied cell on a surface mesh
        int res = (int)std::ceil(std::sqrt((double)np) * 0.7);
        res = std::max(4, std::min(res, 512));
        m_h = 0.0;
        for (int d = 0; d < 3; ++d) m_h = std::max(m_h, (m_hi[d] - m_lo[d]) / res);
        for (int d = 0; d < 3; ++d) m_n[d] = std::max(1, (int)std::ceil((m_hi[d] - m_lo[d]) / m_h));
        std::vector<std::vector<uint32_t>> cells((size_t)m_n[0] * m_n[1] * m_n[2]);
        for (size_t p = 0; p < np; ++p) {
            V3 plo{1e300, 1e300, 1e300}, phi{-1e300, -1e300, -1e300};
            int nv = m_is_tri ? 3 : 2;
            for (int k = 0; k < nv; ++k) {
                const V3 &v = spec.vertices[m_is_tri ? spec.faces[p][k] : spec.segments[p][k]];
                for (int d = 0; d < 3; ++d) {
                    plo[d] = std::min(plo[d], v[d]);
                    phi[d] = std::max(phi[d], v[d]);
                }
            }
            int c0[3], c1[3];
            for (int d = 0; d < 3; ++d) {
                c0[d] = Clamp((int)std::floor((plo[d] - m_lo[d]) / m_h), d);
                c1[d] = Clamp((int)std::floor((phi[d] - m_lo[d]) / m_h), d);
            }
            for (int i = c0[0]; i <= c1[0]; ++i)
                for (int j = c0[1]; j <= c1[1]; ++j)
                    for (int k = c0[2]; k <= c1[2]; ++k) cells[Cell(i, j, k)].push_back((uint32_t)p);
        }
        m_start.assign(cells.size() + 1, 0);
        for (size_t c = 0; c < cells.size(); ++c) m_start[c + 1] = m_start[c] + cells[c].size();
        m_items.resize(m_start.back());
        for (size_t c = 0; c < cells.size(); ++c) std::copy(cells[c].begin(), cells[c].end(), m_items.begin() + m_start[c]);
    }

    // Exact nearest primitive; ties broken by the lower primitive index.
    void Query(const V3 &x, V3 &cp, double &dist) const {
        bool inside = true;
        for (int d = 0; d < 3; ++d)
            if (x[d] < m_lo[d] || x[d] > m_hi[d]) inside = false;
        double best2 = std::numeric_limits<double>::infinity();
        size_t bestp = (size_t)-1;
        V3 bestcp{0, 0, 0};
        auto test = [&](size_t p) {
            V3 c = Prim(x, p);
            V3 dv = Sub(x, c);
            double d2 = Dot(dv, dv);
            if (d2 < best2 || (d2 == best2 && p < bestp)) {
                best2 = d2;
                bestp = p;
                bestcp = c;
            }
        };
        if (!inside) {
            size_t np = m_is_tri ? m_spec.faces.size() : m_spec.segments.size();
            for (size_t p = 0; p < np; ++p) test(p);
        } else {
            int c[3];
            for (int d = 0; d < 3; ++d) c[d] = Clamp((int)std::floor((x[d] - m_lo[d]) / m_h), d);
            int maxring = std::max(m_n[0], std::max(m_n[1], m_n[2]));
            for (int ring = 0; ring <= maxring; ++ring) {
                for (int i = c[0] - ring; i <= c[0] + ring; ++i)
                    for (int j = c[1] - ring; j <= c[1] + ring; ++j)
                        for (int k = c[2] - ring; k <= c[2] + ring; ++k) {
                            if (std::max(std::abs(i - c[0]), std::max(std::abs(j - c[1]), std::abs(k - c[2]))) != ring) continue;
                            if (i < 0 || j < 0 || k < 0 || i >= m_n[0] || j >= m_n[1] || k >= m_n[2]) continue;
                            size_t cc = Cell(i, j, k);
                            for (size_t t = m_start[cc]; t < m_start[cc + 1]; ++t) test(m_items[t]);
                        }
                // every primitive not yet tested lies in a cell at Chebyshev distance > ring,
                // hence at Euclidean distance >= ring * h from x (x lies inside its cell).
                double reach = ring * m_h;
                if (best2 <= reach * reach) break;
            }
        }
        cp = bestcp;
        dist = std::sqrt(best2);
    }

  private:
    const SurfaceSpec &m_spec;
    bool m_is_tri;
    double m_lo[3], m_hi[3], m_h;
    int m_n[3];
    std::vector<size_t> m_start;
    std::vector<uint32_t> m_items;

    int Clamp(int v, int d) const { return std::max(0, std::min(v, m_n[d] - 1)); }
    size_t Cell(int i, int j, int k) const { return ((size_t)i * m_n[1] + j) * m_n[2] + k; }
    V3 Prim(const V3 &x, size_t p) const {
        if (m_is_tri) {
            const auto &f = m_spec.faces[p];
            return ClosestPtPointTriangle(x, m_spec.vertices[f[0]], m_spec.vertices[f[1]], m_spec.vertices[f[2]]);
        }
        const auto &s = m_spec.segments[p];
        return ClosestPtPointSegment(x, m_spec.vertices[s[0]], m_spec.vertices[s[1]]);
    }
};

// ---------------------------------------------------------------------------

Surface::Surface(const SurfaceSpec &spec) : m_spec(spec) {
    if (m_spec.kind == SurfaceKind::Triangulation || m_spec.kind == SurfaceKind::Polyline) {
        m_grid = new MeshGrid(m_spec);
        m_xp = m_spec.vertices;  // parameterization comes from the vertices (src/Surface.cpp:199-202)
    } else {
        Parameterize();
    }
}

Surface::~Surface() { delete m_grid; }

Surface::Surface(Surface &&o) noexcept
    : m_spec(std::move(o.m_spec)), m_xp(std::move(o.m_xp)), m_thetap(std::move(o.m_thetap)), m_phip(std::move(o.m_phip)), m_grid(nullptr) {
    if (o.m_grid) {
        delete o.m_grid;
        o.m_grid = nullptr;
        m_grid = new MeshGrid(m_spec);
    }
}

Surface &Surface::operator=(Surface &&o) noexcept {
    if (this != &o) {
        delete m_grid;
        m_grid = nullptr;
        m_spec = std::move(o.m_spec);
        m_xp = std::move(o.m_xp);
        m_thetap = std::move(o.m_thetap);
        m_phip = std::move(o.m_phip);
        if (o.m_grid) {
            delete o.m_grid;
            o.m_grid = nullptr;
            m_grid = new MeshGrid(m_spec);
        }
    }
    return *this;
}

// Surface::ClosestPoint dispatch (src/Surface.cpp:61-190), in-scope kinds only.
void Surface::ClosestPoint(const V3 &x, V3 &cpx, double &dist, size_t &bdy) const {
    switch (m_spec.kind) {
        case SurfaceKind::Sphere:
            bdy = 0;
            cpSphere(x, cpx, dist);
            break;
        case SurfaceKind::Torus:
            bdy = 0;
            cpTorus(x, cpx, dist);
            break;
        case SurfaceKind::Circle3D:
            bdy = 0;
            cpCircle3D(x, cpx, dist);
            break;
        case SurfaceKind::Point:
            bdy = 0;
            cpPoint(x, cpx, dist);
            break;
        case SurfaceKind::Triangulation:
        case SurfaceKind::Polyline:
            cpMesh(x, cpx, dist, bdy);
            break;
        default:
            throw std::runtime_error("Invalid surface in Surface::ClosestPoint");
    }
}

// cpSphere (src/Surface.cpp:710-741).
void Surface::cpSphere(const V3 &x, V3 &cpx, double &dist) const {
    const double R = m_spec.params[0];
    V3 cen{0.0, 0.0, 0.0};
    if (m_spec.params.size() > 1) cen = V3{m_spec.params[1], m_spec.params[2], m_spec.params[3]};
    V3 xs = Sub(x, cen);
    double phi;
    double theta = std::atan2(xs[1], xs[0]);
    dist = std::sqrt(xs[0] * xs[0] + xs[1] * xs[1] + xs[2] * xs[2]);
    if (dist != 0)
        phi = std::acos(xs[2] / dist);
    else
        phi = 0.0;
    cpx[0] = R * std::sin(phi) * std::cos(theta);
    cpx[1] = R * std::sin(phi) * std::sin(theta);
    cpx[2] = R * std::cos(phi);
    cpx = Add(cpx, cen);
    dist -= R;
}

// cpTorus + cpInnerTorusCircle (src/Surface.cpp:800-838).
void Surface::cpTorus(const V3 &x, V3 &cpx, double &dist) const {
    double theta = std::atan2(x[1], x[0]);
    double r = std::sqrt(x[0] * x[0] + x[1] * x[1]);
    const double Rmaj = m_spec.params[0];
    const double rmin = m_spec.params[1];
    // cylx = (r, z); cen = (R, 0); shift = cylx - cen
    double s0 = r - Rmaj, s1 = x[2] - 0.0;
    double th = std::atan2(s1, s0);
    double c0 = rmin * std::cos(th) + Rmaj;
    double c1 = rmin * std::sin(th) + 0.0;
    double a = r - c0, b = x[2] - c1;
    double acc = 0.0;
    acc += a * a;
    acc += b * b;
    dist = std::sqrt(acc);
    cpx[0] = c0 * std::cos(theta);
    cpx[1] = c0 * std::sin(theta);
    cpx[2] = c1;
}

void ComputeOrthogonalBasis(const V3 &n, V3 &t1, V3 &t2) {
    if (std::abs(n[0]) > std::abs(n[1])) {
        t1 = V3{-n[2], 0, n[0]};
    } else {
        t1 = V3{0, n[2], -n[1]};
    }
    t2 = Cross(n, t1);
}

// cpCircle3D (src/Surface.cpp:464-504).
void Surface::cpCircle3D(const V3 &x, V3 &cpx, double &dist) const {
    const auto &p = m_spec.params;
    const double R = p[0];
    V3 centre{p[1], p[2], p[3]};
    V3 normal{p[4], p[5], p[6]};
    V3 t1, t2;
    ComputeOrthogonalBasis(normal, t1, t2);
    V3 ctx = Sub(x, centre);
    double a = Dot(normal, normal) * Dot(t1, ctx);
    double b = Dot(t2, ctx);
    V3 s = Add(Scale(a, t1), Scale(b, t2));
    double ns = Norm(s);
    if (ns > 0) {
        cpx = Add(centre, Div(Scale(R, s), Norm(s)));
        double height = Dot(normal, ctx);
        double radial = Norm(Cross(normal, ctx)) - R;
        dist = std::sqrt(height * height + radial * radial);
    } else {
        if (Norm(t1) > Norm(t2))
            cpx = Add(centre, Div(Scale(R, t1), Norm(t1)));
        else
            cpx = Add(centre, Div(Scale(R, t2), Norm(t2)));
        dist = R;
    }
}

// cpPoint (src/Surface.cpp:840-848).
void Surface::cpPoint(const V3 &x, V3 &cpx, double &dist) const {
    for (int d = 0; d < 3; ++d) cpx[d] = m_spec.params[d];
    dist = Distance(x, cpx);
}

// Mesh / polyline closest point: exact FP64 in place of fcpw (src/Surface.cpp:1751-1780).
// Closed polylines and closed meshes carry bdy = 0 (src/Surface.cpp:2614-2637 tags only open curves).
void Surface::cpMesh(const V3 &x, V3 &cpx, double &dist, size_t &bdy) const {
    m_grid->Query(x, cpx, dist);
    bdy = 0;
}

// Parameterisation points used for error measurement (src/Surface.cpp:193-300,
// paramSphere :1973-1999, paramTorus :2063-2092, paramCircle3D :1883-1904).
void Surface::Parameterize() {
    const double PI = M_PI;
    switch (m_spec.kind) {
        case SurfaceKind::Sphere: {
            size_t Np = 40000, s = 200;
            m_xp.resize(Np);
            m_thetap.resize(Np);
            m_phip.resize(Np);
            double R = m_spec.params[0];
            double dtheta = 2 * PI / (s - 1), dphi = PI / (s - 1);
            for (size_t i = 0; i < s; ++i)
                for (size_t j = 0; j < s; ++j) {
                    m_thetap[i * s + j] = i * dtheta;
                    m_phip[i * s + j] = j * dphi;
                }
            for (size_t i = 0; i < Np; ++i) {
                m_xp[i][0] = R * std::sin(m_phip[i]) * std::cos(m_thetap[i]);
                m_xp[i][1] = R * std::sin(m_phip[i]) * std::sin(m_thetap[i]);
                m_xp[i][2] = R * std::cos(m_phip[i]);
            }
            break;
        }
        case SurfaceKind::Torus: {
            size_t Np = 90000, s = 300;
            m_xp.resize(Np);
            m_thetap.resize(Np);
            m_phip.resize(Np);
            double R = m_spec.params[0], r = m_spec.params[1];
            double du = 2 * PI / (s - 1);
            for (size_t i = 0; i < s; ++i)
                for (size_t j = 0; j < s; ++j) {
                    m_phip[i * s + j] = i * du;
                    m_thetap[i * s + j] = j * du;
                }
            for (size_t i = 0; i < Np; ++i) {
                m_xp[i][0] = (R + r * std::cos(m_thetap[i])) * std::cos(m_phip[i]);
                m_xp[i][1] = (R + r * std::cos(m_thetap[i])) * std::sin(m_phip[i]);
                m_xp[i][2] = r * std::sin(m_thetap[i]);
            }
            break;
        }
        case SurfaceKind::Circle3D: {
            size_t Np = 100;
            m_xp.resize(Np);
            m_thetap.resize(Np);
            const auto &p = m_spec.params;
            double R = p[0];
            V3 centre{p[1], p[2], p[3]}, normal{p[4], p[5], p[6]};
            double dtheta = 2 * PI / (Np - 1);
            V3 t1, t2;
            ComputeOrthogonalBasis(normal, t1, t2);
            Normalize(t1, 0.0);
            Normalize(t2, 0.0);
            for (size_t i = 0; i < Np; ++i) {
                m_thetap[i] = i * dtheta;
                double x1 = std::cos(m_thetap[i]);
                double x2 = std::sin(m_thetap[i]);
                m_xp[i] = Add(centre, Scale(R, Add(Scale(x1, t1), Scale(x2, t2))));
            }
            break;
        }
        case SurfaceKind::Point: {
            m_xp.resize(1);
            for (int d = 0; d < 3; ++d) m_xp[0][d] = m_spec.params[d];
            break;
        }
        default:
            break;
    }
}

// Ericson, Real-Time Collision Detection (2005), 5.1.5 ClosestPtPointTriangle:
// region tests on the barycentric parameters, exact in FP64 up to rounding.
V3 ClosestPtPointTriangle(const V3 &p, const V3 &a, const V3 &b, const V3 &c) {
    V3 ab = Sub(b, a), ac = Sub(c, a), ap = Sub(p, a);
    double d1 = Dot(ab, ap), d2 = Dot(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) return a;
    V3 bp = Sub(p, b);
    double d3 = Dot(ab, bp), d4 = Dot(ac, bp);
    if (d3 >= 0.0 && d4 <= d3) return b;
    double vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        double v = d1 / (d1 - d3);
        return Add(a, Scale(v, ab));
    }
    V3 cp = Sub(p, c);
    double d5 = Dot(ab, cp), d6 = Dot(ac, cp);
    if (d6 >= 0.0 && d5 <= d6) return c;
    double vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        double w = d2 / (d2 - d6);
        return Add(a, Scale(w, ac));
    }
    double va = d3 * d6 - d5 * d4;
    if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
        double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        return Add(b, Scale(w, Sub(c, b)));
    }
    double denom = 1.0 / (va + vb + vc);
    double v = vb * denom, w = vc * denom;
    return Add(a, Add(Scale(v, ab), Scale(w, ac)));
}

// Ericson 5.1.2 ClosestPtPointSegment.
V3 ClosestPtPointSegment(const V3 &p, const V3 &a, const V3 &b) {
    V3 ab = Sub(b, a);
    double t = Dot(Sub(p, a), ab);
    if (t <= 0.0) return a;
    double denom = Dot(ab, ab);
    if (t >= denom) return b;
    t = t / denom;
    return Add(a, Scale(t, ab));
}

}  // namespace cpmref
