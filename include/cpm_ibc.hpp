// C++ classes with the reference's names over the C-ABI of cpm_gpu.h, so that
// code written against cpm-ibc's custom-solver path (Tube, Solver,
// PoissonWithIBC, HeatWithIBC, GeodesicDistance) can call the GB300 path.
//
// Differences a caller sees:
//   * vectors are std::vector<double> (the reference uses Eigen::VectorX);
//     they are in the reference's row layout: tube rows in the reference's
//     breadth-first node numbering (src/Tube.cpp:321-454), then the IBC DOF
//     rows and Dirichlet value rows (src/IBCSubsets.cpp:74-116);
//   * errors throw std::runtime_error with the library's message where the
//     reference throws, and also where it would return silently (a solve
//     that does not converge, src/BiCGStab.h:107);
//   * a Solver can run the reference's FP64 BiCGStab (precision 0) or FP32
//     BiCGStab with FP64 reliable updates (precision 1).
// Header-only; link against libcpmgpu.so.
#pragma once

#include <algorithm>
#include <array>
#include <cctype>
#include <cstdint>
#include <fstream>
#include <functional>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "cpm_gpu.h"

namespace cpm_gb300 {

using Scalar = double;
using VectorX = std::vector<Scalar>;
using Point3 = std::array<Scalar, 3>;

// src/Defines.h:13-18
enum class Preconditioner { identity = 0, diagonal = 1, jacobi = 2 };

inline void check(int rc) {
    if (rc != CPM_OK) throw std::runtime_error(std::string("cpm_gb300: ") + cpm_last_error());
}

// SimplePolygonMesh (src/SimplePolygonMesh.h): a polygon mesh or polyline read
// from an OBJ file (SimplePolygonMesh::readMeshFromFile / readMeshFromObjFile,
// src/SimplePolygonMesh.cpp:103-222): "v" records are vertices, "f" records
// faces whose tokens are "v", "v/vt", "v//vn" or "v/vt/vn" (1-based; a "\"
// token continues the face on the next line), "l" records polylines, kept as
// their consecutive segments; other records are skipped.
class SimplePolygonMesh {
  public:
    std::vector<std::vector<Scalar>> vertices;
    std::vector<std::vector<size_t>> faces;

    SimplePolygonMesh() = default;
    explicit SimplePolygonMesh(const std::string &filename) { readMeshFromFile(filename); }
    size_t nVertices() const { return vertices.size(); }
    size_t nFaces() const { return faces.size(); }

    void readMeshFromFile(const std::string &filename) {
        const std::string::size_type dot = filename.rfind('.');
        std::string ext = dot == std::string::npos ? "" : filename.substr(dot + 1);
        for (char &c : ext) c = (char)std::tolower((unsigned char)c);
        if (ext != "obj") throw std::runtime_error("Did not recognize mesh file type " + ext);
        std::ifstream in(filename, std::ios::binary);
        if (!in) throw std::runtime_error("couldn't open file " + filename);
        readMeshFromObjFile(in);
    }

    void readMeshFromObjFile(std::istream &in) {
        vertices.clear();
        faces.clear();
        std::string line;
        while (std::getline(in, line)) {
            std::istringstream ss(line);
            std::string rec;
            if (!(ss >> rec)) continue;
            if (rec == "v") {
                std::vector<Scalar> p;
                Scalar v;
                while (ss >> v) p.push_back(v);
                vertices.push_back(p);
            } else if (rec == "f") {
                std::vector<size_t> f;
                std::string tok;
                for (;;) {
                    if (!(ss >> tok)) break;
                    if (tok == "\\") {  // continued on the next line
                        if (!std::getline(in, line)) break;
                        ss.clear();
                        ss.str(line);
                        continue;
                    }
                    f.push_back(index_of(tok.substr(0, tok.find('/'))));
                }
                faces.push_back(f);
            } else if (rec == "l") {
                std::vector<size_t> ids;
                std::string tok;
                while (ss >> tok) ids.push_back(index_of(tok));
                for (size_t i = 0; i + 1 < ids.size(); ++i) faces.push_back({ids[i], ids[i + 1]});
            }
        }
    }

  private:
    static size_t index_of(const std::string &tok) {
        const long long i = std::stoll(tok);
        if (i < 1) throw std::runtime_error("OBJ index " + tok + " is not a 1-based vertex index");
        return (size_t)(i - 1);
    }
};

// Helpers::WriteCSV / ReadCSV (src/Helpers.cpp:11-82): one vector as one line of
// comma-separated values, or a table as one line per row; values written with
// the stream's default formatting, read with std::stod.
struct Helpers {
    template <class V>
    static void WriteCSV(const V &data, const std::string &filename) {
        std::ofstream f(filename);
        for (size_t i = 0; i < data.size(); ++i) f << data[i] << (i + 1 < data.size() ? "," : "\n");
    }
    static void WriteCSV(const std::vector<std::vector<Scalar>> &data, const std::string &filename) {
        std::ofstream f(filename);
        for (const auto &row : data)
            for (size_t i = 0; i < row.size(); ++i) f << row[i] << (i + 1 < row.size() ? "," : "\n");
    }
    static void ReadCSV(const std::string &filename, std::vector<std::vector<Scalar>> &data) {
        std::ifstream in(filename);
        std::string line;
        while (std::getline(in, line)) {
            std::istringstream ss(line);
            std::string tok;
            std::vector<Scalar> row;
            while (std::getline(ss, tok, ',')) row.push_back(std::stod(tok));
            data.push_back(row);
        }
    }
    static void ReadCSV(const std::string &filename, VectorX &data) {
        std::vector<std::vector<Scalar>> t;
        ReadCSV(filename, t);
        if (t.size() != 1)
            throw std::runtime_error("In Helpers::ReadCSV(), " + filename + " does not contain one line of comma separated values");
        data = t[0];
    }
};

// SurfaceSpecifier (src/SurfaceSpecifier.h:198-216) with the IBCMetaData
// fields (src/IBCMetaData.h:9-24) an IBC curve carries.
class SurfaceSpecifier {
  public:
    static SurfaceSpecifier Sphere(Scalar R = 1.0, std::array<Scalar, 2> bbox = {-1.0, 1.0}) {
        return analytic(CPM_SPHERE, {R}, bbox);
    }
    static SurfaceSpecifier Torus(Scalar R, Scalar r, std::array<Scalar, 2> bbox) { return analytic(CPM_TORUS, {R, r}, bbox); }
    static SurfaceSpecifier Circle3D(Scalar R, Point3 centre, Point3 normal, std::array<Scalar, 2> bbox) {
        return analytic(CPM_CIRCLE3D, {R, centre[0], centre[1], centre[2], normal[0], normal[1], normal[2]}, bbox);
    }
    static SurfaceSpecifier Point(Point3 p, std::array<Scalar, 2> bbox) { return analytic(CPM_POINT, {p[0], p[1], p[2]}, bbox); }
    // a triangle mesh: 3 coordinates per vertex, 3 vertex indices per face; the
    // bounding interval is derived as SurfaceSpecifier::SetSurface does
    // (src/SurfaceSpecifier.cpp:346-361)
    static SurfaceSpecifier Triangulation(std::vector<Scalar> verts, std::vector<int64_t> faces) {
        Scalar lo = 0.0, hi = 0.0;
        for (Scalar v : verts) {
            lo = std::min(lo, v);
            hi = std::max(hi, v);
        }
        SurfaceSpecifier s = analytic(CPM_TRIANGULATION, {}, {lo, hi});
        s.verts_ = std::move(verts);
        s.prims_ = std::move(faces);
        return s;
    }
    // a polyline on a surface: 3 coordinates per vertex, 2 vertex indices per segment
    static SurfaceSpecifier Polyline(std::vector<Scalar> verts, std::vector<int64_t> segments, std::array<Scalar, 2> bbox) {
        SurfaceSpecifier s = analytic(CPM_POLYLINE, {}, bbox);
        s.verts_ = std::move(verts);
        s.prims_ = std::move(segments);
        return s;
    }

    // SurfaceSpecifier(SimplePolygonMesh) (src/SurfaceSpecifier.cpp:299-361): a
    // triangulation when the first face has 3 vertices, a polyline when it has 2;
    // the bounding interval spans the vertex coordinates and 0
    static SurfaceSpecifier FromMesh(const SimplePolygonMesh &mesh) {
        if (mesh.faces.empty() || mesh.vertices.empty()) throw std::runtime_error("cpm_gb300: empty mesh");
        std::vector<Scalar> v;
        Scalar lo = 0.0, hi = 0.0;
        for (const auto &p : mesh.vertices) {
            if (p.size() != 3) throw std::runtime_error("cpm_gb300: mesh vertices need 3 coordinates");
            for (Scalar c : p) {
                v.push_back(c);
                lo = std::min(lo, c);
                hi = std::max(hi, c);
            }
        }
        const size_t per = mesh.faces[0].size();
        if (per != 3 && per != 2) throw std::runtime_error("cpm_gb300: faces of 3 (triangulation) or 2 (polyline) vertices");
        std::vector<int64_t> prims;
        for (const auto &f : mesh.faces) {
            if (f.size() != per) throw std::runtime_error("cpm_gb300: faces of mixed sizes");
            for (size_t i : f) prims.push_back((int64_t)i);
        }
        return per == 3 ? Triangulation(std::move(v), std::move(prims)) : Polyline(std::move(v), std::move(prims), {lo, hi});
    }

    // IBCMetaData fields
    SurfaceSpecifier &boundary_order(int order) { d_.boundary_order = order; return *this; }
    SurfaceSpecifier &boundary_type(int side1, int side2) { d_.boundary_type[0] = side1; d_.boundary_type[1] = side2; return *this; }
    SurfaceSpecifier &on_ibc_tolerance(Scalar tol) { d_.on_ibc_tolerance = tol; return *this; }
    SurfaceSpecifier &is_oriented(bool o) { d_.is_oriented = o; return *this; }

    // the descriptor, with its array pointers bound to this object's storage
    const cpm_surface_desc &desc() const {
        d_.nverts = (int64_t)(verts_.size() / 3);
        d_.verts = verts_.empty() ? nullptr : verts_.data();
        const int per = d_.kind == CPM_POLYLINE ? 2 : 3;
        d_.nprims = (int64_t)(prims_.size() / per);
        d_.prims = prims_.empty() ? nullptr : prims_.data();
        return d_;
    }

  private:
    static SurfaceSpecifier analytic(int kind, std::vector<Scalar> params, std::array<Scalar, 2> bbox) {
        SurfaceSpecifier s;
        s.d_ = cpm_surface_desc{};
        s.d_.kind = kind;
        s.d_.nparams = (int32_t)params.size();
        for (size_t i = 0; i < params.size() && i < 8; ++i) s.d_.params[i] = params[i];
        s.d_.bbox[0] = bbox[0];
        s.d_.bbox[1] = bbox[1];
        s.d_.boundary_order = 1;
        s.d_.use_Jcp_surface_normals = 1;
        s.d_.dof_radius_scale = 1.0;
        return s;
    }
    mutable cpm_surface_desc d_{};
    std::vector<Scalar> verts_;
    std::vector<int64_t> prims_;
};

// Surface (src/Surface.h:23-45): ClosestPoint of any surface kind, evaluated on
// the device.  bdy is not reported.  ClosestPoints answers many points in one
// call; max_dist > 0 bounds mesh and polyline searches, and points farther than
// max_dist then report dist > max_dist.
class Surface {
  public:
    explicit Surface(const SurfaceSpecifier &spec) : spec_(spec) {}
    void ClosestPoint(const Point3 &x, Point3 &cpx) const {
        Scalar d = 0;
        ClosestPoint(x, cpx, d);
    }
    void ClosestPoint(const Point3 &x, Point3 &cpx, Scalar &dist) const {
        check(cpm_closest_points(&spec_.desc(), 1, x.data(), 0.0, cpx.data(), &dist));
    }
    void ClosestPoints(const std::vector<Point3> &x, std::vector<Point3> &cpx, std::vector<Scalar> &dist,
                       Scalar max_dist = 0.0) const {
        cpx.resize(x.size());
        dist.resize(x.size());
        if (x.empty()) return;
        check(cpm_closest_points(&spec_.desc(), (int64_t)x.size(), x[0].data(), max_dist, cpx[0].data(), dist.data()));
    }

  private:
    SurfaceSpecifier spec_;
};

// Tube(SurfaceSpecifier&, size_t p, Scalar dx) (src/Tube.h:45) on the device.
class Tube {
  public:
    Tube(const SurfaceSpecifier &surface, size_t p, Scalar dx) {
        cpm_tube_t t = nullptr;
        check(cpm_tube_build(&surface.desc(), (int32_t)p, dx, &t));
        h_.reset(t);
        check(cpm_tube_info_get(t, &info_));
        order_.resize((size_t)info_.n_nodes);
        check(cpm_tube_reference_order(t, order_.data()));
    }
    size_t nNodes() const { return (size_t)info_.n_nodes; }
    size_t N1d() const { return (size_t)info_.n1d; }
    Scalar dx() const { return info_.dx; }
    Scalar xstart() const { return info_.xstart; }
    Scalar TubeRadius() const { return info_.radius; }
    // grid coordinates and closest points in the reference's node numbering
    std::vector<Point3> x() const { return points(true); }
    std::vector<Point3> cpx() const { return points(false); }
    // device index of reference node i (cpm_tube_reference_order)
    const std::vector<int64_t> &device_index() const { return order_; }
    cpm_tube_t handle() const { return h_.get(); }

  private:
    std::vector<Point3> points(bool grid) const {
        const size_t N = nNodes();
        std::vector<Scalar> a(3 * N);
        check(cpm_tube_export(h_.get(), nullptr, grid ? a.data() : nullptr, grid ? nullptr : a.data(), nullptr, nullptr,
                              nullptr, nullptr));
        std::vector<Point3> out(N);
        for (size_t i = 0; i < N; ++i) {
            const size_t q = (size_t)order_[i];
            out[i] = {a[3 * q], a[3 * q + 1], a[3 * q + 2]};
        }
        return out;
    }
    struct Del {
        void operator()(cpm_tube_t t) const { cpm_tube_destroy(t); }
    };
    std::unique_ptr<cpm_tube_s, Del> h_;
    cpm_tube_info info_{};
    std::vector<int64_t> order_;
};

// Lfull, Efull and the identity rows of a tube with IBC curves
// (Helpers::SetupMatrices, IBCSubsets::Initialize, IBCMatrixManipulations
// AddIBCFiniteDifference / AddIBCExtension) kept on the device.
class SystemOperator {
  public:
    SystemOperator(const Tube &tube, const std::vector<SurfaceSpecifier> &ibcs) : tube_(&tube) {
        std::vector<cpm_surface_desc> d;
        for (const auto &s : ibcs) d.push_back(s.desc());
        cpm_opset_t o = nullptr;
        check(cpm_opset_create(tube.handle(), (int32_t)d.size(), d.empty() ? nullptr : d.data(), &o));
        init(tube, o);
    }
    // the nearest-node baselines' operator: plain L and E with identity rows at the
    // given tube rows (reference numbering)
    struct IdentityRows {
        explicit IdentityRows(std::vector<size_t> r) : rows(std::move(r)) {}
        std::vector<size_t> rows;
    };
    SystemOperator(const Tube &tube, const IdentityRows &identity) : tube_(&tube) {
        std::vector<int64_t> rows;
        for (size_t r : identity.rows) rows.push_back(tube.device_index()[r]);
        cpm_opset_t o = nullptr;
        check(cpm_opset_create_identity(tube.handle(), (int64_t)rows.size(), rows.empty() ? nullptr : rows.data(), &o));
        init(tube, o);
    }

  private:
    void init(const Tube &tube, cpm_opset_t o) {
        h_.reset(o);
        int64_t sz[9];
        check(cpm_opset_sizes(o, sz));
        D_ = sz[0];
        N_ = sz[1];
        total_ibc_dofs_ = sz[2];
        n_ibc_ = sz[4];
        const size_t D = (size_t)D_;
        std::vector<uint8_t> ident(D);
        kind_.resize(D);
        ibc_.resize(D);
        std::vector<Scalar> pt(3 * D);
        check(cpm_opset_rows(o, ident.data(), kind_.data(), ibc_.data(), pt.data()));
        side_.resize(D);
        check(cpm_opset_row_sides(o, side_.data()));
        // reference row r -> device row
        dev_.resize(D);
        for (size_t r = 0; r < D; ++r) dev_[r] = r < (size_t)N_ ? tube.device_index()[r] : (int64_t)r;
        point_.resize(D);
        identity_.resize(D);
        for (size_t r = 0; r < D; ++r) {
            const size_t q = (size_t)dev_[r];
            point_[r] = {pt[3 * q], pt[3 * q + 1], pt[3 * q + 2]};
            identity_[r] = ident[q] != 0;
        }
    }

  public:
    size_t rows() const { return (size_t)D_; }
    size_t nNodes() const { return (size_t)N_; }
    size_t TotalIBCDOFs() const { return (size_t)total_ibc_dofs_; }
    size_t NumIBCs() const { return (size_t)n_ibc_; }
    const std::vector<bool> &identity_rows() const { return identity_; }
    // per reference row: 0 tube row, 1 IBC DOF row, 2 Dirichlet value row; its
    // IBC; the point its right-hand side is evaluated at
    int kind(size_t r) const { return kind_[(size_t)dev_[r]]; }
    int ibc(size_t r) const { return ibc_[(size_t)dev_[r]]; }
    // IBCDOFSubset::which_side of an IBC row (1 or 2 on an oriented IBC, 0 otherwise)
    size_t side(size_t r) const { return (size_t)side_[(size_t)dev_[r]]; }
    const Point3 &point(size_t r) const { return point_[r]; }
    VectorX to_device(const VectorX &ref) const {
        VectorX d(ref.size());
        for (size_t r = 0; r < ref.size(); ++r) d[(size_t)dev_[r]] = ref[r];
        return d;
    }
    VectorX from_device(const VectorX &dev) const {
        VectorX ref(dev.size());
        for (size_t r = 0; r < dev.size(); ++r) ref[r] = dev[(size_t)dev_[r]];
        return ref;
    }
    cpm_opset_t handle() const { return h_.get(); }
    const Tube &tube() const { return *tube_; }
    // a solution (reference row order) at surface points, through the interpolation
    // with IBC columns (Helpers::GetPlotInterpMatrix + AddIBCPlotInterpolation,
    // src/Helpers.cpp:97-103, src/IBCMatrixManipulations.cpp:84-106)
    VectorX Evaluate(const VectorX &u, const std::vector<Point3> &xp) const {
        const int64_t n = (int64_t)xp.size();
        std::vector<Scalar> pts(3 * (size_t)n);
        for (size_t i = 0; i < xp.size(); ++i)
            for (int k = 0; k < 3; ++k) pts[3 * i + (size_t)k] = xp[i][(size_t)k];
        int64_t nnz = 0;
        check(cpm_opset_plot_interp_csr(h_.get(), n, pts.data(), &nnz, nullptr, nullptr, nullptr));
        std::vector<int64_t> ptr((size_t)n + 1), cols((size_t)nnz);
        std::vector<Scalar> vals((size_t)nnz);
        check(cpm_opset_plot_interp_csr(h_.get(), n, pts.data(), &nnz, ptr.data(), cols.data(), vals.data()));
        const VectorX ud = to_device(u);
        VectorX out((size_t)n, 0.0);
        for (size_t i = 0; i < (size_t)n; ++i)
            for (int64_t e = ptr[i]; e < ptr[i + 1]; ++e) out[i] += vals[(size_t)e] * ud[(size_t)cols[(size_t)e]];
        return out;
    }

  private:
    struct Del {
        void operator()(cpm_opset_t o) const { cpm_opset_destroy(o); }
    };
    const Tube *tube_;
    std::unique_ptr<cpm_opset_s, Del> h_;
    int64_t D_ = 0, N_ = 0, total_ibc_dofs_ = 0, n_ibc_ = 0;
    std::vector<int64_t> dev_;
    std::vector<int32_t> kind_, ibc_, side_;
    std::vector<Point3> point_;
    std::vector<bool> identity_;
};

// Solver (src/Solver.h:22-26): Init(m, n, ...), SetPrecond, Solve, Multiply.
class Solver {
  public:
    void Init(Scalar m, Scalar n, const SystemOperator &op, Preconditioner p = Preconditioner::diagonal) {
        op_ = &op;
        m_ = m;
        n_ = n;
        precond_ = p;
        cpm_solver_t s = nullptr;
        check(cpm_solver_create(op.handle(), m, n, 1, &s));
        h_.reset(s);
    }
    void SetPrecond(int precond_iters) { precond_iters_ = precond_iters; }
    // 0: the reference's FP64 BiCGStab; 1: FP32 BiCGStab with FP64 reliable updates
    void SetPrecision(int precision) { precision_ = precision; }
    void SetTolerance(Scalar tol) { tol_ = tol; }
    VectorX Solve(const VectorX &rhs) {
        require();
        VectorX b = op_->to_device(rhs), x(b.size());
        cpm_solve_opts o{};
        o.tol = tol_;
        o.max_iters = 100000;
        o.precision = precision_;
        o.precond = (int32_t)precond_;
        o.precond_iters = precond_iters_;
        check(cpm_solve(h_.get(), 1, b.data(), x.data(), &o, &stats_));
        return op_->from_device(x);
    }
    // b = m x + n (diag(L) x + offdiag(L) E~ x), identity rows b = x
    void Multiply(const VectorX &x, VectorX &b, Scalar m, Scalar n) const {
        require();
        VectorX xd = op_->to_device(x), yd(xd.size());
        check(cpm_apply(op_->handle(), m, n, 1, xd.data(), yd.data()));
        b = op_->from_device(yd);
    }
    const cpm_solve_stats &stats() const { return stats_; }

  private:
    void require() const {
        if (!op_ || !h_) throw std::runtime_error("cpm_gb300: Solver::Init was not called");
    }
    struct Del {
        void operator()(cpm_solver_t s) const { cpm_solver_destroy(s); }
    };
    const SystemOperator *op_ = nullptr;
    std::unique_ptr<cpm_solver_s, Del> h_;
    Scalar m_ = 0, n_ = 0, tol_ = 1e-10;
    Preconditioner precond_ = Preconditioner::diagonal;
    int precond_iters_ = 0, precision_ = 0;
    cpm_solve_stats stats_{};
};

using SourceFn = std::function<Scalar(const Point3 &)>;
// Dirichlet value on IBC c at its closest point (side is 0 for non-oriented curves)
using IBCFn = std::function<Scalar(size_t c, size_t side, const Point3 &)>;

// PoissonWithIBC (problems/PoissonWithIBC.h:17-117): -Delta_S u = f with
// Dirichlet values on IBC curves, solved with Init(0, -1, diagonal).
class PoissonWithIBC {
  public:
    PoissonWithIBC(const SurfaceSpecifier &surface, const std::vector<SurfaceSpecifier> &ibcs, Scalar dx,
                   size_t interp_deg = 3, int precision = 0)
        : tube_(surface, interp_deg, dx), op_(tube_, ibcs) {
        sv_.Init(0.0, -1.0, op_);
        sv_.SetPrecision(precision);
    }
    // PoissonWithIBC::GetRHS (problems/PoissonWithIBC.cpp:162-192)
    VectorX GetRHS(const SourceFn &f, const IBCFn &ibc_exact) const {
        VectorX b(op_.rows(), 0.0);
        for (size_t r = 0; r < b.size(); ++r)
            b[r] = op_.kind(r) == 2 ? ibc_exact((size_t)op_.ibc(r), op_.side(r), op_.point(r)) : f(op_.point(r));
        return b;
    }
    VectorX Solve(const VectorX &rhs) { return sv_.Solve(rhs); }
    const Tube &tube() const { return tube_; }
    const SystemOperator &system() const { return op_; }
    Solver &solver() { return sv_; }

  private:
    Tube tube_;
    SystemOperator op_;
    Solver sv_;
};

// PoissonWithIBCNearest (problems/PoissonWithIBCNearest.cpp:5-89): the
// nearest-node baseline.  No IBC columns: identity rows hold exact surface
// values, at the tube rows of each IBC's DOF subset with the value at their IBC
// closest point (freeze_nearest false), or at the tube rows nearest to each
// IBC curve's own plot points with the value there (freeze_nearest true); the
// plain L and E elsewhere, solved with Init(0, -1).
class PoissonWithIBCNearest {
  public:
    PoissonWithIBCNearest(const SurfaceSpecifier &surface, const std::vector<SurfaceSpecifier> &ibcs, Scalar dx,
                          bool freeze_nearest = false, size_t interp_deg = 3, int precision = 0)
        : tube_(surface, interp_deg, dx),
          op_(tube_, SystemOperator::IdentityRows{nearest_rows(tube_, ibcs, freeze_nearest, rows_, cp_)}) {
        sv_.Init(0.0, -1.0, op_);
        sv_.SetPrecision(precision);
    }
    // PoissonWithIBCNearest::GetRHS (problems/PoissonWithIBCNearest.cpp:36-60)
    VectorX GetRHS(const SourceFn &f, const SourceFn &surface_exact) const {
        VectorX b(op_.rows(), 0.0);
        for (size_t r = 0; r < b.size(); ++r) b[r] = f(op_.point(r));
        for (size_t i = 0; i < rows_.size(); ++i) b[rows_[i]] = surface_exact(cp_[i]);
        return b;
    }
    VectorX Solve(const VectorX &rhs) { return sv_.Solve(rhs); }
    const Tube &tube() const { return tube_; }
    const SystemOperator &system() const { return op_; }
    const std::vector<bool> &GetIdentityRows() const { return op_.identity_rows(); }

  private:
    static const std::vector<size_t> &nearest_rows(const Tube &tube, const std::vector<SurfaceSpecifier> &ibcs, bool freeze,
                                                   std::vector<size_t> &rows, std::vector<Point3> &cp) {
        std::vector<size_t> ref_of(tube.nNodes());
        for (size_t r = 0; r < ref_of.size(); ++r) ref_of[(size_t)tube.device_index()[r]] = r;
        if (freeze) {
            for (const auto &ibc : ibcs) {
                int64_t n = 0;
                check(cpm_ibc_plot_points(&ibc.desc(), &n, nullptr));
                std::vector<Scalar> xp(3 * (size_t)n);
                check(cpm_ibc_plot_points(&ibc.desc(), &n, xp.data()));
                std::vector<int64_t> idx((size_t)n);
                check(cpm_tube_nearest(tube.handle(), n, xp.data(), idx.data()));
                for (size_t i = 0; i < (size_t)n; ++i) {
                    if (idx[i] < 0) throw std::runtime_error("cpm_gb300: an IBC plot point has no tube node nearby");
                    rows.push_back(ref_of[(size_t)idx[i]]);
                    cp.push_back({xp[3 * i], xp[3 * i + 1], xp[3 * i + 2]});
                }
            }
            return rows;
        }
        SystemOperator with_ibc(tube, ibcs);
        for (size_t c = 0; c < ibcs.size(); ++c) {
            int64_t sz[5];
            check(cpm_opset_ibc_sizes(with_ibc.handle(), (int32_t)c, sz));
            std::vector<int64_t> tag((size_t)sz[0]), dof((size_t)sz[1]);
            std::vector<Scalar> dcp(3 * (size_t)sz[1]);
            check(cpm_opset_ibc_export(with_ibc.handle(), (int32_t)c, tag.data(), dof.data(), dcp.data()));
            for (size_t i = 0; i < dof.size(); ++i) {
                rows.push_back(ref_of[(size_t)dof[i]]);
                cp.push_back({dcp[3 * i], dcp[3 * i + 1], dcp[3 * i + 2]});
            }
        }
        return rows;
    }
    Tube tube_;
    std::vector<size_t> rows_;
    std::vector<Point3> cp_;
    SystemOperator op_;
    Solver sv_;
};

// HeatWithIBC (problems/HeatWithIBC.h:17-60): time steps of u_t = Delta_S u
// with Dirichlet IBC values; time_stepping_method 0 is explicit (u <- Efull
// (u + dt Lfull u)), 1 backward Euler (Init(1, -dt)), 2 Crank-Nicolson
// (Init(1, -dt/2) with the right-hand side Multiply(u, 1, dt/2)), as
// problems/HeatWithIBC.cpp:115-132.
class HeatWithIBC {
  public:
    HeatWithIBC(const SurfaceSpecifier &surface, const std::vector<SurfaceSpecifier> &ibcs, Scalar dx, Scalar dt,
                size_t time_stepping_method, size_t interp_deg = 3, int precision = 0)
        : tube_(surface, interp_deg, dx), op_(tube_, ibcs), dt_(dt), method_(time_stepping_method) {
        if (method_ > 2) throw std::runtime_error("cpm_gb300: HeatWithIBC time_stepping_method is 0, 1 or 2");
        if (method_ > 0) {
            const Scalar r = method_ == 1 ? 1.0 : 0.5;
            sv_.Init(1.0, -r * dt_, op_);
            sv_.SetPrecision(precision);
        }
    }
    // HeatWithIBC::TimeStep (problems/HeatWithIBC.cpp:104-132): returns u at the next time
    VectorX TimeStep(VectorX &ufull, const IBCFn &ibc_exact) {
        if (method_ == 0) {
            VectorX dev = op_.to_device(ufull), out(dev.size());
            check(cpm_explicit_step(op_.handle(), dt_, 1, dev.data(), out.data()));
            ufull = op_.from_device(out);
            set_dirichlet(ufull, ibc_exact);
            return ufull;
        }
        if (method_ == 2) {
            VectorX tmp;
            sv_.Multiply(ufull, tmp, 1.0, 0.5 * dt_);
            ufull = tmp;
        }
        set_dirichlet(ufull, ibc_exact);
        return sv_.Solve(ufull);
    }
    const Tube &tube() const { return tube_; }
    const SystemOperator &system() const { return op_; }

  private:
    // SetDirichletValue (problems/HeatWithIBC.cpp:62-85)
    void set_dirichlet(VectorX &ufull, const IBCFn &ibc_exact) const {
        for (size_t r = 0; r < ufull.size(); ++r)
            if (op_.kind(r) == 2) ufull[r] = ibc_exact((size_t)op_.ibc(r), op_.side(r), op_.point(r));
    }
    Tube tube_;
    SystemOperator op_;
    Scalar dt_;
    size_t method_;
    Solver sv_;
};

// ReactionDiffusionWithIBC (problems/ReactionDiffusionWithIBC.h): explicit
// Gray-Scott steps (F = 0.054, k = 0.063, nu_u = (dx / 3)^2, nu_v = nu_u / 3)
// of u and v with Dirichlet IBC values, as problems/ReactionDiffusionWithIBC.cpp:93-117.
class ReactionDiffusionWithIBC {
  public:
    ReactionDiffusionWithIBC(const SurfaceSpecifier &surface, const std::vector<SurfaceSpecifier> &ibcs, Scalar dx, Scalar dt,
                             size_t interp_deg = 3)
        : tube_(surface, interp_deg, dx), op_(tube_, ibcs), dt_(dt) {}
    void TimeStep(VectorX &ufull, VectorX &vfull, const IBCFn &ibc_exact_u, const IBCFn &ibc_exact_v) {
        VectorX u = op_.to_device(ufull), v = op_.to_device(vfull);
        check(cpm_gray_scott_step(op_.handle(), dt_, 0.054, 0.063, u.data(), v.data()));
        ufull = op_.from_device(u);
        vfull = op_.from_device(v);
        set_dirichlet(ufull, ibc_exact_u);
        set_dirichlet(vfull, ibc_exact_v);
    }
    const Tube &tube() const { return tube_; }
    const SystemOperator &system() const { return op_; }

  private:
    // SetDirichletValue (problems/ReactionDiffusionWithIBC.cpp:60-90)
    void set_dirichlet(VectorX &ufull, const IBCFn &ibc_exact) const {
        for (size_t r = 0; r < ufull.size(); ++r)
            if (op_.kind(r) == 2) ufull[r] = ibc_exact((size_t)op_.ibc(r), op_.side(r), op_.point(r));
    }
    Tube tube_;
    SystemOperator op_;
    Scalar dt_;
};

// GeodesicDistance::ComputeDistance (problems/GeodesicDistance.cpp:11-69) from
// a point source: returns phi on the tube rows (reference numbering) and the
// point IBC's DOF rows.
class GeodesicDistance {
  public:
    explicit GeodesicDistance(int precision = 0) : precision_(precision) {}
    VectorX ComputeDistance(const Tube &tube, const Point3 &source, Scalar dt) {
        cpm_geodesic_t g = nullptr;
        int64_t D = 0;
        check(cpm_geodesic_create(tube.handle(), source.data(), &g, &D));
        std::unique_ptr<cpm_geodesic_s, Del> hold(g);
        VectorX phi((size_t)D);
        check(cpm_geodesic_run(g, dt, precision_, 1e-10, 2000, phi.data(), iterations_.data()));
        VectorX out(phi);
        for (size_t i = 0; i < tube.nNodes(); ++i) out[i] = phi[(size_t)tube.device_index()[i]];
        return out;
    }
    const std::array<int32_t, 4> &iterations() const { return iterations_; }

  private:
    struct Del {
        void operator()(cpm_geodesic_t g) const { cpm_geodesic_destroy(g); }
    };
    int precision_;
    std::array<int32_t, 4> iterations_{};
};

// GeodesicDistanceNearest (problems/GeodesicDistanceNearest.h:21-49): the heat
// method on the plain tube operator with identity rows at each curve's
// constraint nodes and smoothed heat sources at the nodes inside the curves'
// tubes (the caller's lists, reference row order, as
// examples/GeodesicDistanceBeetle/GeodesicDistanceBeetle.cpp:36-52 builds
// them).  ComputeDistance returns phi on the tube rows (reference order); Plot
// gives plotE * phi at surface points (the reference's return value, :48-52).
class GeodesicDistanceNearest {
  public:
    explicit GeodesicDistanceNearest(bool visualize = false, int precision = 0) : precision_(precision) { (void)visualize; }
    VectorX ComputeDistance(const Tube &tube, const std::vector<std::vector<size_t>> &ibc_idx,
                            const std::vector<std::vector<size_t>> &inside_ibc_idx,
                            const std::vector<std::vector<Scalar>> &inside_ibc_idx_dist, Scalar dt) {
        const size_t N = tube.nNodes();
        auto dev = [&](size_t r) {
            if (r >= N) throw std::runtime_error("cpm_gb300: GeodesicDistanceNearest row outside the tube");
            return tube.device_index()[r];
        };
        std::vector<int64_t> a, b;
        std::vector<Scalar> d;
        for (const auto &c : ibc_idx)
            for (size_t r : c) a.push_back(dev(r));
        if (inside_ibc_idx.size() != inside_ibc_idx_dist.size())
            throw std::runtime_error("cpm_gb300: inside_ibc_idx and inside_ibc_idx_dist differ in size");
        for (size_t c = 0; c < inside_ibc_idx.size(); ++c) {
            if (inside_ibc_idx[c].size() != inside_ibc_idx_dist[c].size())
                throw std::runtime_error("cpm_gb300: inside_ibc_idx and inside_ibc_idx_dist differ in size");
            for (size_t i = 0; i < inside_ibc_idx[c].size(); ++i) {
                b.push_back(dev(inside_ibc_idx[c][i]));
                d.push_back(inside_ibc_idx_dist[c][i]);
            }
        }
        cpm_geodesic_nearest_t g = nullptr;
        check(cpm_geodesic_nearest_create(tube.handle(), (int64_t)a.size(), a.data(), (int64_t)b.size(), b.data(), d.data(), &g));
        std::unique_ptr<cpm_geodesic_nearest_s, Del> hold(g);
        VectorX phi(N);
        check(cpm_geodesic_nearest_run(g, dt, precision_, 1e-10, 2000, phi.data(), iterations_.data()));
        VectorX out(N);
        for (size_t i = 0; i < N; ++i) out[i] = phi[(size_t)tube.device_index()[i]];
        return out;
    }
    // plotE * phi (Helpers::GetPlotInterpMatrix, src/Helpers.cpp:97-103) at the points xp
    static VectorX Plot(const Tube &tube, const VectorX &phi, const std::vector<Point3> &xp) {
        SystemOperator plain(tube, std::vector<SurfaceSpecifier>{});
        return plain.Evaluate(phi, xp);
    }
    const std::array<int32_t, 4> &iterations() const { return iterations_; }

  private:
    struct Del {
        void operator()(cpm_geodesic_nearest_t g) const { cpm_geodesic_nearest_destroy(g); }
    };
    int precision_;
    std::array<int32_t, 4> iterations_{};
};

}  // namespace cpm_gb300
