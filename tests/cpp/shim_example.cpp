// Drives the C++ classes of include/cpm_ibc.hpp the way the reference's
// convergence studies drive cpm-ibc (Tube, Solver::Init/Solve,
// PoissonWithIBC::GetRHS/Solve, GeodesicDistance::ComputeDistance) and writes
// the solutions, in the reference's row layout, to a binary file:
//   int64 n, then n doubles, for each of: the screened Poisson solution, the two-circle
//   IBC Laplace FP64 and mixed solutions, geodesic distance, the nearest-node Poisson baselines,
//   the nearest-node geodesic distance and three plotted values of it, and three
//   HeatWithIBC steps (Crank-Nicolson, Dirichlet circle; backward Euler, Neumann circle).
#include <cmath>
#include <cstdio>
#include <vector>

#include "cpm_ibc.hpp"

using namespace cpm_gb300;

static void put(FILE *f, const VectorX &v) {
    int64_t n = (int64_t)v.size();
    fwrite(&n, sizeof(n), 1, f);
    fwrite(v.data(), sizeof(double), v.size(), f);
}

int main(int argc, char **argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: %s out.bin\n", argv[0]);
        return 2;
    }
    FILE *f = fopen(argv[1], "wb");
    if (!f) return 2;
    try {
        // screened Poisson -Delta_S u + u = 3z on the unit sphere, dx = 0.1 (exact u = z)
        SurfaceSpecifier sphere = SurfaceSpecifier::Sphere();
        Tube tube(sphere, 3, 0.1);
        SystemOperator op(tube, {});
        Solver sv;
        sv.Init(1.0, -1.0, op);
        VectorX b(op.rows());
        for (size_t r = 0; r < b.size(); ++r) b[r] = 3.0 * op.point(r)[2];
        VectorX u = sv.Solve(b);
        put(f, u);
        // Laplace with Dirichlet circles z = 0.3 (u = 1) and z = -0.5 (u = 0), dx = 0.05
        const double dx = 0.05;
        std::vector<SurfaceSpecifier> ibcs = {
            SurfaceSpecifier::Circle3D(std::sqrt(1 - 0.09), {0, 0, 0.3}, {0, 0, 1}, {-1, 1}).boundary_order(2).on_ibc_tolerance(0.1 * dx * dx),
            SurfaceSpecifier::Circle3D(std::sqrt(1 - 0.25), {0, 0, -0.5}, {0, 0, 1}, {-1, 1}).boundary_order(2).on_ibc_tolerance(0.1 * dx * dx)};
        PoissonWithIBC p(sphere, ibcs, dx);
        VectorX rhs = p.GetRHS([](const Point3 &) { return 0.0; },
                               [](size_t c, size_t, const Point3 &) { return c == 0 ? 1.0 : 0.0; });
        put(f, p.Solve(rhs));
        p.solver().SetPrecision(1);
        put(f, p.Solve(rhs));
        // heat-method geodesic distance from (0.36, 0.48, 0.8) on the sphere, dx = 0.1
        GeodesicDistance gd;
        put(f, gd.ComputeDistance(tube, {0.36, 0.48, 0.8}, 0.01));
        // nearest-node baselines on the same circles: solution, identity rows, right-hand side
        for (bool freeze : {false, true}) {
            PoissonWithIBCNearest pn(sphere, ibcs, dx, freeze);
            VectorX rn = pn.GetRHS([](const Point3 &) { return 0.0; }, [](const Point3 &x) { return x[2]; });
            put(f, pn.Solve(rn));
            VectorX id(rn.size());
            for (size_t r = 0; r < id.size(); ++r) id[r] = pn.GetIdentityRows()[r] ? 1.0 : 0.0;
            put(f, id);
            put(f, rn);
        }
        // GeodesicDistanceNearest from the closest point of reference row 100 (a point curve),
        // constraints built as examples/GeodesicDistanceBeetle/GeodesicDistanceBeetle.cpp:36-52
        {
            const std::vector<Point3> xs = tube.x(), cps = tube.cpx();
            const Point3 src = cps[100];
            auto dist = [](const Point3 &u, const Point3 &v) {
                double s = 0.0;
                for (size_t k = 0; k < 3; ++k) s += (u[k] - v[k]) * (u[k] - v[k]);
                return std::sqrt(s);
            };
            std::vector<std::vector<size_t>> con(1), ins(1);
            std::vector<std::vector<Scalar>> insd(1);
            Surface bc(SurfaceSpecifier::Point(src, {-1.0, 1.0}));
            std::vector<Point3> cpc;
            std::vector<Scalar> dc;
            bc.ClosestPoints(xs, cpc, dc);
            for (size_t i = 0; i < tube.nNodes(); ++i) {
                if (dist(cpc[i], cps[i]) < 1e-6) {
                    con[0].push_back(i);
                } else if (dist(xs[i], cpc[i]) < tube.TubeRadius()) {
                    ins[0].push_back(i);
                    insd[0].push_back(dist(xs[i], cpc[i]));
                }
            }
            GeodesicDistanceNearest gn;
            VectorX phin = gn.ComputeDistance(tube, con, ins, insd, 0.01);
            put(f, phin);
            put(f, GeodesicDistanceNearest::Plot(tube, phin, {Point3{0, 0, 1}, Point3{0.6, 0, 0.8}, Point3{-1, 0, 0}}));
        }
        // HeatWithIBC on the heat study's circles (HeatProblemsWithIBC.cpp:68-106, :307, :318),
        // dx = 0.1, u(0) = z, dt = 0.01, three steps each: Crank-Nicolson with the 2nd-order
        // Dirichlet circle (u = exp(-2t) z there), backward Euler with the zero-Neumann great circle
        {
            const double hdx = 0.1, hdt = 0.01;
            double nv[3] = {1.1, 1.234, 1.321};
            const double nn = std::sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
            for (double &v : nv) v /= nn;
            const double r = 0.27, th = 0.132, ph = 0.221;
            const double pop[3] = {r * std::cos(ph) * std::sin(th), r * std::sin(ph) * std::sin(th), r * std::cos(th)};
            const double rho = -(pop[0] * nv[0] + pop[1] * nv[1] + pop[2] * nv[2]);
            SurfaceSpecifier dcirc = SurfaceSpecifier::Circle3D(std::sqrt(1 - rho * rho), {rho * nv[0], rho * nv[1], rho * nv[2]},
                                                                {nv[0], nv[1], nv[2]}, {-1, 1})
                                         .boundary_order(2)
                                         .on_ibc_tolerance(0.1 * hdx * hdx);
            SurfaceSpecifier ncirc = SurfaceSpecifier::Circle3D(1.0, {0, 0, 0}, {0, 1, 0}, {-1, 1})
                                         .boundary_order(2)
                                         .boundary_type(1, 0)
                                         .on_ibc_tolerance(0.1 * hdx * hdx);
            for (int which = 0; which < 2; ++which) {
                HeatWithIBC heat(sphere, {which == 0 ? dcirc : ncirc}, hdx, hdt, which == 0 ? 2 : 1);
                VectorX u(heat.system().rows());
                for (size_t q = 0; q < u.size(); ++q) u[q] = heat.system().point(q)[2];
                for (int k = 1; k <= 3; ++k) {
                    const double t = k * hdt;
                    u = heat.TimeStep(u, [t](size_t, size_t, const Point3 &x) { return std::exp(-2.0 * t) * x[2]; });
                }
                put(f, u);
            }
        }
        printf("nodes %zu rows %zu ibc_dofs %zu iterations %d\n", tube.nNodes(), p.system().rows(),
               p.system().TotalIBCDOFs(), p.solver().stats().iterations);
    } catch (const std::exception &e) {
        fprintf(stderr, "error: %s\n", e.what());
        fclose(f);
        return 1;
    }
    fclose(f);
    return 0;
}
