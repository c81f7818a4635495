"""The C++ classes of include/cpm_ibc.hpp (reference names over the C-ABI).

CPU: the header and the example compile.  GPU: the example's solutions, which
the classes return in the reference's row layout (breadth-first tube node
numbering), equal the oracle's vectors entry by entry, with no permutation:
screened Poisson on the sphere and the two-circle IBC Laplace (FP64) within
1e-8 relative l_inf (the device computes its own closest points, which differ
from glibc's by ulps), mixed precision within 1e-8 of the FP64 run, and the
geodesic and the nearest-node geodesic within 1e-6 of the oracle's, and three
HeatWithIBC time steps (Crank-Nicolson with a Dirichlet circle, backward Euler
with a zero-Neumann circle) within 1e-8."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import studies as S
from test_gpu_setup import two_circle_ibcs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "shim_example.cpp")


def _gxx():
    g = shutil.which("g++")
    if not g:
        pytest.skip("g++ not found")
    return g


def test_shim_header_compiles():
    subprocess.run([_gxx(), "-std=c++17", "-Wall", "-Werror", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), SRC],
                   check=True)


def _read(path):
    out = []
    with open(path, "rb") as f:
        while True:
            n = np.fromfile(f, dtype=np.int64, count=1)
            if len(n) == 0:
                return out
            out.append(np.fromfile(f, dtype=np.float64, count=int(n[0])))


@pytest.mark.gpu
def test_shim_example_matches_oracle(gpu, oracle, tmp_path):
    libdir = os.path.join(ROOT, "cpm-ibc_gb300", "_build")
    exe = str(tmp_path / "shim_example")
    subprocess.run([_gxx(), "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-L", libdir, "-lcpmgpu",
                    f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    out = str(tmp_path / "out.bin")
    subprocess.run([exe, out], check=True)
    c1, c2, c2m, geo, n_u, n_id, n_b, f_u, f_id, f_b, gn, gn_plot, heat_cn, heat_be_neu = _read(out)
    # screened Poisson on the sphere, dx = 0.1
    P1 = oracle.RefProblem(oracle.sphere_desc(), [], 3, 0.1)
    b1 = 3.0 * P1.rows()["point"][:, 2]
    x1, _ = P1.solve(1.0, -1.0, b1)
    assert len(c1) == P1.D
    assert np.max(np.abs(c1 - x1)) / np.max(np.abs(x1)) <= 1e-8
    # Laplace with the two circle IBCs at dx = 0.05
    P2 = oracle.RefProblem(oracle.sphere_desc(), two_circle_ibcs(oracle, 0.05), 3, 0.05)
    b2 = S.build_rhs(P2.rows(), lambda x: np.zeros(len(x)), lambda c, x: np.full(len(x), 1.0 if c == 0 else 0.0))
    x2, _ = P2.solve(0.0, -1.0, b2)
    assert len(c2) == P2.D
    assert np.max(np.abs(c2 - x2)) / np.max(np.abs(x2)) <= 1e-8
    assert np.max(np.abs(c2m - c2)) / np.max(np.abs(c2)) <= 1e-8
    # geodesic from (0.36, 0.48, 0.8), a point off the grid planes
    Pg = oracle.RefProblem(oracle.sphere_desc(), [oracle.point_desc((0.36, 0.48, 0.8), 0.1)], 3, 0.1)
    pg, _ = Pg.geodesic(0.01, 2000)
    assert len(geo) == Pg.D
    assert np.max(np.abs(geo - pg)) / np.max(np.abs(pg)) <= 1e-6
    # nearest-node baselines: identity rows at the DOF subsets' nodes (as many as the IBC
    # DOFs) or at the nodes nearest the circles' 100 plot points each, holding their values
    assert len(n_u) == P2.N and int(n_id.sum()) == P2.total_ibc_dofs
    assert 0 < int(f_id.sum()) <= 200
    for u, ident, b in ((n_u, n_id, n_b), (f_u, f_id, f_b)):
        m = ident > 0
        assert np.max(np.abs(u[m] - b[m])) <= 1e-12
        assert np.all(np.abs(b[m]) <= 1.0) and np.all(b[~m] == 0.0)
    # nearest-node geodesic from the closest point of row 100, same constraint rule as the example
    P1n = oracle.RefProblem(oracle.sphere_desc(), [], 3, 0.1)
    t1 = P1n.tube()
    src = t1["cp"][100]
    dcp = np.linalg.norm(t1["cp"] - src, axis=1)
    dxs = np.linalg.norm(t1["x"] - src, axis=1)
    con = np.nonzero(dcp < 1e-6)[0]
    ins = np.nonzero((dcp >= 1e-6) & (dxs < P1n.radius))[0]
    ref, _ = P1n.geodesic_nearest(con, ins, dxs[ins], 0.01, 2000)
    assert len(gn) == P1n.N
    assert np.max(np.abs(gn - ref)) / np.max(np.abs(ref)) <= 1e-6
    assert len(gn_plot) == 3 and np.all(np.isfinite(gn_plot)) and np.all(gn_plot >= -0.1)
    # HeatWithIBC::TimeStep (problems/HeatWithIBC.cpp:104-132): three Crank-Nicolson steps with the
    # Dirichlet circle and three backward-Euler steps with the zero-Neumann circle, dx = 0.1, dt = 0.01
    for got, bt, method in ((heat_cn, 0, 2), (heat_be_neu, 1, 1)):
        R, c, n = S.heat_circle_params(boundary_type=bt)
        ibc = oracle.circle3d_desc(R, c, n, 0.1, boundary_order=2)
        ibc.boundary_type[0] = bt
        Ph = oracle.RefProblem(oracle.sphere_desc(), [ibc], 3, 0.1)
        rows = Ph.rows()
        u = rows["point"][:, 2].copy()
        dirichlet = rows["kind"] == 2
        for k in range(1, 4):
            t = k * 0.01
            if method == 2:
                u = Ph.apply(1.0, 0.5 * 0.01, u)
            u = np.array(u, copy=True)
            u[dirichlet] = np.exp(-2 * t) * rows["point"][dirichlet, 2]
            u, _ = Ph.solve(1.0, -(0.5 if method == 2 else 1.0) * 0.01, u)
        assert len(got) == Ph.D
        assert np.max(np.abs(got - u)) / np.max(np.abs(u)) <= 1e-8
