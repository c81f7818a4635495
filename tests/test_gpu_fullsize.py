"""The configurations at full size, through properties that hold at any size
(the oracle finishes only the small cases in seconds):

* The sphere with two circle IBCs at dx = 0.025 (215,662 rows): the
  batched mixed-precision solve is linear in the right-hand side (solve(a b1 +
  b2) = a solve(b1) + solve(b2), within the solver tolerance) and equals the
  FP64 solves (<= 1e-8 relative l_inf).
* The torus R = 1, r = 0.4 at dx = 0.01 (1.31 M nodes): the heat-method
  geodesic distance from a tube node's closest point is >= 0 up to the
  discretisation error, smallest at the source, and orders the points near the
  source as the chord length does (geodesic and Euclidean distances agree to
  second order there; the heat method's own error near a point source is
  10 - 30 %, so the order, not the value, is checked: rank correlation >= 0.85
  within chord 0.2, where no chord crosses the tube of minor radius 0.4).
* The perturbed icosphere at level 7 (327,680 triangles) with 16 polyline
  IBCs at dx = 0.005: device closest points equal the oracle's exact FP64
  point-triangle closest points on a sample of tube nodes (<= 1e-12), and the
  3-RHS mixed solve equals the FP64 solves (<= 1e-8)."""
import numpy as np
import pytest

from cpm_gb300 import workloads as W
from test_gpu_setup import two_circle_ibcs

pytestmark = pytest.mark.gpu


def test_two_circle_sphere_full_size_linearity_and_fp64_agreement(gpu):
    dx = 0.025
    O = gpu.OpSet(gpu.Tube(gpu.desc(gpu.SPHERE, [1.0]), 3, dx), two_circle_ibcs(gpu, dx))
    rows = O.rows()
    d = rows["kind"] == 2
    rng = np.random.default_rng(21)
    B = np.zeros((3, O.D))
    for j in range(2):
        B[j][d] = rng.uniform(0, 1, 2)[rows["ibc"][d]]
    a = 0.37
    B[2] = a * B[0] + B[1]
    X, st = gpu.Solver(O, 0.0, -1.0, kslots=32).solve(B, tol=1e-10, precision=1)
    assert all(s["status"] == 0 for s in st)
    scale = np.max(np.abs(X[2]))
    assert np.max(np.abs(X[2] - (a * X[0] + X[1]))) <= 1e-8 * scale
    S1 = gpu.Solver(O, 0.0, -1.0, kslots=1)
    for j in range(3):
        x64, _ = S1.solve(B[j], tol=1e-10, precision=0)
        assert np.max(np.abs(X[j] - x64[0])) <= 1e-8 * np.max(np.abs(x64[0]))


def test_torus_full_size_geodesic_near_source(gpu):
    dx = 0.01
    T = gpu.Tube(gpu.desc(gpu.TORUS, [1.0, 0.4], (-1.4, 1.4)), 3, dx)
    g = T.export()
    src = g["cp"][np.random.default_rng(12).integers(T.N)]
    phi, _ = gpu.Geodesic(T, src).run(dx * dx, precision=0)
    phi = phi[:T.N]
    assert np.min(phi) >= -2 * dx
    chord = np.linalg.norm(g["cp"] - src, axis=1)
    assert chord[np.argmin(phi)] < 5 * dx
    near = chord < 0.2
    assert near.sum() > 1000
    rank = lambda a: np.argsort(np.argsort(a)).astype(np.float64)
    assert np.corrcoef(rank(phi[near]), rank(chord[near]))[0, 1] >= 0.85


def test_mesh_full_size_closest_points_and_solves(gpu, oracle):
    dx = 0.005
    v, f = W.perturbed_icosphere(7, seed=3)
    bb = W.mesh_bbox(v)
    T = gpu.Tube(gpu.desc(gpu.TRIANGULATION, (), bb, verts=v, prims=f), 3, dx)
    g = T.export()
    sample = np.random.default_rng(5).choice(T.N, 400, replace=False)
    cp, dist = oracle.closest_points(oracle.make_desc(oracle.TRIANGULATION, (), bb, verts=v, prims=f), g["x"][sample])
    assert np.max(np.abs(g["cp"][sample] - cp)) <= 1e-12
    assert np.max(np.abs(g["dist"][sample] - dist)) <= 1e-12
    curves, _ = W.parallel_plane_curves(v, f, 16, seed=4)
    O = gpu.OpSet(T, [gpu.desc(gpu.POLYLINE, (), bb, boundary_order=2, on_ibc_tolerance=0.1 * dx * dx, verts=p,
                               prims=s) for p, s in curves])
    rows = O.rows()
    d = rows["kind"] == 2
    rgb = np.random.default_rng(9).uniform(0, 1, (16, 3))
    B = np.zeros((3, O.D))
    for ch in range(3):
        B[ch][d] = rgb[rows["ibc"][d], ch]
    X, st = gpu.Solver(O, 0.0, -1.0, kslots=32).solve(B, tol=1e-10, precision=1)
    assert all(s["status"] == 0 for s in st)
    S1 = gpu.Solver(O, 0.0, -1.0, kslots=1)
    for ch in range(3):
        x64, _ = S1.solve(B[ch], tol=1e-10, precision=0)
        assert np.max(np.abs(X[ch] - x64[0])) <= 1e-8 * np.max(np.abs(x64[0]))
