"""Triangle-mesh surfaces and polyline IBCs on the device against the oracle.

The reference queries mesh and polyline closest points through fcpw (a float
BVH that is not vendored); the oracle computes them exactly in FP64 (Ericson's
point-triangle and point-segment closest points), so the device's closest
points are checked against that (<= 1e-12) and the rest of the pipeline is
bit-exact given the oracle's closest points, as for the analytic surfaces.

Tolerances: closest points and distances <= 1e-12; tube, base points, weights,
IBC subsets and operator rows bit-exact given the same closest points; FP64
solve <= 1e-10 relative l_inf of the oracle's, both solved to relative
residual 1e-12; mixed precision <= 1e-8."""
import numpy as np
import pytest

import studies as S
from test_gpu_parity_c2 import assert_rows_bit_exact, same_cp_pair
from test_gpu_setup import ref_to_gpu_index
from cpm_gb300 import workloads as W

pytestmark = pytest.mark.gpu

DX = 0.04


def _mesh(level=4, seed=3):
    v, f = W.perturbed_icosphere(level, seed=seed)
    return v, f, W.mesh_bbox(v)


def _descs(gpu, oracle, v, f, bb):
    return (oracle.make_desc(oracle.TRIANGULATION, (), bb, verts=v, prims=f),
            gpu.desc(gpu.TRIANGULATION, (), bb, verts=v, prims=f))


def _curves(mod, v, f, bb, n, dx):
    curves, _ = W.parallel_plane_curves(v, f, n, seed=4, spread=0.6)
    mk = mod.make_desc if hasattr(mod, "make_desc") else mod.desc
    return [mk(mod.POLYLINE, (), bb, boundary_order=2, on_ibc_tolerance=0.1 * dx * dx, verts=p, prims=s) for p, s in curves]


def test_mesh_tube_bit_exact_given_same_closest_points(gpu, oracle):
    v, f, bb = _mesh()
    od, gd = _descs(gpu, oracle, v, f, bb)
    P = oracle.RefProblem(od, [], 3, DX, record_visited=True)
    T = gpu.Tube.from_closest_points(gd, 3, DX, *P.visited())
    ref, g = P.tube(), T.export()
    assert T.N == P.N and T.n_visited == P.n_visited and T.xstart == P.xstart
    assert np.array_equal(np.sort(g["rec"]), np.sort(ref["rec"]))
    m = ref_to_gpu_index(ref["rec"], g["rec"])
    assert np.array_equal(g["cp"][m], ref["cp"])
    assert np.array_equal(g["bpt"][m], ref["rec"][ref["bpt"]])
    assert np.array_equal(g["w"][m], P.weights())


def test_mesh_device_closest_points_match_oracle(gpu, oracle):
    v, f, bb = _mesh()
    od, gd = _descs(gpu, oracle, v, f, bb)
    T = gpu.Tube(gd, 3, DX)
    g = T.export()
    cp, dist = oracle.closest_points(od, g["x"])
    assert np.max(np.abs(g["cp"] - cp)) <= 1e-12
    assert np.max(np.abs(g["dist"] - dist)) <= 1e-12
    # membership equals the oracle's except for nodes within rounding of the band edge
    P = oracle.RefProblem(od, [], 3, DX)
    ref = P.tube()
    sym = np.setxor1d(g["rec"], ref["rec"])
    assert len(sym) <= 2
    if len(sym):
        n1 = P.N1d
        idx = np.stack([sym // (n1 * n1), (sym // n1) % n1, sym % n1], 1)
        x = P.xstart + idx * DX
        _, d = oracle.closest_points(od, x)
        assert np.all(np.abs(np.abs(d) - T.radius) < 1e-12)


def test_polyline_ibcs_on_mesh_match_oracle(gpu, oracle):
    v, f, bb = _mesh()
    od, gd = _descs(gpu, oracle, v, f, bb)
    P, T, O, gr = same_cp_pair(gpu, oracle, DX, _curves(oracle, v, f, bb, 2, DX), _curves(gpu, v, f, bb, 2, DX),
                               surface=(od, gd))
    ref, g = P.tube(), T.export()
    assert O.D == P.D and O.total_ibc_dofs == P.total_ibc_dofs
    for c in range(2):
        rs, gs = P.ibc_subsets(c), O.ibc_subsets(c)
        assert np.array_equal(g["rec"][gs["tag_set"]], ref["rec"][rs["tag_set"]])
        assert np.array_equal(g["rec"][gs["dof_set"]], ref["rec"][rs["dof_set"]])
    for which in (0, 1):
        assert_rows_bit_exact(P, O, gr, which)
    # diffusion-curves Laplace, one right-hand side per colour channel
    rows = P.rows()
    rgb = np.random.default_rng(8).uniform(0, 1, size=(2, 3))
    B = [S.build_rhs(rows, lambda x: np.zeros(len(x)), lambda c, x, ch=ch: np.full(len(x), rgb[c, ch]))
         for ch in range(3)]
    Bg = np.zeros((3, O.D))
    for ch in range(3):
        Bg[ch][gr] = B[ch]
    solver = gpu.Solver(O, 0.0, -1.0, kslots=32)
    X64, st = solver.solve(Bg, tol=1e-12, precision=0)
    X32, st32 = solver.solve(Bg, tol=1e-10, precision=1)
    for ch in range(3):
        x_ref, _ = P.solve(0.0, -1.0, B[ch], tol=1e-12)
        scale = np.max(np.abs(x_ref))
        assert st[ch]["status"] == 0 and st32[ch]["status"] == 0
        assert np.max(np.abs(X64[ch][gr] - x_ref)) / scale <= 1e-10
        assert np.max(np.abs(X32[ch][gr] - x_ref)) / scale <= 1e-8
