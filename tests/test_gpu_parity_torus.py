"""Parity at the torus geodesic configuration's size: the torus R = 1, r = 0.4 at
dx = 0.01 (1,306,164 tube nodes) with Dirichlet IBCs on its outer and inner
equators (order 2), the device built from the oracle's closest points.

Checked: tube membership, node order, closest points and weights bit-exact; IBC
tagging and DOF subsets bit-exact; every Lfull and Efull row bit-exact; the plain
FP64 GPU solve within 1e-10 relative l_inf of the oracle's, both solved to a
relative residual of 1e-12."""
import numpy as np
import pytest

import studies as S
from test_gpu_parity_c2 import _rel_inf, assert_rows_bit_exact, same_cp_pair

pytestmark = pytest.mark.gpu

DX = 0.01
BB = (-1.4, 1.4)


def _equators(mod, dx):
    if hasattr(mod, "circle3d_desc"):
        return [mod.circle3d_desc(R, (0, 0, 0), (0, 0, 1), dx, 2, BB) for R in (1.4, 0.6)]
    return [mod.desc(mod.CIRCLE3D, [R, 0, 0, 0, 0, 0, 1], BB, boundary_order=2, on_ibc_tolerance=0.1 * dx * dx)
            for R in (1.4, 0.6)]


@pytest.fixture(scope="module")
def torus(gpu, oracle):
    return same_cp_pair(gpu, oracle, DX, _equators(oracle, DX), _equators(gpu, DX),
                        surface=(oracle.torus_desc(1.0, 0.4, BB), gpu.desc(gpu.TORUS, [1.0, 0.4], BB)))


def test_torus_tube_and_subsets_bit_exact(torus):
    P, T, O, gr = torus
    ref, g = P.tube(), T.export()
    assert T.N == P.N == 1306164 and T.N1d == P.N1d and T.xstart == P.xstart and T.radius == P.radius
    m = gr[:P.N]
    assert np.array_equal(g["rec"][m], ref["rec"])
    assert np.array_equal(g["cp"][m], ref["cp"])
    assert np.array_equal(g["w"][m], P.weights())
    assert O.D == P.D and O.total_ibc_dofs == P.total_ibc_dofs and O.num2 == P.num2
    for c in range(2):
        rs, gs = P.ibc_subsets(c), O.ibc_subsets(c)
        assert np.array_equal(g["rec"][gs["tag_set"]], ref["rec"][rs["tag_set"]])
        assert np.array_equal(g["rec"][gs["dof_set"]], ref["rec"][rs["dof_set"]])
        assert np.array_equal(gs["dof_cp"], rs["dof_cp"])
        assert gs["col_start"] == rs["col_start"] and gs["dcol_start"] == rs["dcol_start"]


@pytest.mark.parametrize("which", [0, 1])
def test_torus_operator_rows_bit_exact(torus, which):
    """every Lfull (which 0) and Efull (which 1, 92 M entries) row equals the oracle's"""
    P, T, O, gr = torus
    assert_rows_bit_exact(P, O, gr, which)


def test_torus_plain_fp64_solve_within_1e10(gpu, torus):
    P, T, O, gr = torus
    rows = P.rows()
    vals = np.random.default_rng(37).uniform(0, 1, 2)
    b = S.build_rhs(rows, lambda x: np.zeros(len(x)), lambda c, x: np.full(len(x), vals[c]))
    x_ref, _ = P.solve(0.0, -1.0, b, tol=1e-12)
    bg = np.empty(O.D)
    bg[gr] = b
    x_gpu, st = gpu.Solver(O, 0.0, -1.0).solve(bg, tol=1e-12, precision=0)
    assert st[0]["status"] == 0 and st[0]["rel_residual"] <= 1e-12
    assert _rel_inf(x_gpu[0][gr], x_ref) <= 1e-10
