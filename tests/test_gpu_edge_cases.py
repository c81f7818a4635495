"""Edge cases of the device path, as the reference meets them:

* a zero right-hand side: BiCGStab::Solve's loop never runs (src/BiCGStab.h:53-56),
  x = 0 at once;
* a non-finite one: a status, never a converged solve, and the other slots of
  the batch unaffected (the same bits as alone);
* ragged batches: fewer right-hand sides than slots, each as alone; more than
  the solver holds, an argument error;
* an evaluation point whose stencil leaves the tube: Tube::ComputeBasePoints
  throws (src/Tube.cpp:477-480), here CPM_ERR_BASEPOINT_OUTSIDE_TUBE;
* empty queries (zero points);
* the iteration cap: the reference returns silently after max_iterations
  (src/BiCGStab.h:107), here CPM_ERR_NOT_CONVERGED with the iterate so far;
* IBCs of different boundary orders in one operator, and a grid past 1024 nodes
  per axis: refused (CPM_ERR_UNSUPPORTED) before any solve."""
import math

import numpy as np
import pytest

from test_gpu_setup import two_circle_ibcs

pytestmark = pytest.mark.gpu

BREAKDOWN, NOT_CONVERGED, UNSUPPORTED, INVALID_ARG, OUTSIDE = -6, -5, -7, -1, -4


@pytest.fixture(scope="module")
def ibc_op(gpu):
    dx = 0.1
    T = gpu.Tube(gpu.desc(gpu.SPHERE, [1.0]), 3, dx)
    O = gpu.OpSet(T, two_circle_ibcs(gpu, dx))
    return T, O


def _rhs(O, rng, k):
    rows = O.rows()
    b = np.zeros((k, O.D))
    d = rows["kind"] == 2
    for j in range(k):
        v = rng.uniform(0, 1, 2)
        b[j, d] = v[rows["ibc"][d]]
    return b


@pytest.mark.parametrize("precision,kslots", [(0, 1), (0, 32), (1, 32)])
def test_zero_rhs_is_zero_at_once(gpu, ibc_op, precision, kslots):
    T, O = ibc_op
    b = np.zeros((kslots if kslots == 1 else 3, O.D))
    x, st = gpu.Solver(O, 0.0, -1.0, kslots=kslots).solve(b, precision=precision)
    assert np.array_equal(x, np.zeros_like(x))
    assert all(s["status"] == 0 and s["iterations"] == 0 for s in st), st


@pytest.mark.parametrize("precision", [0, 1])
def test_nonfinite_rhs_is_a_status_and_leaves_the_batch_alone(gpu, ibc_op, precision):
    T, O = ibc_op
    b = _rhs(O, np.random.default_rng(2), 3)
    b[1, 7] = np.nan
    b[2, 11] = np.inf
    sv = gpu.Solver(O, 0.0, -1.0, kslots=32)
    x, st = sv.solve(b, precision=precision, raise_on_error=False)
    assert st[0]["status"] == 0
    assert st[1]["status"] == BREAKDOWN and st[2]["status"] == BREAKDOWN
    xa, sa = sv.solve(b[:1], precision=precision)
    assert np.array_equal(x[0], xa[0])


def test_ragged_batches(gpu, ibc_op):
    T, O = ibc_op
    b = _rhs(O, np.random.default_rng(3), 5)
    sv = gpu.Solver(O, 0.0, -1.0, kslots=32)
    x, st = sv.solve(b, precision=1)
    assert len(st) == 5 and all(s["status"] == 0 for s in st)
    for j in (0, 4):
        xa, _ = sv.solve(b[j:j + 1], precision=1)
        assert np.array_equal(x[j], xa[0])
    with pytest.raises(RuntimeError):
        sv.solve(_rhs(O, np.random.default_rng(4), 33))
    with pytest.raises(RuntimeError):
        gpu.Solver(O, 0.0, -1.0).solve(b[:2])


def test_evaluation_point_off_the_tube_and_empty_queries(gpu, ibc_op):
    T, O = ibc_op
    with pytest.raises(RuntimeError) as e:
        O.plot_interp(np.array([[0.0, 0.0, 0.0]]))  # the sphere's centre: far inside, off the band
    assert e.value.code == OUTSIDE
    with pytest.raises(RuntimeError) as e:
        O.plot_interp_csr(np.array([[5.0, 0.0, 0.0]]))  # off the grid
    assert e.value.code == OUTSIDE
    cols, vals = O.plot_interp(np.zeros((0, 3)))
    assert cols.shape == (0, 64) and vals.shape == (0, 64)
    ptr, c, v = O.plot_interp_csr(np.zeros((0, 3)))
    assert ptr.tolist() == [0] and len(c) == 0 and len(v) == 0
    cp, dist = gpu.closest_points(gpu.desc(gpu.SPHERE, [1.0]), np.zeros((0, 3)))
    assert cp.shape == (0, 3) and dist.shape == (0,)


@pytest.mark.parametrize("precision", [0, 1])
def test_iteration_cap_is_a_status(gpu, ibc_op, precision):
    T, O = ibc_op
    b = _rhs(O, np.random.default_rng(5), 1)
    x, st = gpu.Solver(O, 0.0, -1.0, kslots=32).solve(b, precision=precision, max_iters=5, raise_on_error=False)
    assert st[0]["status"] == NOT_CONVERGED
    if precision == 0:
        assert st[0]["iterations"] == 5
    else:  # the capped mixed solve is solved again in FP64, under the same cap
        assert st[0]["fp64_fallback"] == 1 and 5 <= st[0]["iterations"] <= 10
    assert np.all(np.isfinite(x[0])) and np.any(x[0] != 0.0)


def test_mixed_boundary_orders_and_oversized_grids_are_refused(gpu):
    dx = 0.1
    T = gpu.Tube(gpu.desc(gpu.SPHERE, [1.0]), 3, dx)
    ibcs = [gpu.desc(gpu.CIRCLE3D, [math.sqrt(1 - z * z), 0, 0, z, 0, 0, 1], (-1.0, 1.0), boundary_order=o,
                     on_ibc_tolerance=0.1 * dx * dx) for z, o in ((0.3, 1), (-0.5, 2))]
    with pytest.raises(RuntimeError) as e:
        gpu.OpSet(T, ibcs)
    assert e.value.code == UNSUPPORTED
    with pytest.raises(RuntimeError) as e:
        gpu.Tube(gpu.desc(gpu.SPHERE, [1.0]), 3, 0.001)  # 2049 grid nodes per axis
    assert e.value.code == UNSUPPORTED
