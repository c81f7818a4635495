"""GeodesicDistanceNearest on the device against the oracle.

The device solves the heat step (the transposed implicit-Euler matrix with
identity rows at the constraint nodes) by BiCGStab with 2000 damped Jacobi
sweeps per preconditioner call and an E^T gather over the base groups; the
oracle solves the same matrix assembled explicitly, directly (dense LU, as
the reference's SparseLU) at dx = 0.2 and by the same iteration at dx = 0.1.
Tolerance: relative l_inf <= 1e-7 on phi over the tube rows (four chained
solves to 1e-10 residual each, with a gradient normalisation in between);
mixed precision (FP32 Poisson steps with FP64 reliable updates) within 1e-8
of the FP64 device path."""
import numpy as np
import pytest

from test_gpu_setup import ref_to_gpu_index
from test_oracle_geodesic_nearest import point_constraints

pytestmark = pytest.mark.gpu


def _setup(gpu, oracle, dx, seed=7):
    P = oracle.RefProblem(oracle.sphere_desc(), [], 3, dx, record_visited=True)
    t = P.tube()
    src = t["cp"][np.random.default_rng(seed).integers(P.N)]
    T = gpu.Tube.from_closest_points(gpu.desc(gpu.SPHERE, [1.0]), 3, dx, *P.visited())
    m = ref_to_gpu_index(t["rec"], T.export()["rec"])
    return P, t, T, m, src


@pytest.mark.parametrize("dx,sweeps", [(0.2, 0), (0.1, 2000)])
def test_nearest_geodesic_matches_oracle(gpu, oracle, dx, sweeps):
    P, t, T, m, src = _setup(gpu, oracle, dx)
    ibc, ins, dist = point_constraints(t, src, dx)
    ref, its_ref = P.geodesic_nearest(ibc, ins, dist, dx * dx, sweeps)
    G = gpu.GeodesicNearest(T, m[ibc], m[ins], dist)
    phi, its = G.run(dx * dx, precision=0)
    assert np.max(np.abs(phi[m] - ref)) <= 1e-7 * np.max(np.abs(ref))
    assert phi[m[ibc[0]]] == 0.0
    if sweeps:
        assert its[0] == its_ref[0]


def test_nearest_geodesic_mixed_precision_matches_fp64(gpu, oracle):
    dx = 0.1
    P, t, T, m, src = _setup(gpu, oracle, dx, seed=11)
    ibc, ins, dist = point_constraints(t, src, dx)
    G = gpu.GeodesicNearest(T, m[ibc], m[ins], dist)
    phi64, its64 = G.run(dx * dx, precision=0)
    phi32, its32 = G.run(dx * dx, precision=1)
    assert its32[0] == its64[0]  # the heat step is FP64 in both
    assert np.max(np.abs(phi32 - phi64)) <= 1e-8 * np.max(np.abs(phi64))


def test_nearest_geodesic_rejects_rows_outside_the_tube(gpu, oracle):
    P, t, T, m, src = _setup(gpu, oracle, 0.2)
    with pytest.raises(RuntimeError):
        gpu.GeodesicNearest(T, [T.N], [], [])
    with pytest.raises(RuntimeError):
        gpu.GeodesicNearest(T, [0], [-1], [0.1])
