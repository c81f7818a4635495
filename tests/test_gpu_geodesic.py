"""Heat-method geodesic distance (GeodesicDistance::ComputeDistance) on the
device against the oracle restatement, and against the exact great-circle
distance on the unit sphere.

Both sides precondition the heat step with 2000 damped Jacobi sweeps per
preconditioner call, as problems/GeodesicDistance.cpp:117-119 does.

Tolerances: device FP64 vs oracle, relative l_inf over the tube rows <= 1e-7
(four chained solves to 1e-10 residual each, with a gradient normalisation in
between); distance error vs the exact great-circle distance at the closest
points of near-surface nodes: mean < 0.05, max < 0.1 (first-order heat method
at dx = 0.1); mixed precision (FP32 Poisson steps with FP64 reliable
updates) vs the FP64 device path <= 1e-8 relative at dx = 0.05."""
import numpy as np
import pytest

from test_gpu_setup import ref_to_gpu_index

pytestmark = pytest.mark.gpu


def _setup(gpu, oracle, dx, seed=7):
    P0 = oracle.RefProblem(oracle.sphere_desc(), [], 3, dx, record_visited=True)
    t0 = P0.tube()
    rng = np.random.default_rng(seed)
    src = t0["cp"][rng.integers(P0.N)]
    P = oracle.RefProblem(oracle.sphere_desc(), [oracle.point_desc(src, dx, boundary_order=1)], 3, dx)
    T = gpu.Tube.from_closest_points(gpu.desc(gpu.SPHERE, [1.0]), 3, dx, *P0.visited())
    return P, T, src


def test_geodesic_matches_oracle(gpu, oracle):
    dx = 0.1
    P, T, src = _setup(gpu, oracle, dx)
    phi_ref, its_ref = P.geodesic(dx * dx, 2000)
    G = gpu.Geodesic(T, src)
    assert G.D == P.D
    phi, its = G.run(dx * dx, precision=0)
    ref, g = P.tube(), T.export()
    m = ref_to_gpu_index(ref["rec"], g["rec"])
    a, b = phi[m], phi_ref[:P.N]
    assert np.max(np.abs(a - b)) / np.max(np.abs(b)) <= 1e-7
    # IBC DOF rows follow the reference's layout exactly
    assert np.max(np.abs(phi[P.N:] - phi_ref[P.N:])) <= 1e-7 * np.max(np.abs(b))
    assert its[0] == its_ref[0]
    # exact great-circle distance at the closest points of nodes near the surface
    near = np.abs(ref["dist"]) < dx
    exact = np.arccos(np.clip(ref["cp"][near] @ src, -1, 1))
    err = np.abs(b[near] - exact)
    assert np.mean(err) < 0.05
    assert np.max(err) < 0.1


def test_geodesic_mixed_precision_matches_fp64(gpu, oracle):
    dx = 0.05
    P, T, src = _setup(gpu, oracle, dx, seed=11)
    G = gpu.Geodesic(T, src)
    phi64, its64 = G.run(dx * dx, precision=0, tol=1e-10)
    phi32, its32 = G.run(dx * dx, precision=1, tol=1e-10)
    assert its32[0] == its64[0]  # the heat step is FP64 in both
    assert np.max(np.abs(phi32 - phi64)) / np.max(np.abs(phi64)) <= 1e-8
    # both are within the heat method's own discretisation error of the exact distance
    t0 = P.tube()
    m = ref_to_gpu_index(t0["rec"], T.export()["rec"])
    near = np.abs(t0["dist"]) < dx
    exact = np.arccos(np.clip(t0["cp"][near] @ src, -1, 1))
    err = np.abs(phi32[m][near] - exact)
    assert np.mean(err) < 0.01 and np.max(err) < 0.02


def test_geodesic_batch_equals_one_source_runs(gpu):
    """cpm_geodesic_batch: three sources on one operator, each slot carrying only its
    own point IBC, against cpm_geodesic_run of each source alone (FP64 both):
    relative l_inf <= 1e-8 over the tube rows and the source's DOF rows."""
    dx = 0.1
    T = gpu.Tube(gpu.desc(gpu.SPHERE, [1.0]), 3, dx)
    cp = T.export()["cp"]
    rng = np.random.default_rng(21)
    src = cp[rng.choice(T.N, 3, replace=False)]
    B = gpu.GeodesicBatch(T, src)
    phib, itsb = B.run(dx * dx)
    for k in range(3):
        G = gpu.Geodesic(T, src[k])
        phi, its = G.run(dx * dx, precision=0)
        assert np.max(np.abs(phib[k][:G.D] - phi)) <= 1e-8 * np.max(np.abs(phi))
        assert np.all(phib[k][G.D:] == 0.0)  # the rows of other sources' DOFs
        assert abs(int(itsb[k][0]) - its[0]) <= 1
