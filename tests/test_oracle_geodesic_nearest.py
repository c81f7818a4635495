"""GeodesicDistanceNearest (problems/GeodesicDistanceNearest.cpp:11-345) in
the oracle.

The reference solves its heat step, the transposed implicit-Euler matrix with
identity rows at the constraint nodes, with a sparse LU (:123-133).  The
oracle restates that as a dense LU with partial pivoting (small tubes) and,
for the sizes the device tests use, as BiCGStab with 2000 damped Jacobi
sweeps per preconditioner call: the device's substitute for the direct
solve.  This file pins the substitute to the direct solve (relative l_inf
<= 1e-7 on phi at dx = 0.2) and checks the result against the exact
great-circle distance on the unit sphere.

Constraints are chosen as the reference's caller does
(examples/GeodesicDistanceBeetle/GeodesicDistanceBeetle.cpp:36-52) for a
point curve: constraint rows where the curve's closest point equals the
node's surface closest point (< 1e-6), inside rows where the node lies within
the tube radius of the curve, with that distance."""
import numpy as np
import pytest


def point_constraints(t, src, dx):
    """(constraint rows, inside rows, inside distances) of a point source, in the
    tube's row order, as the reference's caller builds them for a curve."""
    r = 1.0001 * np.sqrt(17.0) * dx
    dcp = np.linalg.norm(t["cp"] - src, axis=1)
    dxs = np.linalg.norm(t["x"] - src, axis=1)
    ibc = np.nonzero(dcp < 1e-6)[0]
    ins = np.nonzero((dcp >= 1e-6) & (dxs < r))[0]
    return ibc, ins, dxs[ins]


def _sphere_point(oracle, dx, seed):
    P = oracle.RefProblem(oracle.sphere_desc(), [], 3, dx)
    t = P.tube()
    src = t["cp"][np.random.default_rng(seed).integers(P.N)]
    return P, t, src


def test_nearest_geodesic_iterative_heat_step_matches_direct_solve(oracle):
    dx = 0.2
    P, t, src = _sphere_point(oracle, dx, 7)
    ibc, ins, dist = point_constraints(t, src, dx)
    assert len(ibc) == 1 and len(ins) > 100
    phd, itd = P.geodesic_nearest(ibc, ins, dist, dx * dx, 0)
    phj, itj = P.geodesic_nearest(ibc, ins, dist, dx * dx, 2000)
    assert np.max(np.abs(phd - phj)) <= 1e-7 * np.max(np.abs(phd))
    assert itd[0] == 0 and itj[0] >= 1
    # phi is 0 at the constraint node (its identity row) and the minimum there
    assert phd[ibc[0]] == 0.0 and np.min(phd) == 0.0


def test_nearest_geodesic_follows_great_circle_distance(oracle):
    """A single constraint node pins phi = 0 there while its neighbours carry the
    discrete point-source offset, so phi - exact is compared up to a constant."""
    dx = 0.1
    P, t, src = _sphere_point(oracle, dx, 7)
    ibc, ins, dist = point_constraints(t, src, dx)
    phi, its = P.geodesic_nearest(ibc, ins, dist, dx * dx, 2000)
    near = (np.abs(t["dist"]) < dx) & (np.arange(P.N) != ibc[0])
    exact = np.arccos(np.clip(t["cp"][near] @ src, -1, 1))
    e = phi[near] - exact
    e -= np.median(e)
    assert np.mean(np.abs(e)) < 0.03 and np.max(np.abs(e)) < 0.1
    assert its[0] >= 1 and all(i > 0 for i in its[1:])


def test_nearest_heat_matrix_matches_sparse_lu_of_scipy_assembly(oracle):
    """The transposed implicit-Euler heat matrix assembled independently with
    scipy.sparse from the oracle's L and E, its constraint rows set to identity
    rows, and solved by SuperLU (a sparse LU, as the reference's SparseLU):
    equal to the oracle's dense-LU heat solution within 1e-10, and to its
    Jacobi-preconditioned BiCGStab solution within 1e-8 (relative l_inf)."""
    sp = pytest.importorskip("scipy.sparse")
    spla = pytest.importorskip("scipy.sparse.linalg")
    dx = 0.2
    P, t, src = _sphere_point(oracle, dx, 7)
    ibc, ins, dist = point_constraints(t, src, dx)
    dt = dx * dx
    N = P.N
    Lm = sp.csr_matrix(tuple(reversed(P.csr(2))), shape=(N, N))
    Em = sp.csr_matrix(tuple(reversed(P.csr(3))), shape=(N, N))
    dL = sp.diags(Lm.diagonal())
    A = sp.identity(N, format="csr") - dt * (dL + (Lm - dL) @ Em)
    Ar = A.T.tolil()
    for k in ibc:
        Ar.rows[k] = [int(k)]
        Ar.data[k] = [1.0]
    scale = np.arctanh(1 - dx) / P.radius
    smooth = lambda s: 0.5 * np.tanh(-scale * s) + 0.5
    rhs = np.zeros(N)
    rhs[ibc] = smooth(-np.linalg.norm(t["x"][ibc] - t["cp"][ibc], axis=1))
    rhs[ins] = smooth(-dist)
    u = spla.spsolve(Ar.tocsc(), rhs)
    ud = P.heat_nearest(ibc, ins, dist, dt, 0)
    uj = P.heat_nearest(ibc, ins, dist, dt, 2000)
    assert np.max(np.abs(ud - u)) <= 1e-10 * np.max(np.abs(u))
    assert np.max(np.abs(uj - u)) <= 1e-8 * np.max(np.abs(u))
