"""Device tube / weights / IBC subsets against the oracle.

Bit-exact given the same closest points (the tube is built from the oracle's
closest points through cpm_tube_build_from_cp), and within 1e-14 for the
device's own closest points (CUDA's libm may differ from glibc by an ulp)."""
import math

import numpy as np
import pytest

import studies as S

pytestmark = pytest.mark.gpu


def ref_to_gpu_index(ref_rec, gpu_rec):
    o = np.argsort(gpu_rec)
    pos = np.searchsorted(gpu_rec[o], ref_rec)
    assert np.all(gpu_rec[o][pos] == ref_rec)
    return o[pos]


@pytest.mark.parametrize("kind,dx", [("sphere", 0.1), ("sphere", 0.05), ("torus", 0.05)])
def test_tube_bit_exact_given_same_closest_points(gpu, oracle, kind, dx):
    if kind == "sphere":
        od, gd = oracle.sphere_desc(), gpu.desc(gpu.SPHERE, [1.0], (-1.0, 1.0))
    else:
        od, gd = oracle.torus_desc(1.0, 0.4, (-1.4, 1.4)), gpu.desc(gpu.TORUS, [1.0, 0.4], (-1.4, 1.4))
    P = oracle.RefProblem(od, [], 3, dx, record_visited=True)
    rec, cp, dist = P.visited()
    T = gpu.Tube.from_closest_points(gd, 3, dx, rec, cp, dist)
    ref = P.tube()
    g = T.export()
    assert T.N == P.N and T.N1d == P.N1d
    assert T.n_visited == P.n_visited
    assert T.xstart == P.xstart and T.radius == P.radius
    # membership
    assert np.array_equal(np.sort(g["rec"]), np.sort(ref["rec"]))
    m = ref_to_gpu_index(ref["rec"], g["rec"])
    # grid coordinates and closest points
    assert np.array_equal(g["x"][m], ref["x"])
    assert np.array_equal(g["cp"][m], ref["cp"])
    # base points (as grid keys) bit-exact
    assert np.array_equal(g["bpt"][m], ref["rec"][ref["bpt"]])
    # tricubic weights bit-exact
    assert np.array_equal(g["w"][m], P.weights())
    # neighbours, mapped to reference indices
    inv = np.empty(T.N, np.int64)
    inv[m] = np.arange(T.N)
    gn = g["nbr"][m]
    gn_ref = np.where(gn >= 0, inv[np.maximum(gn, 0)], -1)
    assert np.array_equal(gn_ref, ref["nbr"])


@pytest.mark.parametrize("kind,dx", [("sphere", 0.1), ("sphere", 0.05), ("torus", 0.05)])
def test_reference_node_order(gpu, oracle, kind, dx):
    """cpm_tube_reference_order reproduces the reference's BFS tube numbering."""
    if kind == "sphere":
        od, gd = oracle.sphere_desc(), gpu.desc(gpu.SPHERE, [1.0], (-1.0, 1.0))
    else:
        od, gd = oracle.torus_desc(1.0, 0.4, (-1.4, 1.4)), gpu.desc(gpu.TORUS, [1.0, 0.4], (-1.4, 1.4))
    P = oracle.RefProblem(od, [], 3, dx, record_visited=True)
    T = gpu.Tube.from_closest_points(gd, 3, dx, *P.visited())
    assert np.array_equal(T.export()["rec"][T.reference_order()], P.tube()["rec"])


@pytest.mark.parametrize("kind,dx", [("sphere", 0.1), ("torus", 0.05)])
def test_device_closest_points_match_oracle(gpu, oracle, kind, dx):
    if kind == "sphere":
        od, gd = oracle.sphere_desc(), gpu.desc(gpu.SPHERE, [1.0], (-1.0, 1.0))
    else:
        od, gd = oracle.torus_desc(1.0, 0.4, (-1.4, 1.4)), gpu.desc(gpu.TORUS, [1.0, 0.4], (-1.4, 1.4))
    P = oracle.RefProblem(od, [], 3, dx)
    T = gpu.Tube(gd, 3, dx)
    ref, g = P.tube(), T.export()
    assert np.array_equal(np.sort(g["rec"]), np.sort(ref["rec"]))
    m = ref_to_gpu_index(ref["rec"], g["rec"])
    assert np.max(np.abs(g["cp"][m] - ref["cp"])) < 1e-14
    assert np.max(np.abs(g["dist"][m] - ref["dist"])) < 1e-14
    # base points: floor((cp - xstart)/dx) can only differ where a closest-point
    # coordinate lies within rounding of a grid plane
    diff = g["bpt"][m] != ref["rec"][ref["bpt"]]
    f = (ref["cp"][diff] - P.xstart) / dx
    assert np.all(np.min(np.abs(f - np.round(f)), axis=1) < 1e-9)
    assert diff.sum() <= max(2, P.N // 1000)
    w_ok = ~diff
    assert np.max(np.abs(g["w"][m][w_ok] - P.weights()[w_ok])) < 1e-12


def test_closest_point_query_matches_oracle(gpu, oracle):
    """cpm_closest_points (Surface::ClosestPoint) for every surface kind at random points
    near the surface: cp and dist within 1e-12 of the oracle's; a mesh search bounded by
    max_dist agrees with the unbounded one for points within max_dist."""
    from cpm_gb300 import workloads as W

    rng = np.random.default_rng(17)
    v, f = W.perturbed_icosphere(3, seed=2)
    bb = W.mesh_bbox(v)
    curves, _ = W.parallel_plane_curves(v, f, 2, seed=3)
    pv, ps = curves[0]
    cases = [
        (gpu.desc(gpu.SPHERE, [1.0]), oracle.sphere_desc(), 1.0),
        (gpu.desc(gpu.TORUS, [1.0, 0.4], (-1.4, 1.4)), oracle.torus_desc(1.0, 0.4, (-1.4, 1.4)), 1.4),
        (gpu.desc(gpu.CIRCLE3D, [0.8, 0.0, 0.0, 0.3, 0.0, 0.0, 1.0]),
         oracle.make_desc(oracle.CIRCLE3D, [0.8, 0.0, 0.0, 0.3, 0.0, 0.0, 1.0]), 1.0),
        (gpu.desc(gpu.POINT, [0.36, 0.48, 0.8]), oracle.make_desc(oracle.POINT, [0.36, 0.48, 0.8]), 1.0),
        (gpu.desc(gpu.TRIANGULATION, (), bb, verts=v, prims=f),
         oracle.make_desc(oracle.TRIANGULATION, (), bb, verts=v, prims=f), 0.6),
        (gpu.desc(gpu.POLYLINE, (), bb, verts=pv, prims=ps), oracle.make_desc(oracle.POLYLINE, (), bb, verts=pv, prims=ps), 0.6),
    ]
    for gd, od, ext in cases:
        x = rng.uniform(-ext, ext, (300, 3))
        cp, dist = gpu.closest_points(gd, x)
        cr, dr = oracle.closest_points(od, x)
        assert np.max(np.abs(cp - cr)) <= 1e-12 and np.max(np.abs(dist - dr)) <= 1e-12
    gd = cases[4][0]
    x = rng.uniform(-0.6, 0.6, (400, 3))
    cp, dist = gpu.closest_points(gd, x)
    cpb, distb = gpu.closest_points(gd, x, max_dist=0.1)
    near = dist < 0.1
    assert near.sum() > 20 and np.all(distb[~near] > 0.1)
    assert np.array_equal(cpb[near], cp[near]) and np.array_equal(distb[near], dist[near])


def test_interp_query_matches_oracle_rows(gpu, oracle):
    dx = 0.1
    P = oracle.RefProblem(oracle.sphere_desc(), [], 3, dx)
    T = gpu.Tube(gpu.desc(gpu.SPHERE, [1.0]), 3, dx)
    ref, g = P.tube(), T.export()
    m = ref_to_gpu_index(ref["rec"], g["rec"])
    inv = np.empty(T.N, np.int64)
    inv[m] = np.arange(T.N)
    ptr, idx, val = P.csr(3)  # E
    cols, vals = T.interp_query(ref["cp"])
    for q in range(0, P.N, 97):
        a = sorted(zip(idx[ptr[q]:ptr[q + 1]].tolist(), val[ptr[q]:ptr[q + 1]].tolist()))
        b = sorted(zip(inv[cols[q]].tolist(), vals[q].tolist()))
        assert [c for c, _ in a] == [c for c, _ in b]
        assert np.max(np.abs(np.array([v for _, v in a]) - np.array([v for _, v in b]))) < 1e-14


def two_circle_ibcs(mod, dx, order=2):
    """The two circle IBCs: z = 0.3 (u = 1) and z = -0.5 (u = 0) on the unit sphere."""
    mk = (lambda R, c, n: mod.circle3d_desc(R, c, n, dx, order)) if hasattr(mod, "circle3d_desc") else (
        lambda R, c, n: mod.desc(mod.CIRCLE3D, [R, *c, *n], (-1.0, 1.0), boundary_order=order, on_ibc_tolerance=0.1 * dx * dx))
    return [mk(math.sqrt(1 - 0.09), (0, 0, 0.3), (0, 0, 1)), mk(math.sqrt(1 - 0.25), (0, 0, -0.5), (0, 0, 1))]


@pytest.mark.parametrize("dx,order", [(0.1, 2), (0.05, 2), (0.05, 1)])
def test_ibc_subsets_bit_exact(gpu, oracle, dx, order):
    P = oracle.RefProblem(oracle.sphere_desc(), two_circle_ibcs(oracle, dx, order), 3, dx, record_visited=True)
    T = gpu.Tube.from_closest_points(gpu.desc(gpu.SPHERE, [1.0]), 3, dx, *P.visited())
    O = gpu.OpSet(T, two_circle_ibcs(gpu, dx, order))
    ref, g = P.tube(), T.export()
    assert O.D == P.D and O.total_ibc_dofs == P.total_ibc_dofs and O.num2 == P.num2
    for c in range(2):
        rs, gs = P.ibc_subsets(c), O.ibc_subsets(c)
        # same nodes in the same (BFS) order, compared as grid keys
        assert np.array_equal(g["rec"][gs["tag_set"]], ref["rec"][rs["tag_set"]])
        assert np.array_equal(g["rec"][gs["dof_set"]], ref["rec"][rs["dof_set"]])
        assert gs["col_start"] == rs["col_start"] and gs["identity_rows_start"] == rs["identity_rows_start"]
    rr, gr = P.rows(), O.rows()
    assert np.array_equal(rr["identity"][P.N:], gr["identity"][P.N:])
    assert np.array_equal(rr["kind"][P.N:], gr["kind"][P.N:])


def _permuted_csr(gpu_csr, m_inv_full, D):
    ptr, idx, val = gpu_csr
    rows = {}
    for r in range(D):
        rows[r] = (m_inv_full[idx[ptr[r]:ptr[r + 1]]], val[ptr[r]:ptr[r + 1]])
    return rows


@pytest.mark.parametrize("which", [0, 1])
def test_ibc_operator_rows_match_oracle(gpu, oracle, which):
    """Lfull / Efull rows (with IBC column moves) equal the oracle's up to rounding of the weights' products."""
    dx = 0.1
    P = oracle.RefProblem(oracle.sphere_desc(), two_circle_ibcs(oracle, dx), 3, dx, record_visited=True)
    T = gpu.Tube.from_closest_points(gpu.desc(gpu.SPHERE, [1.0]), 3, dx, *P.visited())
    O = gpu.OpSet(T, two_circle_ibcs(gpu, dx))
    ref, g = P.tube(), T.export()
    m = ref_to_gpu_index(ref["rec"], g["rec"])
    full = np.arange(O.D)
    full[m] = np.arange(P.N)  # gpu tube row -> reference row; IBC rows unchanged
    # gpu row index for each reference row
    g_of_ref = np.arange(O.D)
    g_of_ref[:P.N] = m
    rp, ri, rv = P.csr(which)
    gp, gi, gv = O.csr(which)
    # cp-bar of every IBC DOF row (oracle), to recognise base points on a grid plane
    cpbar = {}
    for c in range(2):
        s = P.ibc_subsets(c)
        for i, q in enumerate(range(s["col_start"], s["col_start"] + len(s["dof_set"]))):
            cpbar[q] = s["dof_cpbar"][i]
    on_plane = 0
    for r in range(P.D):
        gr = g_of_ref[r]
        a = dict(zip(ri[rp[r]:rp[r + 1]].tolist(), rv[rp[r]:rp[r + 1]].tolist()))
        b = dict(zip(full[gi[gp[gr]:gp[gr + 1]]].tolist(), gv[gp[gr]:gp[gr + 1]].tolist()))
        a = {k: v for k, v in a.items() if v != 0.0}
        b = {k: v for k, v in b.items() if v != 0.0}
        if a.keys() != b.keys() and r in cpbar:
            # the device's cp-bar (CUDA libm) and the oracle's may straddle a grid plane
            f = (cpbar[r] - P.xstart) / dx
            assert np.min(np.abs(f - np.round(f))) < 1e-9, (r, cpbar[r])
            on_plane += 1
            continue
        assert a.keys() == b.keys(), (r, sorted(set(a) ^ set(b)))
        # tube rows are bit-exact given the same closest points; IBC DOF rows
        # interpolate at cp-bar, which the device computes with CUDA's libm
        tol = 0.0 if r < P.N else 1e-13
        for k in a:
            assert abs(a[k] - b[k]) <= tol * max(1.0, abs(a[k])), (r, k, a[k], b[k])
    assert on_plane <= 8


@pytest.mark.parametrize("dx", [0.1, 0.05])
def test_plot_interpolation_with_ibc_columns_matches_oracle(gpu, oracle, dx):
    """Evaluation-point rows (GetPlotInterpMatrix + AddIBCPlotInterpolation) equal the
    oracle's: the same columns, moved to IBC DOF columns across the curves, and the
    same values."""
    P = oracle.RefProblem(oracle.sphere_desc(), two_circle_ibcs(oracle, dx), 3, dx, record_visited=True)
    T = gpu.Tube.from_closest_points(gpu.desc(gpu.SPHERE, [1.0]), 3, dx, *P.visited())
    O = gpu.OpSet(T, two_circle_ibcs(gpu, dx))
    ref, g = P.tube(), T.export()
    m = ref_to_gpu_index(ref["rec"], g["rec"])
    full = np.arange(O.D)
    full[m] = np.arange(P.N)  # gpu tube column -> reference column; IBC columns unchanged
    xp = P.xp()
    rp, ri, rv = P.csr(4)
    cols, vals = O.plot_interp(xp)
    moved = 0
    for i in range(len(xp)):
        a = {k: v for k, v in zip(ri[rp[i]:rp[i + 1]].tolist(), rv[rp[i]:rp[i + 1]].tolist()) if v != 0.0}
        b = {}
        for c, v in zip(full[cols[i]].tolist(), vals[i].tolist()):
            if v != 0.0:
                b[c] = b.get(c, 0.0) + v
        assert a.keys() == b.keys(), (i, sorted(set(a) ^ set(b)))
        for k in a:
            assert abs(a[k] - b[k]) <= 1e-14 * max(1.0, abs(a[k])), (i, k, a[k], b[k])
        moved += sum(1 for k in b if k >= P.N)
    assert moved > 0


def _oracle_pair(gpu, oracle, dx):
    from test_gpu_parity_c2 import same_cp_pair

    return same_cp_pair(gpu, oracle, dx, two_circle_ibcs(oracle, dx), two_circle_ibcs(gpu, dx))


def test_explicit_heat_step_matches_oracle(gpu, oracle):
    """HeatWithIBC's explicit step u <- Efull (u + dt Lfull u) on the device equals the same
    products of the oracle's Lfull / Efull (identity rows included: both hold 1 on their
    diagonal there), on a device operator built from the oracle's closest points."""
    dx = 0.05
    dt = 0.1 * dx * dx
    P, T, O, gr = _oracle_pair(gpu, oracle, dx)
    rng = np.random.default_rng(3)
    u = rng.standard_normal((2, O.D))
    got = O.explicit_step(dt, u)
    Lp, Li, Lv = P.csr(0)
    Ep, Ei, Ev = P.csr(1)
    for j in range(2):
        ur = u[j][gr]
        want = oracle.csr_matvec(Ep, Ei, Ev, ur + dt * oracle.csr_matvec(Lp, Li, Lv, ur))
        assert np.max(np.abs(got[j][gr] - want)) <= 1e-13 * np.max(np.abs(want))


def test_gray_scott_step_matches_oracle(gpu, oracle):
    """ReactionDiffusionWithIBC's Gray-Scott step on the device equals
    Efull (u + nu_u dt Lfull u + dt R_u), Efull (v + nu_v dt Lfull v + dt R_v) with the
    oracle's Lfull / Efull, the reaction terms from the old u, v."""
    dx = 0.05
    dt = 0.2
    P, T, O, gr = _oracle_pair(gpu, oracle, dx)
    rng = np.random.default_rng(4)
    u, v = rng.uniform(0, 1, O.D), rng.uniform(0, 0.5, O.D)
    gu, gv = O.gray_scott_step(dt, u, v)
    Lp, Li, Lv = P.csr(0)
    Ep, Ei, Ev = P.csr(1)
    nu_u = (dx / 3.0) ** 2
    nu_v = nu_u / 3.0
    F, k = 0.054, 0.063
    ur, vr = u[gr], v[gr]
    un = ur + nu_u * dt * oracle.csr_matvec(Lp, Li, Lv, ur) + dt * (-ur * vr * vr + F * (1 - ur))
    vn = vr + nu_v * dt * oracle.csr_matvec(Lp, Li, Lv, vr) + dt * (ur * vr * vr - (F + k) * vr)
    wu, wv = oracle.csr_matvec(Ep, Ei, Ev, un), oracle.csr_matvec(Ep, Ei, Ev, vn)
    assert np.max(np.abs(gu[gr] - wu)) <= 1e-13 * np.max(np.abs(wu))
    assert np.max(np.abs(gv[gr] - wv)) <= 1e-13 * np.max(np.abs(wv))


def test_nearest_baseline_operator_matches_oracle(gpu, oracle):
    """PoissonWithIBCNearest's operator (plain L and E, identity rows at the IBC DOF
    subsets' tube nodes): the device apply equals the reference Multiply assembled
    from the oracle's L and E with the same identity rows, and its FP64 solve
    reaches the tolerance on that operator."""
    dx = 0.1
    P0 = oracle.RefProblem(oracle.sphere_desc(), [], 3, dx, record_visited=True)
    PI = oracle.RefProblem(oracle.sphere_desc(), two_circle_ibcs(oracle, dx), 3, dx)
    T = gpu.Tube.from_closest_points(gpu.desc(gpu.SPHERE, [1.0]), 3, dx, *P0.visited())
    ref, g = P0.tube(), T.export()
    m = ref_to_gpu_index(ref["rec"], g["rec"])  # reference tube row -> device row
    N = P0.N
    ident_ref = np.zeros(N, bool)
    for c in range(2):
        ident_ref[PI.ibc_subsets(c)["dof_set"]] = True
    O = gpu.OpSet(T, identity_rows=np.sort(m[np.nonzero(ident_ref)[0]]))
    assert O.D == N and int(O.rows()["identity"].sum()) == int(ident_ref.sum())
    Lp, Li, Lv = P0.csr(0)
    Ep, Ei, Ev = P0.csr(1)
    diag = np.zeros(N)
    for r in range(N):
        for e in range(Lp[r], Lp[r + 1]):
            if Li[e] == r:
                diag[r] = Lv[e]
    rng = np.random.default_rng(6)
    x_ref = rng.standard_normal(N)
    t = np.where(ident_ref, x_ref, oracle.csr_matvec(Ep, Ei, Ev, x_ref))
    off = oracle.csr_matvec(Lp, Li, Lv, t) - diag * t
    want = np.where(ident_ref, x_ref, 0.0 * x_ref - (diag * x_ref + off))
    x_dev = np.empty(N)
    x_dev[m] = x_ref
    got = O.apply(0.0, -1.0, x_dev)[0][m]
    assert np.max(np.abs(got - want)) <= 1e-12 * np.max(np.abs(want))
    # solve: Dirichlet values at the identity rows, f = 0
    b_ref = np.where(ident_ref, rng.uniform(0, 1, N), 0.0)
    b_dev = np.empty(N)
    b_dev[m] = b_ref
    x, st = gpu.Solver(O, 0.0, -1.0).solve(b_dev, tol=1e-10, precision=0)
    r = O.apply(0.0, -1.0, x[0])[0] - b_dev
    assert st[0]["status"] == 0 and np.linalg.norm(r) <= 1e-9 * np.linalg.norm(b_dev)


def test_tube_nearest_is_grid_rounding(gpu):
    """Tube::NearestTubeIndex: the tube node at each point's rounded grid point, -1 off the tube."""
    dx = 0.1
    T = gpu.Tube(gpu.desc(gpu.SPHERE, [1.0]), 3, dx)
    g = T.export()
    rng = np.random.default_rng(8)
    x = rng.uniform(-1.3, 1.3, (2000, 3))
    idx = T.nearest(x)
    ijk = np.rint((x - T.xstart) / dx).astype(np.int64)
    n1 = T.N1d
    key = (ijk[:, 0] * n1 + ijk[:, 1]) * n1 + ijk[:, 2]
    of_key = {int(k): i for i, k in enumerate(g["rec"])}
    want = np.array([of_key.get(int(k), -1) for k in key])
    assert np.array_equal(idx, want) and (want >= 0).sum() > 100 and (want < 0).sum() > 100
