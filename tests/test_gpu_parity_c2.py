"""Parity with the oracle at the size of the two-circle Laplace configuration
(unit sphere, Dirichlet circles z = 0.3 and z = -0.5, dx = 0.025: 166,390 tube
nodes, 215,662 rows), and on the reference's other IBC options: Neumann rows,
oriented curves, and curves close enough that a stencil entry moves to both.

"Given the same closest points" means: the tube is built from the oracle's
closest points (cpm_tube_build_from_cp), and the IBC build takes the oracle's
IBC closest points at the tube nodes and its cp-bar closest points
(cpm_opset_create_from_cp).  Then, bit for bit:
  * tube membership, coordinates, base points, tricubic weights, neighbours;
  * IBC tagging and DOF subsets in the reference's BFS order, DOF closest
    points, the column layout, every Lfull and Efull entry (no exemptions).
FP64 solves: both sides solved to relative residual 1e-12, solutions within
relative l_inf 1e-10.
"""
import math

import numpy as np
import pytest

import studies as S
from test_gpu_setup import ref_to_gpu_index, two_circle_ibcs

pytestmark = pytest.mark.gpu

FP64_SOLVE_TOL = 1e-12  # relative residual both sides are solved to
FP64_PARITY = 1e-10     # relative l_inf between the device and the oracle solutions


def _rel_inf(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def same_cp_pair(gpu, oracle, dx, ibcs_oracle, ibcs_gpu, surface=None):
    """(oracle problem, device tube, device opset, device row of each reference row)
    with the device built from the oracle's closest points"""
    od = surface[0] if surface else oracle.sphere_desc()
    gd = surface[1] if surface else gpu.desc(gpu.SPHERE, [1.0])
    P = oracle.RefProblem(od, ibcs_oracle, 3, dx, record_visited=True)
    T = gpu.Tube.from_closest_points(gd, 3, dx, *P.visited())
    g = T.export()
    tabs = []
    for d in ibcs_oracle:
        cp, dist = oracle.closest_points(d, g["x"])
        tabs.append(gpu.cp_table(g["x"], cp, dist))
    # cp-bar: the surface's closest points at 2 cp_c - x of every DOF (order 2)
    proj, cpb = [], []
    ref = P.tube()
    for c in range(len(ibcs_oracle)):
        s = P.ibc_subsets(c)
        if len(s["dof_set"]) and ibcs_oracle[c].boundary_order == 2:
            p = 2.0 * s["dof_cp"] - ref["x"][s["dof_set"]]
            proj.append(p)
            cpb.append(oracle.closest_points(od, p)[0])
    surf = gpu.cp_table(np.concatenate(proj), np.concatenate(cpb)) if proj else None
    O = gpu.OpSet(T, ibcs_gpu, ibc_cp=tabs, surface_cp=surf)
    m = ref_to_gpu_index(ref["rec"], g["rec"])
    g_of_ref = np.arange(O.D)
    g_of_ref[:P.N] = m
    return P, T, O, g_of_ref


def _csr_triplets(ptr, idx, val, row_map=None, col_map=None):
    rows = np.repeat(np.arange(len(ptr) - 1), np.diff(ptr))
    cols = np.asarray(idx)
    keep = val != 0.0
    rows, cols, vals = rows[keep], cols[keep], val[keep]
    if row_map is not None:
        rows = row_map[rows]
    if col_map is not None:
        cols = col_map[cols]
    o = np.lexsort((cols, rows))
    return rows[o], cols[o], vals[o]


def assert_rows_bit_exact(P, O, g_of_ref, which):
    """Lfull (which 0) / Efull (1): every reference row equals its device row, entry by entry"""
    ref_of_g = np.empty(O.D, np.int64)
    ref_of_g[g_of_ref] = np.arange(O.D)
    a = _csr_triplets(*P.csr(which))
    b = _csr_triplets(*O.csr(which), row_map=ref_of_g, col_map=ref_of_g)
    assert len(a[0]) == len(b[0])
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(a[2], b[2]), np.max(np.abs(a[2] - b[2]))


@pytest.fixture(scope="module")
def c2(gpu, oracle):
    dx = 0.025
    return same_cp_pair(gpu, oracle, dx, two_circle_ibcs(oracle, dx), two_circle_ibcs(gpu, dx))


def test_c2_tube_bit_exact(c2):
    P, T, O, gr = c2
    ref, g = P.tube(), T.export()
    assert T.N == P.N == 166390 and T.N1d == P.N1d and T.xstart == P.xstart and T.radius == P.radius
    m = gr[:P.N]
    assert np.array_equal(g["rec"][m], ref["rec"])
    assert np.array_equal(g["x"][m], ref["x"]) and np.array_equal(g["cp"][m], ref["cp"])
    assert np.array_equal(g["bpt"][m], ref["rec"][ref["bpt"]])
    assert np.array_equal(g["w"][m], P.weights())
    inv = np.empty(T.N, np.int64)
    inv[m] = np.arange(T.N)
    gn = g["nbr"][m]
    assert np.array_equal(np.where(gn >= 0, inv[np.maximum(gn, 0)], -1), ref["nbr"])
    assert np.array_equal(T.reference_order(), m)


def test_c2_ibc_subsets_bit_exact(c2):
    P, T, O, gr = c2
    ref, g = P.tube(), T.export()
    assert O.D == P.D == 215662 and O.total_ibc_dofs == P.total_ibc_dofs and O.num2 == P.num2
    for c in range(2):
        rs, gs = P.ibc_subsets(c), O.ibc_subsets(c)
        assert np.array_equal(g["rec"][gs["tag_set"]], ref["rec"][rs["tag_set"]])
        assert np.array_equal(g["rec"][gs["dof_set"]], ref["rec"][rs["dof_set"]])
        assert np.array_equal(gs["dof_cp"], rs["dof_cp"])
        assert gs["col_start"] == rs["col_start"] and gs["dcol_start"] == rs["dcol_start"]
        assert gs["identity_rows_start"] == rs["identity_rows_start"]
    rr, gg = P.rows(), O.rows()
    assert np.array_equal(rr["identity"], gg["identity"][gr])
    assert np.array_equal(rr["kind"], gg["kind"][gr])


@pytest.mark.parametrize("which", [0, 1])
def test_c2_operator_rows_bit_exact(c2, which):
    P, T, O, gr = c2
    assert_rows_bit_exact(P, O, gr, which)


@pytest.mark.parametrize("which", [5, 6, 7])
def test_c2_gradient_rows_bit_exact(c2, which):
    """The gradient matrices Dc_x, Dc_y, Dc_z (FDMatrices::BuildGradientMatrices) of the tube
    rows equal the oracle's entry by entry."""
    P, T, O, gr = c2
    assert_rows_bit_exact(P, O, gr, which)


def test_c2_plain_fp64_solve_within_1e10(gpu, c2):
    """The plain FP64 GPU path against the oracle's solve of the same system:
    Laplace with circle values U[0,1], both to relative residual 1e-12."""
    P, T, O, gr = c2
    rows = P.rows()
    vals = np.random.default_rng(31).uniform(0, 1, 2)
    b = S.build_rhs(rows, lambda x: np.zeros(len(x)), lambda c, x: np.full(len(x), vals[c]))
    x_ref, st_ref = P.solve(0.0, -1.0, b, tol=FP64_SOLVE_TOL)
    bg = np.empty(O.D)
    bg[gr] = b
    x_gpu, st = gpu.Solver(O, 0.0, -1.0).solve(bg, tol=FP64_SOLVE_TOL, precision=0)
    assert st[0]["status"] == 0 and st[0]["rel_residual"] <= FP64_SOLVE_TOL
    assert _rel_inf(x_gpu[0][gr], x_ref) <= FP64_PARITY


@pytest.mark.parametrize("dx", [0.1, 0.05])
@pytest.mark.parametrize("order", [1, 2])
def test_two_circle_rows_bit_exact(gpu, oracle, dx, order):
    P, T, O, gr = same_cp_pair(gpu, oracle, dx, two_circle_ibcs(oracle, dx, order), two_circle_ibcs(gpu, dx, order))
    for which in (0, 1):
        assert_rows_bit_exact(P, O, gr, which)


# ---- Neumann IBC rows (boundary_type 1): the zero-Neumann great circle of the
# heat study (convergence_studies/HeatProblemsWithIBC/HeatProblemsWithIBC.cpp:318)

def _neumann_circle(mod, dx, order):
    R, c, n = S.heat_circle_params(boundary_type=1)
    if hasattr(mod, "circle3d_desc"):
        d = mod.circle3d_desc(R, tuple(c), tuple(n), dx, boundary_order=order)
    else:
        d = mod.desc(mod.CIRCLE3D, [R, *c, *n], (-1.0, 1.0), boundary_order=order, on_ibc_tolerance=0.1 * dx * dx)
    d.boundary_type[0] = 1
    return d


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("dx", [0.1, 0.05])
def test_neumann_rows_bit_exact(gpu, oracle, dx, order):
    P, T, O, gr = same_cp_pair(gpu, oracle, dx, [_neumann_circle(oracle, dx, order)], [_neumann_circle(gpu, dx, order)])
    assert O.D == P.D and O.total_ibc_dofs == P.total_ibc_dofs and O.num2 == P.num2 == 0
    rr, gg = P.rows(), O.rows()
    assert np.array_equal(rr["identity"], gg["identity"][gr]) and not rr["identity"].any()
    for which in (0, 1):
        assert_rows_bit_exact(P, O, gr, which)


@pytest.mark.parametrize("order", [1, 2])
def test_neumann_apply_and_backward_euler_match_oracle(gpu, oracle, order):
    """Apply (relative l_inf <= 1e-14) and one backward-Euler heat step
    (I - dt L E) u1 = u0 of the Neumann system (<= 1e-10 at tol 1e-12)."""
    dx = 0.05
    P, T, O, gr = same_cp_pair(gpu, oracle, dx, [_neumann_circle(oracle, dx, order)], [_neumann_circle(gpu, dx, order)])
    rng = np.random.default_rng(5)
    x = rng.standard_normal(P.D)
    xg = np.empty(O.D)
    xg[gr] = x
    dt = 0.1 * dx
    for m, n in ((1.0, -dt), (0.0, -1.0)):
        assert _rel_inf(O.apply(m, n, xg)[0][gr], P.apply(m, n, x)) <= 1e-14
    u0 = P.rows()["point"][:, 2].copy()
    u_ref, _ = P.solve(1.0, -dt, u0, tol=FP64_SOLVE_TOL)
    ug = np.empty(O.D)
    ug[gr] = u0
    u_gpu, st = gpu.Solver(O, 1.0, -dt).solve(ug, tol=FP64_SOLVE_TOL, precision=0)
    assert st[0]["status"] == 0
    assert _rel_inf(u_gpu[0][gr], u_ref) <= FP64_PARITY


# ---- oriented IBCs (IBCMetaData::is_oriented, point_on_side1; IBCDOFSubset::OrientSubset,
# src/IBCDOFSubset.cpp:128-227), as the reference's diffusion-curve programs set them
# (examples/DiffusionCurvesNefertiti/DiffusionCurvesNefertiti.cpp:233-235): the circle
# z = 0.3 on the unit sphere, side 1 toward the point above it

def _oriented_circle(mod, dx, order, bt):
    R = math.sqrt(1 - 0.09)
    if hasattr(mod, "circle3d_desc"):
        d = mod.circle3d_desc(R, (0, 0, 0.3), (0, 0, 1), dx, boundary_order=order)
    else:
        d = mod.desc(mod.CIRCLE3D, [R, 0, 0, 0.3, 0, 0, 1], (-1.0, 1.0), boundary_order=order,
                     on_ibc_tolerance=0.1 * dx * dx)
    d.is_oriented = 1
    d.has_point_on_side1 = 1
    z = 0.45
    d.point_on_side1[0], d.point_on_side1[1], d.point_on_side1[2] = math.sqrt(1 - z * z), 0.0, z
    d.boundary_type[0], d.boundary_type[1] = bt
    return d


@pytest.mark.parametrize("order,bt", [(2, (0, 0)), (2, (0, 1)), (1, (0, 0)), (1, (1, 0))])
def test_oriented_rows_bit_exact(gpu, oracle, order, bt):
    dx = 0.05
    P, T, O, gr = same_cp_pair(gpu, oracle, dx, [_oriented_circle(oracle, dx, order, bt)],
                               [_oriented_circle(gpu, dx, order, bt)])
    assert O.D == P.D and O.total_ibc_dofs == P.total_ibc_dofs and O.num2 == P.num2
    rr, gg = P.rows(), O.rows()
    for k in ("identity", "kind", "ibc", "side"):
        assert np.array_equal(rr[k], gg[k][gr]), k
    sides = rr["side"][P.N:P.N + P.total_ibc_dofs]
    assert set(np.unique(sides).tolist()) == {1, 2}  # both sides of the curve carry DOFs
    for which in (0, 1):
        assert_rows_bit_exact(P, O, gr, which)


def test_oriented_two_valued_dirichlet_solve_within_1e10(gpu, oracle):
    """A curve with a different Dirichlet value on each side (a diffusion curve's two
    colours): GetRHS hands the side to the boundary-value function; the FP64 solve
    equals the oracle's within 1e-10 (both to tol 1e-12)."""
    dx = 0.05
    P, T, O, gr = same_cp_pair(gpu, oracle, dx, [_oriented_circle(oracle, dx, 2, (0, 0))],
                               [_oriented_circle(gpu, dx, 2, (0, 0))])
    rows = P.rows()
    value = {1: 1.0, 2: 0.25}
    b = np.zeros(P.D)
    d = rows["kind"] == 2
    b[d] = [value[int(s)] for s in rows["side"][d]]
    x_ref, _ = P.solve(0.0, -1.0, b, tol=FP64_SOLVE_TOL)
    bg = np.empty(O.D)
    bg[gr] = b
    x_gpu, st = gpu.Solver(O, 0.0, -1.0).solve(bg, tol=FP64_SOLVE_TOL, precision=0)
    assert st[0]["status"] == 0
    assert _rel_inf(x_gpu[0][gr], x_ref) <= FP64_PARITY
    # the two sides really differ: just above and below the curve the solution differs
    up = rows["point"][:P.N, 2] > 0.34
    down = (rows["point"][:P.N, 2] < 0.26) & (rows["point"][:P.N, 2] > 0.2)
    assert np.mean(x_ref[:P.N][up]) > np.mean(x_ref[:P.N][down]) + 0.1


@pytest.mark.parametrize("option", ["use_cp_diff_directions", "no_jcp_normals"])
def test_ibc_direction_options_rows_bit_exact(gpu, oracle, option):
    """IBCMetaData::use_cp_diff_directions (directions = cp_diff, src/IBCSubset.cpp:156-187)
    and use_Jcp_surface_normals = false (frames from the normals x - cp,
    src/Geometry.cpp:101-126) on the two circles, order 2."""
    dx = 0.05
    io, ig = two_circle_ibcs(oracle, dx), two_circle_ibcs(gpu, dx)
    for d in io + ig:
        if option == "use_cp_diff_directions":
            d.use_cp_diff_directions = 1
        else:
            d.use_Jcp_surface_normals = 0
    P, T, O, gr = same_cp_pair(gpu, oracle, dx, io, ig)
    assert O.D == P.D and O.total_ibc_dofs == P.total_ibc_dofs
    for which in (0, 1):
        assert_rows_bit_exact(P, O, gr, which)


# ---- IBCs close enough that one stencil entry lies across both: MoveToIBCColumns
# (src/IBCMatrixManipulations.cpp:189-216) keeps one copy of the entry for every IBC
# whose tag crosses it, each in that IBC's DOF column.  The circles z = 0.3 and
# z = 0.3 + gap on the unit sphere; gap < dx also doubles L entries.

def _close_circles(mod, dx, gap, order):
    zs = (0.3, 0.3 + gap)
    if hasattr(mod, "circle3d_desc"):
        return [mod.circle3d_desc(math.sqrt(1 - z * z), (0, 0, z), (0, 0, 1), dx, boundary_order=order) for z in zs]
    return [mod.desc(mod.CIRCLE3D, [math.sqrt(1 - z * z), 0, 0, z, 0, 0, 1], (-1.0, 1.0), boundary_order=order,
                     on_ibc_tolerance=0.1 * dx * dx) for z in zs]


def _close_pair(gpu, oracle, dx, gap, order):
    return same_cp_pair(gpu, oracle, dx, _close_circles(oracle, dx, gap, order), _close_circles(gpu, dx, gap, order))


@pytest.mark.parametrize("dx,gap,order", [(0.05, 0.06, 2), (0.05, 0.04, 2), (0.05, 0.04, 1), (0.1, 0.08, 2)])
def test_close_circles_rows_bit_exact(gpu, oracle, dx, gap, order):
    P, T, O, gr = _close_pair(gpu, oracle, dx, gap, order)
    assert (np.diff(P.csr(1)[0])[:P.N] > 64).any()  # E entries that move to both circles
    assert (np.diff(P.csr(0)[0])[:P.N] > 7).any() == (gap < dx)  # and L entries
    assert O.D == P.D and O.total_ibc_dofs == P.total_ibc_dofs and O.num2 == P.num2
    rr, gg = P.rows(), O.rows()
    for k in ("identity", "kind", "ibc"):
        assert np.array_equal(rr[k], gg[k][gr]), k
    for which in (0, 1):
        assert_rows_bit_exact(P, O, gr, which)


@pytest.mark.parametrize("order", [1, 2])
def test_close_circles_applies_and_solves_match_oracle(gpu, oracle, order):
    """The operator with doubled E and L entries: the FP64 apply (1 and 32 slots)
    within 1e-13 of the oracle's, the FP32 32-slot apply within 1e-5; Laplace with
    a value per circle: the plain FP64 solve within 1e-10 of the oracle's (both to
    tol 1e-12), the 32-slot mixed-precision solves within 1e-8."""
    import torch

    dx, gap = 0.05, 0.04
    P, T, O, gr = _close_pair(gpu, oracle, dx, gap, order)
    rng = np.random.default_rng(12)
    x = rng.standard_normal(P.D)
    xg = np.empty(O.D)
    xg[gr] = x
    for m, n in ((1.0, -0.1 * dx), (0.0, -1.0)):
        assert _rel_inf(O.apply(m, n, xg)[0][gr], P.apply(m, n, x)) <= 1e-13
    X = rng.uniform(-1, 1, (32, P.D))
    Xg = np.empty((O.D, 32))
    Xg[gr] = X.T
    x64 = torch.from_numpy(Xg).cuda()
    t64, y64 = torch.empty_like(x64), torch.empty_like(x64)
    x32 = x64.float()
    t32, y32 = torch.empty_like(x32), torch.empty_like(x32)
    torch.cuda.synchronize()
    O.apply_device(0.0, -1.0, 32, False, x64.data_ptr(), t64.data_ptr(), y64.data_ptr())
    O.apply_device(0.0, -1.0, 32, True, x32.data_ptr(), t32.data_ptr(), y32.data_ptr())
    gpu.sync()
    Y64, Y32 = y64.cpu().numpy(), y32.cpu().double().numpy()
    for k in (0, 17, 31):
        assert _rel_inf(Y64[gr, k], P.apply(0.0, -1.0, X[k])) <= 1e-13
    assert _rel_inf(Y32, Y64) <= 1e-5
    rows = P.rows()
    vals = rng.uniform(0, 1, (32, 2))

    def rhs(v):
        return S.build_rhs(rows, lambda p: np.zeros(len(p)), lambda c, p: np.full(len(p), v[c]))

    B = np.stack([rhs(v) for v in vals])
    Bg = np.empty((32, O.D))
    Bg[:, gr] = B
    x_ref, _ = P.solve(0.0, -1.0, B[0], tol=FP64_SOLVE_TOL)
    x1, st = gpu.Solver(O, 0.0, -1.0).solve(Bg[0], tol=FP64_SOLVE_TOL, precision=0)
    assert st[0]["status"] == 0
    assert _rel_inf(x1[0][gr], x_ref) <= FP64_PARITY
    Xm, stm = gpu.Solver(O, 0.0, -1.0, kslots=32).solve(Bg, precision=1)
    assert all(s_["status"] == 0 for s_ in stm), stm
    for k in (0, 31):
        xr = x_ref if k == 0 else P.solve(0.0, -1.0, B[k], tol=FP64_SOLVE_TOL)[0]
        assert _rel_inf(Xm[k][gr], xr) <= 1e-8


def test_close_circles_evaluation_rows_match_oracle(gpu, oracle):
    """Evaluation rows (GetPlotInterpMatrix + AddIBCPlotInterpolation) at the
    sphere's plot points: the CSR query carries the doubled entries (points with
    more than 64), with the oracle's columns and values within 1e-14; the fixed
    64-entry query refuses these points."""
    dx, gap = 0.05, 0.04
    P, T, O, gr = _close_pair(gpu, oracle, dx, gap, 2)
    ref_of_g = np.empty(O.D, np.int64)
    ref_of_g[gr] = np.arange(O.D)
    xp = P.xp()
    rp, ri, rv = P.csr(4)
    ptr, cols, vals = O.plot_interp_csr(xp)
    assert (np.diff(rp) > 64).sum() == (np.diff(ptr) > 64).sum() > 0
    a = _csr_triplets(rp, ri, rv)
    b = _csr_triplets(ptr, cols, vals, col_map=ref_of_g)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.all(np.abs(a[2] - b[2]) <= 1e-14 * np.maximum(1.0, np.abs(a[2])))
    with pytest.raises(RuntimeError):
        O.plot_interp(xp)
    keep = np.diff(ptr) == 64  # points with no doubled entry: the two queries agree
    c64, v64 = O.plot_interp(xp[keep][:500])
    sel = np.flatnonzero(keep)[:500]
    assert np.array_equal(c64, cols[ptr[sel][:, None] + np.arange(64)])
    assert np.array_equal(v64, vals[ptr[sel][:, None] + np.arange(64)])


@pytest.mark.parametrize("scale", [0.6, 1.5])
def test_dof_radius_scale_rows_bit_exact(gpu, oracle, scale):
    """IBCMetaData::ibc_DOFSubset_radius_scale (src/IBCDOFSubset.cpp:20,44): the DOF subset is
    the tagged nodes within scale * r of the curve; subsets and every Lfull / Efull row equal
    the oracle's."""
    dx = 0.05
    oi, gi = two_circle_ibcs(oracle, dx), two_circle_ibcs(gpu, dx)
    for d in oi + gi:
        d.dof_radius_scale = scale
    P, T, O, gr = same_cp_pair(gpu, oracle, dx, oi, gi)
    ref, g = P.tube(), T.export()
    assert O.D == P.D and O.total_ibc_dofs == P.total_ibc_dofs and O.num2 == P.num2
    for c in range(2):
        rs, gs = P.ibc_subsets(c), O.ibc_subsets(c)
        assert np.array_equal(g["rec"][gs["dof_set"]], ref["rec"][rs["dof_set"]])
    for which in (0, 1):
        assert_rows_bit_exact(P, O, gr, which)
