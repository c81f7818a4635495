"""The oracle (CPU restatement of the reference's solve path) against the
reference's own known answers: the golden average convergence orders its
convergence studies assert (+-1e-2), and its compile-time self-checks
(row sums of E equal 1, src/Interpolation.cpp:232-239; BFS IBC subset equals
the brute-force subset, src/IBCSubset.cpp:86-153)."""
import math

import numpy as np
import pytest

import studies as S


def test_shifted_poisson_sphere_golden_order(oracle):
    # convergence_studies/PoissonProblems/PoissonProblems.cpp:119-137,169,230,233
    errs = [S.oracle_error(S.shifted_poisson_sphere(dx), dx)[0] for dx in S.DX_3D]
    order, _ = S.convergence_order(errs, S.DX_3D)
    assert abs(order - S.GOLDEN_SHIFTED_POISSON_SPHERE) < 1e-2
    assert abs(order - S.GOLDEN_SHIFTED_POISSON_SPHERE) < 1e-4  # tighter than the reference asks


@pytest.mark.parametrize("i", [0, 1])
def test_sphere_circle_ibc_golden_order(oracle, i):
    # PoissonProblemsWithIBC.cpp:230-272 (order-2 Dirichlet Circle3D IBC), golden list :377
    errs = [S.oracle_error(S.sphere_circle_ibc(dx, i), dx)[0] for dx in S.DX_3D]
    order, _ = S.convergence_order(errs, S.DX_3D)
    assert abs(order - S.GOLDEN_SPHERE_CIRCLE[i]) < 1e-2


@pytest.mark.parametrize("i", [0, 1])
def test_sphere_point_ibc_golden_order(oracle, i):
    # PoissonProblemsWithIBC.cpp:274-317 (order-2 Dirichlet Point IBC), golden list :378
    errs = [S.oracle_error(S.sphere_point_ibc(dx, i), dx)[0] for dx in S.DX_3D]
    order, _ = S.convergence_order(errs, S.DX_3D)
    assert abs(order - S.GOLDEN_SPHERE_POINT[i]) < 1e-2


@pytest.mark.slow
@pytest.mark.parametrize("i", range(2, 10))
def test_sphere_circle_ibc_golden_order_all(oracle, i):
    errs = [S.oracle_error(S.sphere_circle_ibc(dx, i), dx)[0] for dx in S.DX_3D]
    assert abs(S.convergence_order(errs, S.DX_3D)[0] - S.GOLDEN_SPHERE_CIRCLE[i]) < 1e-2


@pytest.mark.slow
@pytest.mark.parametrize("i", range(2, 10))
def test_sphere_point_ibc_golden_order_all(oracle, i):
    errs = [S.oracle_error(S.sphere_point_ibc(dx, i), dx)[0] for dx in S.DX_3D]
    assert abs(S.convergence_order(errs, S.DX_3D)[0] - S.GOLDEN_SPHERE_POINT[i]) < 1e-2


def test_interpolation_rows_sum_to_one(oracle):
    P = oracle.RefProblem(oracle.sphere_desc(), [], 3, 0.1)
    ptr, idx, val = P.csr(3)
    sums = np.add.reduceat(val, ptr[:-1])
    assert np.allclose(sums, 1.0, atol=1e-13)
    assert np.all(np.diff(ptr) == 64)


def test_tube_is_band_component(oracle):
    """Tube = 6-connected component of {|d| <= r} containing the seed (src/Tube.cpp:429-454)."""
    P = oracle.RefProblem(oracle.sphere_desc(), [], 3, 0.1, record_visited=True)
    t = P.tube()
    rec, cp, dist = P.visited()
    inside = np.abs(dist) <= P.radius
    tube_keys = set(t["rec"].tolist())
    assert tube_keys <= set(rec[inside].tolist())
    # every visited node outside the tube is either out of the band or not adjacent... it was visited
    # because it neighbours a tube node; nodes of the band that were visited are all in the tube
    assert set(rec[inside].tolist()) == tube_keys
    assert abs(P.N - 10900) < 400  # about 10.9k nodes at dx = 0.1


def test_ibc_subset_equals_brute_force(oracle):
    """IBC_TESTS idea (src/IBCSubset.cpp:86-108): BFS subset = brute-force {dist_C < 2r}."""
    dx = 0.1
    R, c, n = S.circle3d_params([0.3, 0.2, 0.9])
    ibc = oracle.circle3d_desc(R, c, n, dx)
    P = oracle.RefProblem(oracle.sphere_desc(), [ibc], 3, dx)
    sub = P.ibc_subsets(0)
    t = P.tube()
    _, d = oracle.closest_points(ibc, t["x"])
    brute = np.nonzero(d < 2 * P.radius)[0]
    assert sorted(sub["tag_set"].tolist()) == sorted(brute.tolist())
    dof = sorted(sub["dof_set"].tolist())
    assert dof == sorted(np.nonzero(d < P.radius)[0].tolist())


def test_grid_sizing_matches_reference_formulas(oracle):
    """Tube::ConstructTube sizing (src/Tube.cpp:131-157) at the sphere and torus configs."""
    P = oracle.RefProblem(oracle.sphere_desc(), [], 3, 0.1)
    assert P.N1d == 33 and abs(P.xstart - (-1.6)) < 1e-15
    assert abs(P.radius - 1.0001 * math.sqrt(17) * 0.1) < 1e-15


@pytest.mark.parametrize("case", ["screened_poisson", "two_circle_laplace"])
def test_bicgstab_solution_matches_sparse_lu(oracle, case):
    """The oracle's matrix-free BiCGStab (tol 1e-10) against a direct solve of the
    same system assembled as a matrix with scipy.sparse from the exported Lfull
    and Efull (GeneralizedBiCGStabSystem::Multiply, src/GeneralizedBiCGStabSystem.h:191-233:
    identity rows y = x, other rows m x_q + n (L_qq x_q + sum_{c != q} L_qc t_c) with
    t = Efull x on non-identity rows and t = x on identity rows), solved by SuperLU:
    relative l_inf <= 1e-8."""
    sp = pytest.importorskip("scipy.sparse")
    spla = pytest.importorskip("scipy.sparse.linalg")
    dx = 0.1
    if case == "screened_poisson":
        P = oracle.RefProblem(oracle.sphere_desc(), [], 3, dx)
        m, n = 1.0, -1.0
        f, g = (lambda x: 3.0 * x[:, 2]), (lambda c, x: np.zeros(len(x)))
    else:
        ibcs = [oracle.circle3d_desc(math.sqrt(1 - 0.09), (0, 0, 0.3), (0, 0, 1), dx),
                oracle.circle3d_desc(math.sqrt(1 - 0.25), (0, 0, -0.5), (0, 0, 1), dx)]
        P = oracle.RefProblem(oracle.sphere_desc(), ibcs, 3, dx)
        m, n = 0.0, -1.0
        f, g = (lambda x: np.zeros(len(x))), (lambda c, x: np.full(len(x), 1.0 if c == 0 else 0.0))
    rows = P.rows()
    b = S.build_rhs(rows, f, g)
    D = P.D
    Lf = sp.csr_matrix(tuple(reversed(P.csr(0))), shape=(D, D))
    Ef = sp.csr_matrix(tuple(reversed(P.csr(1))), shape=(D, D)).tolil()
    ident = np.nonzero(rows["identity"])[0]
    for k in ident:
        Ef.rows[k] = [int(k)]
        Ef.data[k] = [1.0]
    dL = sp.diags(Lf.diagonal())
    A = (m * sp.identity(D, format="csr") + n * (dL + (Lf - dL) @ Ef.tocsr())).tolil()
    for k in ident:
        A.rows[k] = [int(k)]
        A.data[k] = [1.0]
    x_lu = spla.spsolve(A.tocsc(), b)
    x, st = P.solve(m, n, b)
    assert np.max(np.abs(x - x_lu)) <= 1e-8 * np.max(np.abs(x_lu))


@pytest.mark.parametrize("method", [0, 1, 2])
def test_heat_sphere_circle_golden_order(oracle, method):
    """HeatProblemsWithIBC's sphere-circle study (explicit, backward Euler, Crank-Nicolson
    time stepping with a 2nd-order Dirichlet circle) through the oracle: the average
    convergence order over dx = 0.1, 0.05, 0.025 equals the reference's golden value
    within 1e-2 (HeatProblemsWithIBC.cpp:307, :372)."""
    errs = [S.heat_sphere_circle_error(dx, method) for dx in S.DX_HEAT_3D]
    avg, _ = S.convergence_order(errs, S.DX_HEAT_3D)
    assert abs(avg - S.GOLDEN_HEAT_SPHERE_CIRCLE[method]) < 1e-2


@pytest.mark.parametrize("implicit", [False, True])
def test_heat_sphere_golden_order(oracle, implicit):
    """HeatProblems' sphere study (Heat::TimeStep, explicit or implicit Euler) through the
    oracle: the average order over dx = 0.2, 0.1, 0.05 equals the reference's golden value
    within 1e-2 (HeatProblems.cpp:156-158, :206)."""
    if not implicit:
        pytest.importorskip("scipy.sparse")
    errs = [S.heat_sphere_error(dx, implicit) for dx in S.DX_3D]
    avg, _ = S.convergence_order(errs, S.DX_3D)
    assert abs(avg - S.GOLDEN_HEAT_SPHERE[implicit]) < 1e-2


@pytest.mark.parametrize("kind", ["circle", "point"])
@pytest.mark.parametrize("freeze", [True, False])
@pytest.mark.parametrize("i", [0, 1])
def test_nearest_baseline_golden_order(oracle, kind, freeze, i):
    """PoissonWithIBCNearest in the reference's IBC study (problems 3, 4, 6, 7 of
    PoissonProblemsWithIBC.cpp:453-469): identity rows at the nodes nearest the IBC's plot
    points (freeze_nearest) or at its DOF subset's nodes, on the oracle's tube, L and E.
    The average order over dx = 0.2, 0.1, 0.05 equals the golden value within 1e-2
    (:383-386)."""
    pytest.importorskip("scipy.sparse.linalg")
    build = S.sphere_circle_ibc if kind == "circle" else S.sphere_point_ibc
    errs = [S.nearest_baseline_error(build(dx, i), dx, freeze) for dx in S.DX_3D]
    golden = (S.GOLDEN_SPHERE_CIRCLE_NEAREST if kind == "circle" else S.GOLDEN_SPHERE_POINT_NEAREST)[freeze][i]
    assert abs(S.convergence_order(errs, S.DX_3D)[0] - golden) < 1e-2


@pytest.mark.parametrize("kind", ["circle", "point"])
@pytest.mark.parametrize("i", [0, 1])
def test_order1_ibc_golden_order(oracle, kind, i):
    """First-order Dirichlet IBCs (boundary_order 1) in the reference's IBC study: the
    average order over dx = 0.2, 0.1, 0.05 equals the golden value within 1e-2
    (PoissonProblemsWithIBC.cpp:369-370)."""
    build = S.sphere_circle_ibc if kind == "circle" else S.sphere_point_ibc
    errs = [S.oracle_error(build(dx, i, order=1), dx)[0] for dx in S.DX_3D]
    golden = (S.GOLDEN_SPHERE_CIRCLE_ORDER1 if kind == "circle" else S.GOLDEN_SPHERE_POINT_ORDER1)[i]
    assert abs(S.convergence_order(errs, S.DX_3D)[0] - golden) < 1e-2


def test_heat_sphere_circle_neumann_golden_order(oracle):
    """The same heat study with a zero-Neumann great circle (boundary_type 1, order 2) and
    backward Euler: average order within 1e-2 of the golden value
    (HeatProblemsWithIBC.cpp:318), pinning the oracle's Neumann IBC rows."""
    errs = [S.heat_sphere_circle_error(dx, 1, boundary_type=1) for dx in S.DX_HEAT_3D]
    avg, _ = S.convergence_order(errs, S.DX_HEAT_3D)
    assert abs(avg - S.GOLDEN_HEAT_SPHERE_CIRCLE_NEUMANN[1]) < 1e-2


def test_gradient_matrices_difference_linear_functions(oracle):
    """Dc_x, Dc_y, Dc_z (FDMatrices::BuildGradientMatrices): central differences of the grid
    coordinates give 1 along their own axis and 0 across it, on every tube node whose two
    neighbours along the axis are in the tube."""
    import numpy as np

    P = oracle.RefProblem(oracle.sphere_desc(), [], 3, 0.2)
    t = P.tube()
    for d in range(3):
        ptr, idx, val = P.csr(5 + d)
        full = np.diff(ptr) == 2
        for a in range(3):
            g = oracle.csr_matvec(ptr, idx, val, t["x"][:, a])
            want = 1.0 if a == d else 0.0
            assert np.allclose(g[full], want, atol=1e-12)
        assert set(np.round(val * P.dx, 12)) <= {0.5, -0.5}
