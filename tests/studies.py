"""Convergence-study problems of the reference, restated for the oracle and the GPU path.

Each builder returns (surface, ibcs, m, n, f, g, exact) for one grid spacing,
following the reference's convergence-study drivers:
  ShiftedPoissonSphere     convergence_studies/PoissonProblems/PoissonProblems.cpp:119-137
  PoissonSphereCircleIBC   convergence_studies/PoissonProblemsWithIBC/PoissonProblemsWithIBC.cpp:230-272
  PoissonSpherePointIBC    convergence_studies/PoissonProblemsWithIBC/PoissonProblemsWithIBC.cpp:274-317
  ComputeCircle3DParams    convergence_studies/PoissonProblemsWithIBC/PoissonProblemsWithIBC.cpp:117-139
  HeatSphereCircleIBC      convergence_studies/HeatProblemsWithIBC/HeatProblemsWithIBC.cpp:68-139,141-283
  HeatSphere               convergence_studies/HeatProblems/HeatProblems.cpp:125-145
  nearest-node baselines   PoissonProblemsWithIBC.cpp:230-317 (ibc_type 1, 2) with
                           problems/PoissonWithIBCNearest.cpp:5-89
Golden average orders (the reference's own pass/fail pins, +-1e-2):
  PoissonProblems.cpp:169, PoissonProblemsWithIBC.cpp:375-379 and
  HeatProblemsWithIBC.cpp:307 (Dirichlet, boundary order 2), HeatProblems.cpp:156-158 and
  PoissonProblemsWithIBC.cpp:383-386 (nearest-node baselines).
"""
import math

import numpy as np

import oracle_lib as ol

GOLDEN_SHIFTED_POISSON_SPHERE = 2.18548
# order-2 lists, PoissonProblemsWithIBC.cpp:377-378
GOLDEN_SPHERE_CIRCLE = [2.03624, 2.20571, 2.09173, 2.0828, 2.1572, 2.10696, 1.97858, 1.97003, 2.17008, 1.9772]
GOLDEN_SPHERE_POINT = [2.16283, 2.13198, 1.92074, 2.22093, 2.27176, 2.36021, 1.89006, 2.12619, 2.22663, 2.70325]
# order-1 lists, PoissonProblemsWithIBC.cpp:369-370
GOLDEN_SPHERE_CIRCLE_ORDER1 = [0.954594, 0.990541, 1.07685, 0.865972, 0.784669, 0.922806, 0.991011, 0.987983, 0.90721,
                               0.956464]
GOLDEN_SPHERE_POINT_ORDER1 = [2.42046, 2.03873, 1.03422, 0.973755, 1.54908, 2.12488, 2.12239, 1.02281, 1.05949, 1.37816]
# PoissonProblemsWithIBC.cpp:399-424
RAND_NUM = [0.0, 0.170, 0.297, 0.331, 0.481, 0.511, 0.631, 0.735, 0.813, 0.973]
RAND_NUM2 = [0.25, 0.874, 0.473, 0.973, 0.812, 0.693, 0.873, 0.912, 0.945, 1.0]
RAND_NUM3 = [0.55, 0.123, -0.743, 0.547, -0.239, -0.693, 0.731, -0.175, 0.453, -0.364]
DX_3D = [0.2, 0.1, 0.05]  # Helpers::ConvergenceStudy(0.2, 3, ...): dx = 0.5^i * 0.2


def sphere_harmonic(x):
    """u = cos(3 theta) sin^3(phi) (9 cos^2(phi) - 1) with theta = atan2(y, x), phi = acos(z)."""
    x = np.atleast_2d(x)
    th = np.arctan2(x[:, 1], x[:, 0])
    ph = np.arccos(np.clip(x[:, 2] / 1.0, -1, 1))
    return np.cos(3 * th) * np.sin(ph) ** 3 * (9 * np.cos(ph) ** 2 - 1)


def circle3d_params(normal):
    n = np.asarray(normal, np.float64)
    n = n / math.sqrt(float(np.dot(n, n)))
    r, theta, phi = 0.2, 0.1, 0.2
    pop = np.array([r * math.cos(phi) * math.sin(theta), r * math.sin(phi) * math.sin(theta), r * math.cos(theta)])
    rho = -float(np.dot(pop, n))
    centre = rho * n
    return math.sqrt(1 - rho * rho), centre, n


def shifted_poisson_sphere(dx):
    surf = ol.sphere_desc()
    return dict(surface=surf, ibcs=[], m=1.0, n=1.0, f=lambda x: -29.0 * sphere_harmonic(x), g=None,
                exact=sphere_harmonic)


def sphere_circle_ibc(dx, i, order=2):
    R, centre, normal = circle3d_params([RAND_NUM[i], RAND_NUM2[i], RAND_NUM3[i]])
    ibc = ol.circle3d_desc(R, centre, normal, dx, boundary_order=order)
    return dict(surface=ol.sphere_desc(), ibcs=[ibc], m=0.0, n=-1.0, f=lambda x: 30.0 * sphere_harmonic(x),
                g=lambda c, x: sphere_harmonic(x), exact=sphere_harmonic,
                ibc_xp=circle3d_plot_points(R, centre, normal))


def sphere_point_ibc(dx, i, order=2):
    th = 2.0 * math.pi * RAND_NUM[i] - math.pi
    ph = 2.0 * math.pi * RAND_NUM2[i] - math.pi
    p = [math.cos(ph) * math.cos(th), math.cos(ph) * math.sin(th), math.sin(ph)]
    ibc = ol.point_desc(p, dx, boundary_order=order)
    return dict(surface=ol.sphere_desc(), ibcs=[ibc], m=0.0, n=-1.0, f=lambda x: 30.0 * sphere_harmonic(x),
                g=lambda c, x: sphere_harmonic(x), exact=sphere_harmonic, ibc_xp=np.array([p]))


# HeatProblemsWithIBC.cpp:307, problems 3-5 (the sphere): explicit, backward Euler, Crank-Nicolson
GOLDEN_HEAT_SPHERE_CIRCLE = [1.98885, 1.15183, 2.01012]
GOLDEN_HEAT_SPHERE_CIRCLE_NEUMANN = [2.07915, 1.15527, 2.04239]  # :318
DX_HEAT_3D = [0.1, 0.05, 0.025]  # Helpers::ConvergenceStudy(0.1, 3, ...) (HeatProblemsWithIBC.cpp:367)
HEAT_FINAL_TIME = 0.1  # g_final_time (HeatProblemsWithIBC.cpp:19)


def heat_circle_params(boundary_type=0):
    """ComputeCircle3DParams (HeatProblemsWithIBC.cpp:68-86) for the plane of SphereCircleIBC
    (:94-106): Dirichlet, normal (1.1, 1.234, 1.321) through the point r = 0.27, theta = 0.132,
    phi = 0.221; Neumann, normal (0, 1, 0) through the origin."""
    if boundary_type == 1:
        n, pop = np.array([0.0, 1.0, 0.0]), np.zeros(3)
        rho = -float(np.dot(pop, n))
        return math.sqrt(1 - rho * rho), rho * n, n
    n = np.array([1.1, 1.234, 1.321])
    n = n / math.sqrt(float(np.dot(n, n)))
    r, th, ph = 0.27, 0.132, 0.221
    pop = np.array([r * math.cos(ph) * math.sin(th), r * math.sin(ph) * math.sin(th), r * math.cos(th)])
    rho = -float(np.dot(pop, n))
    return math.sqrt(1 - rho * rho), rho * n, n


def heat_sphere_circle_error(dx, method, boundary_type=0):
    """SphereCircleIBC (HeatProblemsWithIBC.cpp:88-283) through the oracle: u = cos(phi) = z on
    the unit sphere decays as exp(-2t); Dirichlet circle, boundary order 2; method 0 explicit
    (dt = 0.1 dx^2), 1 backward Euler, 2 Crank-Nicolson (dt = 0.1 dx), both adjusted to an
    integer number of steps to t = 0.1 (:118-129); HeatWithIBC::TimeStep and SetDirichletValue
    (problems/HeatWithIBC.cpp:50-100).  Returns the l_inf error at the plot points (:24-40)."""
    R, c, n = heat_circle_params(boundary_type)
    ibc = ol.circle3d_desc(R, c, n, dx, boundary_order=2)
    ibc.boundary_type[0] = boundary_type
    P = ol.RefProblem(ol.sphere_desc(), [ibc], 3, dx)
    rows = P.rows()
    T = HEAT_FINAL_TIME
    dt = 0.1 * dx if method > 0 else 0.1 * dx * dx
    steps = math.ceil(T / dt)
    dt = T / steps
    f = lambda x: x[:, 2]
    u = f(rows["point"])
    dirichlet = rows["kind"] == 2
    fd = f(rows["point"][dirichlet])
    for k in range(steps):
        t = (k + 1) * dt
        if method == 0:
            u = P.csr_multiply(1, u + dt * P.csr_multiply(0, u))
            u[dirichlet] = math.exp(-2 * t) * fd
        else:
            if method == 2:
                u = P.apply(1.0, 0.5 * dt, u)
            u = np.array(u, copy=True)
            u[dirichlet] = math.exp(-2 * t) * fd
            u, _ = P.solve(1.0, -(1.0 if method == 1 else 0.5) * dt, u)
    ptr, idx, val = P.csr(4)
    up = ol.csr_matvec(ptr, idx, val, u)
    return float(np.max(np.abs(up - math.exp(-2 * T) * f(P.xp()))))


# HeatProblems.cpp:156-158, problem 3 (the sphere): explicit, implicit Euler
GOLDEN_HEAT_SPHERE = {False: 2.39477, True: 2.08643}


def heat_sphere_error(dx, implicit):
    """Sphere (convergence_studies/HeatProblems/HeatProblems.cpp:125-145) through the oracle:
    u = cos(phi) = z decays as exp(-2t) to t = 0.1 with dt = 0.2 dx^2 adjusted to an integer
    number of steps (problems/Heat.cpp:118-120); Heat::TimeStep (:77-92) explicit
    u = E (u + dt L u) or implicit Euler Solve(1, -dt); l_inf error at the plot points (:54-77)."""
    P = ol.RefProblem(ol.sphere_desc(), [], 3, dx)
    T = 0.1
    dt = 0.2 * dx * dx
    steps = math.ceil(T / dt)
    dt = T / steps
    u = P.rows()["point"][:, 2].copy()
    if not implicit:
        import scipy.sparse as sp

        Lm = sp.csr_matrix(tuple(reversed(P.csr(2))), shape=(P.N, P.N))
        Em = sp.csr_matrix(tuple(reversed(P.csr(3))), shape=(P.N, P.N))
    for _ in range(steps):
        if implicit:
            u, _ = P.solve(1.0, -dt, u)
        else:
            u = Em @ (u + dt * (Lm @ u))
    ptr, idx, val = P.csr(4)
    up = ol.csr_matvec(ptr, idx, val, u)
    return float(np.max(np.abs(up - math.exp(-2 * T) * P.xp()[:, 2])))


# PoissonProblemsWithIBC.cpp:383-386: problems 3 / 6 (freeze_nearest) and 4 / 7 (DOF-subset nodes)
GOLDEN_SPHERE_CIRCLE_NEAREST = {True: [0.945984, 0.82667, 0.98775, 0.703821, 1.18035, 1.12101, 0.867009, 1.09471,
                                       0.962311, 0.786675],
                                False: [0.626507, 0.64894, 0.659936, 0.804202, 0.608543, 0.790434, 0.892918, 0.639867,
                                        0.666589, 0.727743]}
GOLDEN_SPHERE_POINT_NEAREST = {True: [2.15041, 2.23765, 0.959175, 0.911574, 1.21328, 2.55332, 1.55977, 1.03094, 1.15633,
                                      1.03559],
                               False: [2.15603, 1.17371, 0.763936, 0.639966, 0.838463, 0.896607, 0.640536, 0.59289,
                                       0.304371, 1.15492]}


def circle3d_plot_points(R, centre, normal, n_points=100):
    """Surface::paramCircle3D (src/Surface.cpp:1881-1904) with ComputeOrthogonalBasis (:442-460)."""
    nrm = np.asarray(normal, np.float64)
    if abs(nrm[0]) > abs(nrm[1]):
        t1 = np.array([-nrm[2], 0.0, nrm[0]])
    else:
        t1 = np.array([0.0, nrm[2], -nrm[1]])
    t2 = np.cross(nrm, t1)
    t1 = t1 / math.sqrt(float(np.dot(t1, t1)))
    t2 = t2 / math.sqrt(float(np.dot(t2, t2)))
    th = np.arange(n_points) * (2 * math.pi / (n_points - 1))
    return np.asarray(centre)[None, :] + R * (np.cos(th)[:, None] * t1[None, :] + np.sin(th)[:, None] * t2[None, :])


def nearest_baseline_error(spec, dx, freeze):
    """PoissonWithIBCNearest (problems/PoissonWithIBCNearest.cpp:5-89) on a convergence-study
    problem: identity rows at Tube::NearestTubeIndex of the IBC's plot points (freeze_nearest) or at the
    IBC DOF subset's nodes, holding the exact solution there; f at the closest points
    elsewhere; error at the plot points through the plain plot interpolation.  Solved
    matrix-free by scipy's BiCGStab to relative residual 1e-10 with the reference's diagonal
    preconditioner m + n L_qq (src/GeneralizedBiCGStabSystem.h:281-340)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    P = ol.RefProblem(spec["surface"], spec["ibcs"], 3, dx)
    P0 = ol.RefProblem(spec["surface"], [], 3, dx)
    t = P0.tube()
    N = P0.N
    exact = spec["exact"]
    if freeze:
        pts = spec["ibc_xp"]
        key = np.round((pts - P0.xstart) / dx).astype(np.int64)
        rec = (key[:, 0] * P0.N1d + key[:, 1]) * P0.N1d + key[:, 2]
        order = np.argsort(t["rec"])
        pos = np.searchsorted(t["rec"][order], rec)
        idx = order[pos]
        assert np.array_equal(t["rec"][idx], rec)
        vals = exact(pts)
    else:
        sub = P.ibc_subsets(0)
        idx, vals = sub["dof_set"], exact(sub["dof_cp"])
    b = spec["f"](t["cp"])
    b[idx] = vals
    Lm = sp.csr_matrix(tuple(reversed(P0.csr(2))), shape=(N, N))
    Em = sp.csr_matrix(tuple(reversed(P0.csr(3))), shape=(N, N)).tolil()
    ident = np.unique(idx)
    for k in ident:
        Em.rows[k] = [int(k)]
        Em.data[k] = [1.0]
    Em = Em.tocsr()
    ld = Lm.diagonal()
    Loff = (Lm - sp.diags(ld)).tocsr()
    m, n = spec["m"], spec["n"]
    is_id = np.zeros(N, bool)
    is_id[ident] = True

    def mv(x):  # GeneralizedBiCGStabSystem::Multiply (src/GeneralizedBiCGStabSystem.h:191-233)
        y = m * x + n * (ld * x + Loff @ (Em @ x))
        y[is_id] = x[is_id]
        return y

    d = np.where(is_id, 1.0, m + n * ld)
    A = spla.LinearOperator((N, N), matvec=mv, dtype=np.float64)
    M = spla.LinearOperator((N, N), matvec=lambda r: r / d, dtype=np.float64)
    u, info = spla.bicgstab(A, b, rtol=1e-10, atol=0.0, maxiter=100000, M=M)
    assert info == 0
    ptr, pidx, pval = P0.csr(4)
    return float(np.max(np.abs(ol.csr_matvec(ptr, pidx, pval, u) - exact(P0.xp()))))


def build_rhs(rows, f, g):
    """PoissonWithIBC::GetRHS (problems/PoissonWithIBC.cpp:92-133) from the exported row layout."""
    kind, ibc, pt = rows["kind"], rows["ibc"], rows["point"]
    b = np.zeros(len(kind))
    m = (kind == 0) | (kind == 1)
    b[m] = f(pt[m])
    d = kind == 2
    if d.any():
        for c in np.unique(ibc[d]):
            sel = d & (ibc == c)
            b[sel] = g(int(c), pt[sel])
    return b


def convergence_order(errors, dxs):
    """Helpers::ConvergenceOrder / AverageConvergenceOrder (src/Helpers.cpp:446-463)."""
    orders = [math.log(errors[i - 1] / errors[i]) / math.log(dxs[i - 1] / dxs[i]) for i in range(1, len(errors))]
    return sum(orders) / len(orders), orders


def oracle_error(spec, dx):
    P = ol.RefProblem(spec["surface"], spec["ibcs"], 3, dx)
    rows = P.rows()
    b = build_rhs(rows, spec["f"], spec["g"] or (lambda c, x: 0.0))
    u, st = P.solve(spec["m"], spec["n"], b)
    ptr, idx, val = P.csr(4)
    uplot = ol.csr_matvec(ptr, idx, val, u)
    err = float(np.max(np.abs(uplot - spec["exact"](P.xp()))))
    return err, st
