"""Device operator apply and BiCGStab solves against the oracle.

The device operator is built from the oracle's closest points (tube, IBC
closest points and cp-bar), so both sides solve the same system bit for bit.

Tolerances (written here, used below):
  apply, FP64:               relative l_inf <= 1e-14 (only summation order differs)
  plain FP64 solve vs oracle: relative l_inf <= 1e-10, both sides solved to
                              ||r|| <= 1e-12 ||b|| (iterates differ by rounding)
  FP32-inner + FP64 refinement vs FP64 oracle: relative l_inf <= 1e-8
"""
import math

import numpy as np
import pytest

import studies as S
from test_gpu_parity_c2 import same_cp_pair
from test_gpu_setup import two_circle_ibcs

pytestmark = pytest.mark.gpu

SOLVE_TOL = 1e-12     # relative residual of both sides in the FP64 parity solves
FP64_PARITY = 1e-10   # relative l_inf of the FP64 device solution against the oracle's


def _pair(gpu, oracle, dx, ibc=False, order=2):
    if ibc:
        return same_cp_pair(gpu, oracle, dx, two_circle_ibcs(oracle, dx, order), two_circle_ibcs(gpu, dx, order))
    return same_cp_pair(gpu, oracle, dx, [], [])


def _rel_inf(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("ibc", [False, True])
@pytest.mark.parametrize("mn", [(1.0, -1.0), (0.0, -1.0), (1.0, -0.01)])
def test_apply_matches_oracle(gpu, oracle, ibc, mn):
    P, T, O, gr = _pair(gpu, oracle, 0.1, ibc)
    rng = np.random.default_rng(7)
    x_ref = rng.standard_normal(P.D)
    y_ref = P.apply(mn[0], mn[1], x_ref)
    x_gpu = np.empty(O.D)
    x_gpu[gr] = x_ref
    y_gpu = O.apply(mn[0], mn[1], x_gpu)[0]
    assert _rel_inf(y_gpu[gr], y_ref) <= 1e-14


def test_fp32_batched_apply_matches_fp64(gpu):
    """The FP32 32-RHS apply (E pass, IBC patch pass, L pass) against the
    FP64 apply of the same inputs: relative l_inf <= 1e-5 per batch (FP32
    rounding of 84 FMAs per row and the 1/dx^2 Laplacian)."""
    import torch

    dx = 0.05
    T = gpu.Tube(gpu.desc(gpu.SPHERE, [1.0]), 3, dx)
    O = gpu.OpSet(T, two_circle_ibcs(gpu, dx))
    gen = torch.Generator().manual_seed(4)
    x = (torch.rand((O.D, 32), generator=gen, dtype=torch.float32) * 2 - 1).cuda()
    x64 = x.double()
    t, y = torch.empty_like(x), torch.empty_like(x)
    t64, y64 = torch.empty_like(x64), torch.empty_like(x64)
    torch.cuda.synchronize()
    O.apply_device(0.0, -1.0, 32, True, x.data_ptr(), t.data_ptr(), y.data_ptr())
    O.apply_device(0.0, -1.0, 32, False, x64.data_ptr(), t64.data_ptr(), y64.data_ptr())
    gpu.sync()
    a, b = y.cpu().double().numpy(), y64.cpu().numpy()
    assert _rel_inf(a, b) <= 1e-5
    assert _rel_inf(t.cpu().double().numpy(), t64.cpu().numpy()) <= 1e-5


def test_plain_fp64_solve_matches_oracle_screened_poisson(gpu, oracle):
    """Screened Poisson -Delta_S u + u = f on the unit sphere, f = 3z (exact u = z), dx = 0.1."""
    dx = 0.1
    P, T, O, gr = _pair(gpu, oracle, dx)
    rows = P.rows()
    b = 3.0 * rows["point"][:, 2]
    x_ref, st_ref = P.solve(1.0, -1.0, b, tol=SOLVE_TOL)
    bg = np.empty(O.D)
    bg[gr] = b
    x_gpu, st = gpu.Solver(O, 1.0, -1.0).solve(bg, tol=SOLVE_TOL)
    assert st[0]["status"] == 0
    assert abs(st[0]["iterations"] - st_ref["iterations"]) <= 2
    assert _rel_inf(x_gpu[0][gr], x_ref) <= FP64_PARITY
    # accuracy against the analytic solution, measured like the reference's studies:
    # interpolated to the surface parameterisation points (src/Helpers.cpp:97-103)
    xp = P.xp()
    cols, vals = T.interp_query(xp)
    uplot = np.sum(vals * x_gpu[0][cols], axis=1)
    assert np.max(np.abs(uplot - xp[:, 2])) < 5e-3


def test_plain_fp64_ibc_solve_matches_oracle(gpu, oracle):
    dx = 0.05
    P, T, O, gr = _pair(gpu, oracle, dx, ibc=True)
    rows = P.rows()
    b = S.build_rhs(rows, lambda x: np.zeros(len(x)), lambda c, x: np.full(len(x), 1.0 if c == 0 else 0.0))
    x_ref, st_ref = P.solve(0.0, -1.0, b, tol=SOLVE_TOL)
    bg = np.empty(O.D)
    bg[gr] = b
    x_gpu, st = gpu.Solver(O, 0.0, -1.0).solve(bg, tol=SOLVE_TOL)
    assert st[0]["status"] == 0
    assert _rel_inf(x_gpu[0][gr], x_ref) <= FP64_PARITY


@pytest.mark.parametrize("kslots", [1, 32])
@pytest.mark.parametrize("precond,sweeps", [(0, 0), (2, 1), (2, 25)])
def test_preconditioners_match_oracle(gpu, oracle, precond, sweeps, kslots):
    """Identity and damped-Jacobi preconditioning (src/GeneralizedBiCGStabSystem.h:350-385)
    on the backward-Euler heat operator with the two circle IBCs at dx = 0.1."""
    dx = 0.1
    P, T, O, gr = _pair(gpu, oracle, dx, ibc=True)
    rows = P.rows()
    b = S.build_rhs(rows, lambda x: x[:, 0], lambda c, x: np.full(len(x), 0.25 + 0.5 * c))
    dt = dx * dx
    x_ref, st_ref = P.solve(1.0, -dt, b, precond=precond, precond_iters=sweeps, tol=SOLVE_TOL)
    bg = np.empty(O.D)
    bg[gr] = b
    x_gpu, st = gpu.Solver(O, 1.0, -dt, kslots=kslots).solve(bg, precond=precond, precond_iters=sweeps, tol=SOLVE_TOL)
    assert st[0]["status"] == 0
    assert abs(st[0]["iterations"] - st_ref["iterations"]) <= 1
    assert _rel_inf(x_gpu[0][gr], x_ref) <= FP64_PARITY


def test_jacobi_rejects_fp32(gpu, oracle):
    P, T, O, gr = _pair(gpu, oracle, 0.1)
    with pytest.raises(gpu.CpmError):
        gpu.Solver(O, 1.0, -0.01).solve(np.ones(O.D), precision=1, precond=2, precond_iters=10)


def test_mixed_precision_matches_fp64_oracle(gpu, oracle):
    dx = 0.05
    P, T, O, gr = _pair(gpu, oracle, dx, ibc=True)
    rows = P.rows()
    rng = np.random.default_rng(3)
    vals = rng.uniform(0, 1, size=2)
    b = S.build_rhs(rows, lambda x: np.zeros(len(x)), lambda c, x: np.full(len(x), vals[c]))
    x_ref, _ = P.solve(0.0, -1.0, b, tol=1e-12)
    bg = np.empty(O.D)
    bg[gr] = b
    x_gpu, st = gpu.Solver(O, 0.0, -1.0, kslots=32).solve(bg, precision=1, tol=1e-10)
    assert st[0]["status"] == 0 and st[0]["refinements"] >= 2
    assert _rel_inf(x_gpu[0][gr], x_ref) <= 1e-8


def test_batched_equals_alone_bitwise(gpu, oracle):
    """A right-hand side gives the same bits alone or in a batch of 32 (per-slot arithmetic)."""
    dx = 0.1
    P, T, O, gr = _pair(gpu, oracle, dx, ibc=True)
    rows = P.rows()
    rng = np.random.default_rng(11)
    B = np.stack([S.build_rhs(rows, lambda x: np.zeros(len(x)), lambda c, x, v=rng.uniform(0, 1, 2): np.full(len(x), v[c]))
                  for _ in range(32)])
    Bg = np.empty_like(B)
    Bg[:, gr] = B
    sv = gpu.Solver(O, 0.0, -1.0, kslots=32)
    for prec in (0, 1):
        xb, _ = sv.solve(Bg, precision=prec)
        for j in (0, 17, 31):
            xa, _ = sv.solve(Bg[j:j + 1], precision=prec)
            assert np.array_equal(xa[0], xb[j])


def test_golden_order_through_device_solver(gpu, oracle):
    """ShiftedPoissonSphere convergence order (PoissonProblems.cpp:169) with the device FP64 path."""
    errs = []
    for dx in S.DX_3D:
        spec = S.shifted_poisson_sphere(dx)
        T = gpu.Tube(gpu.desc(gpu.SPHERE, [1.0]), 3, dx)
        O = gpu.OpSet(T)
        rows = O.rows()
        b = spec["f"](rows["point"])
        x, st = gpu.Solver(O, 1.0, 1.0).solve(b)
        P = oracle.RefProblem(oracle.sphere_desc(), [], 3, dx)
        xp = P.xp()
        cols, vals = T.interp_query(xp)
        uplot = np.sum(vals * x[0][cols], axis=1)
        errs.append(float(np.max(np.abs(uplot - spec["exact"](xp)))))
    order, _ = S.convergence_order(errs, S.DX_3D)
    assert abs(order - S.GOLDEN_SHIFTED_POISSON_SPHERE) < 1e-2


@pytest.mark.parametrize("dx", [0.05, 0.025])
def test_fp32_batched_apply_against_fp64_and_alignment(gpu, dx):
    """The FP32 32-slot apply (E pass, IBC patch pass, L pass) of x in [-1, 1]:
    within 1e-5 of the FP64 32-slot apply of the same values (relative to max |y|;
    the FP32 row keeps its O(1/dx^2) terms apart, so the error stays near FP32
    rounding); for an input 4 bytes past a 16-byte boundary (the L pass then
    reads slots one at a time instead of four) the same E-pass bits and y within
    1e-6, on two consecutive calls."""
    import torch

    O = gpu.OpSet(gpu.Tube(gpu.desc(gpu.SPHERE, [1.0]), 3, dx), two_circle_ibcs(gpu, dx))
    gen = torch.Generator().manual_seed(9)
    x = (torch.rand((O.D, 32), generator=gen, dtype=torch.float32) * 2 - 1).cuda()
    buf = torch.empty(O.D * 32 + 4, dtype=torch.float32, device="cuda")
    xm = buf[1:1 + O.D * 32].view(O.D, 32)  # 4 bytes past a 16-byte boundary
    xm.copy_(x)
    assert xm.data_ptr() % 16 == 4
    t_a, y_a = torch.full_like(x, float("nan")), torch.empty_like(x)
    t_m, y_m = torch.full_like(x, float("nan")), torch.empty_like(x)
    x64 = x.double()
    t64, y64 = torch.empty_like(x64), torch.empty_like(x64)
    torch.cuda.synchronize()
    for _ in range(2):
        O.apply_device(0.0, -1.0, 32, True, x.data_ptr(), t_a.data_ptr(), y_a.data_ptr())
        O.apply_device(0.0, -1.0, 32, True, xm.data_ptr(), t_m.data_ptr(), y_m.data_ptr())
        gpu.sync()
        assert torch.equal(t_a, t_m)
        assert _rel_inf(y_m.cpu().double().numpy(), y_a.cpu().double().numpy()) <= 1e-6
    O.apply_device(0.0, -1.0, 32, False, x64.data_ptr(), t64.data_ptr(), y64.data_ptr())
    gpu.sync()
    assert _rel_inf(y_a.cpu().double().numpy(), y64.cpu().numpy()) <= 1e-5
    assert _rel_inf(t_a.cpu().double().numpy(), t64.cpu().numpy()) <= 1e-6
