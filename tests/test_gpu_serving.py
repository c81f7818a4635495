"""Continuous batching: requests admitted into free slots of a running 32-slot
mixed-precision solver.

Tolerances: every served solution within 1e-8 relative l_inf of the FP64
device solve of the same right-hand side (tol 1e-12); the same request served
alone and in the mix agree within 1e-8 relative l_inf (reliable updates fall at
different points of its iteration in the two runs, so the bits may differ)."""
import numpy as np
import pytest

import studies as S
from test_gpu_setup import two_circle_ibcs

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _setup(gpu, dx=0.05):
    T = gpu.Tube(gpu.desc(gpu.SPHERE, [1.0]), 3, dx)
    O = gpu.OpSet(T, two_circle_ibcs(gpu, dx, 2))
    rows = O.rows()
    return T, O, rows


def _rhs(rows, vals):
    return S.build_rhs(rows, lambda x: np.zeros(len(x)), lambda c, x: np.full(len(x), vals[c]))


def test_server_mix_matches_fp64_and_alone(gpu):
    T, O, rows = _setup(gpu)
    rng = np.random.default_rng(21)
    n_req = 45  # more than 32: later requests are admitted while others run
    vals = rng.uniform(0, 1, size=(n_req, 2))
    B = [_rhs(rows, v) for v in vals]
    srv = gpu.Server(O, 0.0, -1.0)
    for k in range(n_req):
        srv.submit(B[k], k)
    out = srv.drain()
    assert sorted(out) == list(range(n_req))
    ref = gpu.Solver(O, 0.0, -1.0, kslots=32)
    X64, _ = ref.solve(np.stack(B[:32]), tol=1e-12, precision=0)
    X64b, _ = ref.solve(np.stack(B[32:]), tol=1e-12, precision=0)
    X64 = np.concatenate([X64, X64b])
    for k in range(n_req):
        x, st = out[k]
        assert st["status"] == 0
        assert st["rel_residual"] <= 1e-10
        assert _rel(x, X64[k]) <= 1e-8
    # request 40 (admitted mid-stream) alone in a fresh server
    alone = gpu.Server(O, 0.0, -1.0)
    alone.submit(B[40], 40)
    xa, sa = alone.drain()[40]
    assert sa["status"] == 0
    assert _rel(out[40][0], xa) <= 1e-8


def test_server_interleaved_submission(gpu):
    """Requests submitted between steps (as a serving loop would) all finish."""
    T, O, rows = _setup(gpu, dx=0.1)
    rng = np.random.default_rng(5)
    srv = gpu.Server(O, 0.0, -1.0)
    got = {}
    for k in range(20):
        srv.submit(_rhs(rows, rng.uniform(0, 1, 2)), k)
        srv.step()
        while (r := srv.poll()) is not None:
            got[r[0]] = r[2]
    got.update({k: v[1] for k, v in srv.drain().items()})
    assert sorted(got) == list(range(20))
    assert all(v["status"] == 0 and v["latency"] > 0 for v in got.values())


def test_server_plain_fp64_mode(gpu):
    """A server on the plain FP64 path (precision 0) returns the FP64 solve's results."""
    T, O, rows = _setup(gpu, dx=0.1)
    rng = np.random.default_rng(9)
    B = [_rhs(rows, rng.uniform(0, 1, 2)) for _ in range(40)]
    srv = gpu.Server(O, 0.0, -1.0, precision=0)
    for k, b in enumerate(B):
        srv.submit(b, k)
    out = srv.drain()
    ref = gpu.Solver(O, 0.0, -1.0, kslots=1)
    for k in (0, 17, 39):
        x, st = out[k]
        assert st["status"] == 0 and st["fp64_fallback"] == 0
        x64, _ = ref.solve(B[k], tol=1e-12, precision=0)
        assert _rel(x, x64[0]) <= 1e-9


@pytest.mark.parametrize("precision", [1, 0])
def test_server_two_concurrent_batches(gpu, precision):
    """A server over two 32-slot batches on their own streams (cpm_server_create_batches):
    80 requests, each within 1e-8 of its FP64 solve (tol 1e-12); with device right-hand
    sides and destinations as well as host ones."""
    import torch

    T, O, rows = _setup(gpu, dx=0.05)
    rng = np.random.default_rng(33)
    n_req = 80
    B = np.stack([_rhs(rows, rng.uniform(0, 1, 2)) for _ in range(n_req)])
    srv = gpu.Server(O, 0.0, -1.0, precision=precision, batches=2)
    b_dev = torch.from_numpy(B[40:]).cuda()
    x_dev = torch.zeros_like(b_dev)
    torch.cuda.synchronize()
    for k in range(40):
        srv.submit(B[k], k)
    for k in range(40, n_req):
        srv.submit_device(b_dev[k - 40].data_ptr(), x_dev[k - 40].data_ptr(), k)
    out = srv.drain()
    assert sorted(out) == list(range(n_req))
    xd = x_dev.cpu().numpy()
    ref = gpu.Solver(O, 0.0, -1.0, kslots=32)
    for lo in range(0, n_req, 32):
        X64, _ = ref.solve(B[lo:lo + 32], tol=1e-12, precision=0)
        for j in range(len(X64)):
            k = lo + j
            x, st = out[k]
            assert st["status"] == 0 and st["rel_residual"] <= 1e-10
            got = x if k < 40 else xd[k - 40]
            assert _rel(got, X64[j]) <= 1e-8


def test_server_pipelined_steps(gpu):
    """cpm_server_step_async: each call harvests what the previous one launched and
    returns with the next graphs running; host and device destinations give every
    request within 1e-8 of its FP64 solve, like the synchronous steps, and a
    request's result appears one call later than with them."""
    import torch

    T, O, rows = _setup(gpu, dx=0.1)
    rng = np.random.default_rng(21)
    B = np.stack([_rhs(rows, rng.uniform(0, 1, 2)) for _ in range(48)])
    b_dev = torch.from_numpy(B[24:]).cuda()
    x_dev = torch.zeros_like(b_dev)
    torch.cuda.synchronize()
    out = {}
    for pipelined in (True, False):
        srv = gpu.Server(O, 0.0, -1.0, batches=2)
        for k in range(24):
            srv.submit(B[k], k)
        for k in range(24, 48):
            srv.submit_device(b_dev[k - 24].data_ptr(), x_dev[k - 24].data_ptr(), k)
        out[pipelined] = srv.drain(pipelined=pipelined)
        xd = x_dev.cpu().numpy()
        for k in range(24, 48):
            out[pipelined][k] = (xd[k - 24].copy(), out[pipelined][k][1])
        x_dev.zero_()
        torch.cuda.synchronize()
    ref = gpu.Solver(O, 0.0, -1.0)
    for pipelined in (True, False):
        assert sorted(out[pipelined]) == list(range(48))
        assert all(v[1]["status"] == 0 for v in out[pipelined].values())
        for k in (0, 23, 24, 47):
            x64, _ = ref.solve(B[k], tol=1e-12, precision=0)
            assert _rel(out[pipelined][k][0], x64[0]) <= 1e-8
    # the first pipelined call only launches; the synchronous call already harvests
    srv = gpu.Server(O, 0.0, -1.0)
    srv.submit(np.zeros(O.D), 0)  # zero right-hand side: done at its start
    assert srv.step(pipelined=True)[2] == 0
    assert srv.step(pipelined=True)[2] == 1 and srv.poll()[0] == 0
    srv.submit(np.zeros(O.D), 1)
    assert srv.step()[2] == 1 and srv.poll()[0] == 1
