"""The serving loops' host logic (CPU, no device): surfaces whose solvers are
fakes that return x = 2 b after a fixed number of steps, so the tests check what
the loops decide and deliver, not the numbers.  Both loops (run and
run_concurrent) serve every request exactly once with its own result, batch
the requests waiting on one surface, and run the geodesics waiting on one
surface as one batch."""
import threading

import numpy as np
import pytest

from cpm_gb300 import serving as SV


class FakeServer:
    """32 slots; a request finishes after STEPS calls of step() once admitted"""
    STEPS = 3
    created = []

    def __init__(self, opset, m, n, tol=1e-10, precision=1, max_iters=100000):
        self.queue, self.slots, self.done = [], {}, []
        self.precision = precision
        FakeServer.created.append(self)

    def submit(self, b, tag):
        self.queue.append((tag, np.array(b)))

    def step(self):
        while self.queue and len(self.slots) < 32:
            tag, b = self.queue.pop(0)
            self.slots[tag] = [b, 0]
        for tag in list(self.slots):
            self.slots[tag][1] += 1
            if self.slots[tag][1] >= self.STEPS:
                b, k = self.slots.pop(tag)
                self.done.append((tag, 2.0 * b, dict(status=0, iterations=10 * k, fp64_fallback=0, service=0.0)))
        return len(self.slots), len(self.queue), 0

    def poll(self, want_x=True):
        return self.done.pop(0) if self.done else None

    @staticmethod
    def device_bytes(opset, batches=1):
        return 1 << 20


class FakeSolver:
    def __init__(self, opset, m, n, kslots=1):
        pass

    def solve(self, b, tol=1e-10, precision=0, precond=None):
        return 2.0 * np.atleast_2d(b), [dict(status=0, iterations=10)]


class FakeGeodesic:
    calls = []

    def __init__(self, tube, source):
        self.tube, self.src = tube, np.asarray(source)

    def run(self, dt, precision=0, tol=1e-10):
        FakeGeodesic.calls.append(1)
        return np.full(self.tube.N + 2, self.src.sum()), [1, 2, 3, 4]


class FakeGeodesicBatch:
    calls = []

    def __init__(self, tube, sources):
        self.tube, self.src = tube, np.asarray(sources)

    def run(self, dt, tol=1e-10):
        FakeGeodesicBatch.calls.append(len(self.src))
        return (np.stack([np.full(self.tube.N + 5, s.sum()) for s in self.src]),
                np.ones((len(self.src), 4), np.int32))


class FakeTube:
    def __init__(self, N):
        self.N, self.dx = N, 0.1


class FakeOpSet:
    def __init__(self, D):
        self.D = D


def _surface(name, D, n_ibc):
    s = object.__new__(SV.ServedSurface)
    s.name, s.tube, s.opset = name, FakeTube(D - 10), FakeOpSet(D)
    s.rows = {"kind": np.r_[np.zeros(D - 10, int), np.full(10, 2)], "ibc": np.r_[np.zeros(D - 10, int),
                                                                                 np.arange(10) % n_ibc]}
    s.n_ibc, s.m, s.n, s.tol = n_ibc, 0.0, -1.0, 1e-10
    s.server, s.bytes, s.waiting, s.active = None, 1 << 20, [], False
    s.precision, s.finished, s.fallbacks, s.switch_pending = 1, 0, 0, False
    s.inflight_arrival, s.submitted, s.solo, s.fp64_iters, s.mixed_iters = {}, 0, None, None, None
    s._cp = np.arange(3 * (D - 10), dtype=float).reshape(-1, 3)
    s.busy, s.tuning = threading.Lock(), None
    return s


@pytest.fixture
def fakes(monkeypatch):
    monkeypatch.setattr(SV, "Server", FakeServer)
    monkeypatch.setattr(SV, "Solver", FakeSolver)
    monkeypatch.setattr(SV, "Geodesic", FakeGeodesic)
    monkeypatch.setattr(SV, "GeodesicBatch", FakeGeodesicBatch)
    monkeypatch.setattr(SV.ServingLoop, "_worker_stream", staticmethod(lambda: (lambda: (lambda: None))))
    FakeServer.created, FakeGeodesic.calls, FakeGeodesicBatch.calls = [], [], []
    yield


@pytest.mark.parametrize("concurrent", [False, True])
def test_every_request_once_with_its_own_result(fakes, concurrent):
    surfaces = [_surface("a", 60, 2), _surface("b", 80, 3), _surface("c", 40, 1)]
    reqs = SV.poisson_stream(surfaces, 150, rate=0.0, geodesic_every=25, seed=3)
    loop = SV.ServingLoop(surfaces, hbm_budget=1 << 30)
    out = (loop.run_concurrent if concurrent else loop.run)(reqs, keep_solutions=True)
    assert sorted(out) == sorted(r["id"] for r in reqs)
    by = {s.name: s for s in surfaces}
    for r in reqs:
        rec = out[r["id"]]
        s = by[r["surface"]]
        assert rec["surface"] == r["surface"] and rec["kind"] == r["kind"] and rec["latency"] >= 0
        if r["kind"] == "laplace":
            assert np.array_equal(rec["x"], 2.0 * s.rhs(r["values"]))
        else:
            assert np.all(rec["x"] == np.asarray(r["source"]).sum()) and len(rec["x"]) == s.tube.N
    # with every request waiting at once, each surface batched its Laplace requests
    assert all(any(o["mode"] == "batched" for o in out.values() if o["surface"] == s.name and o["kind"] == "laplace")
               for s in surfaces)


@pytest.mark.parametrize("concurrent", [False, True])
def test_waiting_geodesics_of_a_surface_form_one_batch(fakes, concurrent):
    s = _surface("a", 60, 2)
    reqs = [dict(id=k, t=0.0, surface="a", kind="geodesic", source=s._cp[k]) for k in range(40)]
    loop = SV.ServingLoop([s], hbm_budget=1 << 30, geodesic_batch_min=8)
    out = (loop.run_concurrent if concurrent else loop.run)(reqs, keep_solutions=True)
    assert sorted(out) == list(range(40))
    assert FakeGeodesicBatch.calls == [32, 8] and not FakeGeodesic.calls
    assert all(out[k]["x"][0] == s._cp[k].sum() for k in range(40))


@pytest.mark.parametrize("concurrent", [False, True])
def test_few_waiting_geodesics_run_alone(fakes, concurrent):
    """below geodesic_batch_min waiting, each geodesic runs alone (a batch costs as much as 32)"""
    s = _surface("a", 60, 2)
    reqs = [dict(id=k, t=0.0, surface="a", kind="geodesic", source=s._cp[k]) for k in range(5)]
    loop = SV.ServingLoop([s], hbm_budget=1 << 30)
    out = (loop.run_concurrent if concurrent else loop.run)(reqs, keep_solutions=True)
    assert sorted(out) == list(range(5))
    assert not FakeGeodesicBatch.calls and len(FakeGeodesic.calls) == 5
    assert all(out[k]["x"][0] == s._cp[k].sum() for k in range(5))
