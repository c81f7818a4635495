"""Request serving over several device-resident surfaces.

No counterpart in the reference, whose solves are one blocking call each
(src/Solver.cpp:104-113).  Each surface keeps its tube and operator (with its
fixed IBC curves) on the device.  Requests arrive over time:

* ``laplace``: an IBC Laplace solve with given Dirichlet values per curve
  (PoissonWithIBC with f = 0, problems/PoissonWithIBC.cpp:162-192), served by
  the surface's continuous-batching server (32 slots, FP32 iterations with
  FP64 reliable updates; slots refill as solves finish);
* ``geodesic``: heat-method distance from a tube node
  (GeodesicDistance::ComputeDistance, problems/GeodesicDistance.cpp:11-69),
  which carries its own point-IBC operator and runs as one pipeline.

A surface's server is admitted only while the device has room for it (its
estimated bytes within the HBM budget); an idle server is released to make
room for another surface's.  A surface starts on the mixed-precision server;
once a quarter of its finished requests (at least 8 finished) needed the FP64
re-solve, it drains that server and continues on a plain FP64 32-slot server.
Latency is measured from a request's arrival to the harvest of its result.
"""
import heapq
import time

import numpy as np

from . import DIAGONAL, Geodesic, OpSet, Server, Solver, device_info

MAX_SLOTS = 32


class ServedSurface:
    """A device-resident surface: its tube, operator (with IBC curves) and, while
    admitted, its server."""

    def __init__(self, name, tube, ibcs, m=0.0, n=-1.0, tol=1e-10):
        self.name, self.tube = name, tube
        self.opset = OpSet(tube, ibcs)
        self.rows = self.opset.rows()
        self.n_ibc = len(ibcs)
        self.m, self.n, self.tol = m, n, tol
        self.server = None
        self.bytes = Server.device_bytes(self.opset)
        self.waiting = []  # (request id, rhs, arrival time) not yet submitted
        self.active = False  # requests in the server's slots or queue
        self.precision = 1  # the server's precision: 1 mixed, 0 plain FP64
        self.finished = 0
        self.fallbacks = 0
        self.switch_pending = False
        self.inflight = 0  # submitted to the server and not yet harvested
        self._cp = None

    def rhs(self, values):
        """PoissonWithIBC::GetRHS with f = 0: Dirichlet value values[c] on curve c."""
        b = np.zeros(self.opset.D)
        d = self.rows["kind"] == 2
        b[d] = np.asarray(values, np.float64)[self.rows["ibc"][d]]
        return b

    def closest_points(self):
        if self._cp is None:
            self._cp = self.tube.export()["cp"]
        return self._cp


class ServingLoop:
    """Serves a stream of requests over ServedSurfaces.

    hbm_budget: bytes the servers may hold together (default: the device's free
    memory when the loop is created, less ``reserve`` bytes)."""

    def __init__(self, surfaces, hbm_budget=None, reserve=1 << 30, geodesic_precision=1, dt_scale=1.0):
        self.surfaces = {s.name: s for s in surfaces}
        if hbm_budget is None:
            hbm_budget = max(0, device_info()["free"] - reserve)
        self.budget = int(hbm_budget)
        self.geodesic_precision = geodesic_precision
        self.dt_scale = dt_scale
        self.admissions = 0
        self.evictions = 0
        self.precision_switches = 0

    def _held(self):
        return sum(s.bytes for s in self.surfaces.values() if s.server is not None)

    def _admit(self, s):
        """Create s's server if the HBM budget allows, releasing idle servers first."""
        if s.server is not None:
            return True
        if s.bytes > self.budget:
            raise MemoryError(f"surface {s.name}: a server needs {s.bytes} bytes, the budget is {self.budget}")
        if self._held() + s.bytes > self.budget:
            for o in self.surfaces.values():
                if o is not s and o.server is not None and not o.active and not o.waiting:
                    o.server = None
                    self.evictions += 1
                    if self._held() + s.bytes <= self.budget:
                        break
        if self._held() + s.bytes > self.budget:
            return False
        s.server = Server(s.opset, s.m, s.n, tol=s.tol, precision=s.precision)
        self.admissions += 1
        return True

    def run(self, requests, keep_solutions=False):
        """requests: list of dicts {id, t (arrival, seconds from start), surface,
        kind ('laplace' | 'geodesic'), values | source}.  Returns {id: record}
        with arrival, completion, latency, kind, surface, stats (and x if kept)."""
        order = sorted(requests, key=lambda r: r["t"])
        heap = [(r["t"], i, r) for i, r in enumerate(order)]
        heapq.heapify(heap)
        geo_wait = []
        out = {}
        arrival = {}
        t0 = time.perf_counter()
        total = len(order)
        while len(out) < total:
            now = time.perf_counter() - t0
            while heap and heap[0][0] <= now:
                _, _, r = heapq.heappop(heap)
                arrival[r["id"]] = r["t"]
                s = self.surfaces[r["surface"]]
                if r["kind"] == "laplace":
                    s.waiting.append((r["id"], s.rhs(r["values"]), r["t"]))
                else:
                    geo_wait.append(r)
            progressed = False
            for s in self.surfaces.values():
                if s.switch_pending and s.server is not None and not s.active:
                    s.server = None
                    s.precision = 0
                    s.switch_pending = False
                    self.precision_switches += 1
                if s.waiting and not s.switch_pending and self._admit(s):
                    # at most two batches in the server, so a precision switch takes
                    # effect within two batches
                    take = max(0, min(len(s.waiting), 2 * MAX_SLOTS - s.inflight))
                    for rid, b, _ in s.waiting[:take]:
                        s.server.submit(b, rid)
                    s.waiting = s.waiting[take:]
                    s.inflight += take
                    s.active = s.active or take > 0
                if s.server is not None and s.active:
                    a, q, _ = s.server.step()
                    s.active = (a + q) > 0
                    progressed = True
                    while True:
                        res = s.server.poll(want_x=keep_solutions)
                        if res is None:
                            break
                        rid, x, st = res
                        done = time.perf_counter() - t0
                        rec = dict(kind="laplace", surface=s.name, arrival=arrival[rid], completion=done,
                                   latency=done - arrival[rid], stats=st, precision=s.precision)
                        s.finished += 1
                        s.inflight -= 1
                        s.fallbacks += int(st.get("fp64_fallback", 0))
                        if s.precision == 1 and s.finished >= 8 and 4 * s.fallbacks >= s.finished:
                            s.switch_pending = True
                        if keep_solutions:
                            rec["x"] = x
                        out[rid] = rec
            if geo_wait:
                r = geo_wait.pop(0)
                s = self.surfaces[r["surface"]]
                g = Geodesic(s.tube, r["source"])
                dx = s.tube.dx
                # a surface whose Laplace solves left mixed precision runs its geodesics in FP64 too
                prec = min(self.geodesic_precision, s.precision)
                phi, its = g.run(self.dt_scale * dx * dx, precision=prec, tol=s.tol)
                done = time.perf_counter() - t0
                rec = dict(kind="geodesic", surface=s.name, arrival=r["t"], completion=done, latency=done - r["t"],
                           stats=dict(iterations=its))
                if keep_solutions:
                    rec["x"] = phi
                out[r["id"]] = rec
                progressed = True
            if not progressed and heap:
                time.sleep(max(0.0, min(0.002, heap[0][0] - (time.perf_counter() - t0))))
        return out


def poisson_stream(surfaces, count, rate, geodesic_every=32, seed=0):
    """A seeded request stream: exponential inter-arrival times of mean 1/rate
    (all at t = 0 if rate is 0); surfaces drawn uniformly; one request in
    ``geodesic_every`` (at a seeded offset) a geodesic from a random tube node,
    the rest IBC Laplace solves with Dirichlet values U[0,1] per curve."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=count)) if rate > 0 else np.zeros(count)
    by = {s.name: s for s in surfaces}
    names = list(by)
    off = int(rng.integers(geodesic_every)) if geodesic_every else -1
    reqs = []
    for i in range(count):
        s = by[names[int(rng.integers(len(names)))]]
        if geodesic_every and i % geodesic_every == off:
            cp = s.closest_points()
            reqs.append(dict(id=i, t=float(t[i]), surface=s.name, kind="geodesic", source=cp[int(rng.integers(len(cp)))]))
        else:
            reqs.append(dict(id=i, t=float(t[i]), surface=s.name, kind="laplace",
                             values=rng.uniform(0, 1, size=s.n_ibc)))
    return reqs


def fp64_one_at_a_time(surfaces, requests, geodesic_precision=0, dt_scale=1.0):
    """The plain FP64 path, one request after another (no batching): seconds per request."""
    by = {s.name: s for s in surfaces}
    solvers = {}
    times = []
    for r in requests:
        s = by[r["surface"]]
        t = time.perf_counter()
        if r["kind"] == "laplace":
            if s.name not in solvers:
                solvers[s.name] = Solver(s.opset, s.m, s.n, kslots=1)
            solvers[s.name].solve(s.rhs(r["values"]), tol=s.tol, precision=0, precond=DIAGONAL)
        else:
            g = Geodesic(s.tube, r["source"])
            g.run(dt_scale * s.tube.dx ** 2, precision=geodesic_precision, tol=s.tol)
        times.append(time.perf_counter() - t)
    return times
