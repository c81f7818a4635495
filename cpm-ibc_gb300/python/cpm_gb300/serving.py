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
  which carries its own point-IBC operator and runs as one pipeline; once
  GEO_BATCH_MIN geodesics wait on one surface they run together (up to 32) as one
  batch on a slot-patched operator.

A surface's server is admitted only while the device has room for it (its
estimated bytes within the HBM budget); an idle server is released to make
room for another surface's.

A 32-slot batch costs about the same whether it holds one request or 32, so
requests are solved alone by the plain FP64 path (the reference's algorithm,
one right-hand side) while a surface's server is idle and fewer of them wait
than the break-even count: a 32-slot iteration costs about K32_MIXED (FP32
with FP64 reliable updates) or K32_FP64 one-RHS FP64 iterations, times the
surface's measured ratio of mixed to FP64 iteration counts.  A surface's first
request is always solved alone, which measures its FP64 iteration count; its
mixed-precision server then stops a solve after 6x that many iterations (and
re-solves it in FP64).  The first mixed batch is a probe of PROBE requests
(others are served alone meanwhile); once a quarter of a surface's finished
batched requests (at least two of at least two) needed the FP64 re-solve, it
stops feeding that server, serves its requests alone while it drains, and
continues on a plain FP64 32-slot server.
Latency is measured from a request's arrival to the harvest of its result.
"""
import heapq
import threading
import time

import numpy as np

from . import DIAGONAL, Geodesic, GeodesicBatch, OpSet, Server, Solver, device_info

MAX_SLOTS = 32
PROBE = 2  # requests in a surface's first mixed-precision batch
K32_MIXED = 2.3  # 32-slot FP32 iteration (reliable updates amortised) / one-RHS FP64 iteration
K32_FP64 = 14.0  # 32-slot FP64 iteration / one-RHS FP64 iteration
# geodesics waiting on one surface from which a batch beats solving them one by one: the
# 32-source batch costs the same with 2 or 32 sources (FP64, lane = source), 146.9 s on the
# torus against 6.27 s for one source alone
GEO_BATCH_MIN = 24


class ServedSurface:
    """A device-resident surface: its tube, operator (with IBC curves) and, while
    admitted, its server."""

    def __init__(self, name, tube, ibcs, m=0.0, n=-1.0, tol=1e-10, autotune=True):
        self.name, self.tube = name, tube
        self.opset = OpSet(tube, ibcs)
        # launch shapes of this surface's E passes, timed once and kept with the operator
        self.tuning = self.opset.autotune(reps=10, fp64=True) if autotune else None
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
        self.inflight_arrival = {}  # submitted to the server, not yet harvested: id -> arrival
        self.submitted = 0  # requests ever submitted to a mixed-precision server
        self.solo = None  # one-RHS FP64 solver for requests served alone
        self.fp64_iters = None  # running mean iterations of a solo FP64 solve
        self.mixed_iters = None  # running mean iterations of a batched mixed solve
        self._cp = None
        self.busy = threading.Lock()  # held while a unit of this surface's work runs

    def break_even(self):
        """requests waiting from which a 32-slot batch beats solving them one by one
        (None until the surface's FP64 iteration count is measured)"""
        if self.fp64_iters is None:
            return None
        if self.precision == 0:
            return max(2, int(np.ceil(K32_FP64)))
        ratio = self.mixed_iters / self.fp64_iters if self.mixed_iters else 2.0
        return max(2, int(np.ceil(K32_MIXED * ratio)))

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

    def __init__(self, surfaces, hbm_budget=None, reserve=1 << 30, geodesic_precision=1, dt_scale=1.0,
                 geodesic_batch_min=GEO_BATCH_MIN):
        self.surfaces = {s.name: s for s in surfaces}
        self.geodesic_batch_min = geodesic_batch_min
        if hbm_budget is None:
            hbm_budget = max(0, device_info()["free"] - reserve)
        self.budget = int(hbm_budget)
        self.geodesic_precision = geodesic_precision
        self.dt_scale = dt_scale
        self.admissions = 0
        self.evictions = 0
        self.precision_switches = 0
        self.solo_solves = 0
        self._lock = threading.RLock()  # admissions and counters shared by the worker threads

    def _held(self):
        return sum(s.bytes for s in self.surfaces.values() if s.server is not None)

    def _admit(self, s):
        """Create s's server if the HBM budget allows, releasing idle servers first
        (a server whose surface is in the middle of a unit of work is never released)."""
        if s.server is not None:
            return True
        if s.bytes > self.budget:
            raise MemoryError(f"surface {s.name}: a server needs {s.bytes} bytes, the budget is {self.budget}")
        with self._lock:
            if self._held() + s.bytes > self.budget:
                for o in self.surfaces.values():
                    if o is s or o.server is None or o.active or o.waiting or not o.busy.acquire(blocking=False):
                        continue
                    try:
                        if o.server is not None and not o.active and not o.waiting:
                            o.server = None
                            self.evictions += 1
                    finally:
                        o.busy.release()
                    if self._held() + s.bytes <= self.budget:
                        break
            if self._held() + s.bytes > self.budget:
                return False
            cap = max(200, int(6 * s.fp64_iters)) if (s.precision == 1 and s.fp64_iters) else 100000
            s.server = Server(s.opset, s.m, s.n, tol=s.tol, precision=s.precision, max_iters=cap)
            self.admissions += 1
        return True

    def _solo(self, s, keep_solutions, t0, out):
        """the oldest waiting request of s alone, plain FP64"""
        rid, b, arr = s.waiting.pop(0)
        if s.solo is None:
            s.solo = Solver(s.opset, s.m, s.n, kslots=1)
        t = time.perf_counter()
        x, st = s.solo.solve(b, tol=s.tol, precision=0, precond=DIAGONAL)
        dt = time.perf_counter() - t
        it = float(st[0]["iterations"])
        s.fp64_iters = it if s.fp64_iters is None else 0.7 * s.fp64_iters + 0.3 * it
        with self._lock:
            self.solo_solves += 1
        done = time.perf_counter() - t0
        rec = dict(kind="laplace", surface=s.name, arrival=arr, completion=done, latency=done - arr,
                   stats=dict(st[0], service=dt), precision=0, mode="solo")
        if keep_solutions:
            rec["x"] = x[0]
        out[rid] = rec

    def _step(self, s, keep_solutions, t0, out):
        """one iteration graph of s's server, then its finished requests"""
        a, q, _ = s.server.step()
        s.active = (a + q) > 0
        while True:
            res = s.server.poll(want_x=keep_solutions)
            if res is None:
                break
            rid, x, st = res
            done = time.perf_counter() - t0
            arr = s.inflight_arrival.pop(rid)
            rec = dict(kind="laplace", surface=s.name, arrival=arr, completion=done, latency=done - arr, stats=st,
                       precision=s.precision, mode="batched")
            if s.precision == 1 and not st.get("fp64_fallback"):
                it = float(st["iterations"])
                s.mixed_iters = it if s.mixed_iters is None else 0.7 * s.mixed_iters + 0.3 * it
            s.finished += 1
            s.fallbacks += int(st.get("fp64_fallback", 0))
            if s.precision == 1 and s.fallbacks >= 2 and 4 * s.fallbacks >= s.finished:
                s.switch_pending = True
            if keep_solutions:
                rec["x"] = x
            out[rid] = rec

    def run(self, requests, keep_solutions=False):
        """requests: list of dicts {id, t (arrival, seconds from start), surface,
        kind ('laplace' | 'geodesic'), values | source}.  Returns {id: record}
        with arrival, completion, latency, kind, surface, stats (and x if kept).

        Earliest arrival first: each pass runs the one unit of work (an
        iteration graph of a server, a request solved alone, a batch submitted
        to a server, or a geodesic) whose oldest request arrived first."""
        order = sorted(requests, key=lambda r: r["t"])
        heap = [(r["t"], i, r) for i, r in enumerate(order)]
        heapq.heapify(heap)
        geo_wait = []
        out = {}
        t0 = time.perf_counter()
        total = len(order)
        for s in self.surfaces.values():
            s.inflight_arrival = {}
        while len(out) < total:
            now = time.perf_counter() - t0
            while heap and heap[0][0] <= now:
                _, _, r = heapq.heappop(heap)
                s = self.surfaces[r["surface"]]
                if r["kind"] == "laplace":
                    s.waiting.append((r["id"], s.rhs(r["values"]), r["t"]))
                else:
                    geo_wait.append(r)
            # candidate units of work, keyed by the arrival of their oldest request
            cands = []
            for s in self.surfaces.values():
                c = self._candidate(s, now)
                if c is not None:
                    cands.append((c[0], c[1], s.name, c[2]))
            if geo_wait:
                cands.append((geo_wait[0]["t"], 2, None, "geodesic"))
            if not cands:
                if heap:
                    time.sleep(max(0.0, min(0.002, heap[0][0] - (time.perf_counter() - t0))))
                continue
            _, _, name, what = min(cands)
            if what == "geodesic":
                name0 = geo_wait[0]["surface"]
                take = self._geo_take([r for r in geo_wait if r["surface"] == name0])
                geo_wait = [r for r in geo_wait if r not in take]
                self._geodesics(self.surfaces[name0], take, keep_solutions, t0, out)
                continue
            self._unit(self.surfaces[name], what, keep_solutions, t0, out)
        return out

    def _geo_take(self, waiting):
        """the geodesics to run next from those waiting on one surface (oldest first): up
        to 32 as one batch once geodesic_batch_min wait, else the oldest alone"""
        return waiting[:MAX_SLOTS] if len(waiting) >= self.geodesic_batch_min else waiting[:1]

    def _geodesics(self, s, batch, keep_solutions, t0, out):
        """the waiting geodesics of surface s: one alone (its own point-IBC operator), two or
        more as one batch on a slot-patched operator (GeodesicBatch, FP64).  Results are the
        distances on the tube rows."""
        N = s.tube.N
        if len(batch) == 1:
            r = batch[0]
            # a surface whose Laplace solves left mixed precision runs its geodesics in FP64 too
            prec = min(self.geodesic_precision, s.precision)
            phi, its = Geodesic(s.tube, r["source"]).run(self.dt_scale * s.tube.dx ** 2, precision=prec, tol=s.tol)
            phis, stats = [phi], [dict(iterations=its, batched=1)]
        else:
            B = GeodesicBatch(s.tube, np.stack([r["source"] for r in batch]))
            phib, itsb = B.run(self.dt_scale * s.tube.dx ** 2, tol=s.tol)
            phis = list(phib)
            stats = [dict(iterations=itsb[k].tolist(), batched=len(batch)) for k in range(len(batch))]
        done = time.perf_counter() - t0
        for r, phi, st in zip(batch, phis, stats):
            rec = dict(kind="geodesic", surface=s.name, arrival=r["t"], completion=done, latency=done - r["t"], stats=st)
            if keep_solutions:
                rec["x"] = phi[:N]
            out[r["id"]] = rec

    def _unit(self, s, what, keep_solutions, t0, out):
        """one unit of work of surface s: 'solo', 'step' or 'submit'"""
        with s.busy:
            self._unit_locked(s, what, keep_solutions, t0, out)

    def _unit_locked(self, s, what, keep_solutions, t0, out):
        if what == "solo":
            self._solo(s, keep_solutions, t0, out)
        elif what == "step":
            self._step(s, keep_solutions, t0, out)
        elif self._admit(s):
            # at most two batches in the server, so a precision switch takes effect within two batches
            take = max(0, min(len(s.waiting), 2 * MAX_SLOTS - len(s.inflight_arrival)))
            if s.precision == 1 and s.finished < PROBE:
                take = min(take, max(0, PROBE - s.submitted))
            if s.precision == 1:
                s.submitted += take
            for rid, b, arr in s.waiting[:take]:
                s.server.submit(b, rid)
                s.inflight_arrival[rid] = arr
            s.waiting = s.waiting[take:]
            s.active = s.active or take > 0
            if s.active:
                self._step(s, keep_solutions, t0, out)
        else:
            # no room on the device for this surface's server: serve the request alone
            self._solo(s, keep_solutions, t0, out)

    def _candidate(self, s, now):
        """(arrival of its oldest request, kind) of surface s's next unit of Laplace work, or None"""
        if s.switch_pending and s.server is not None and not s.active:
            s.server = None
            s.precision = 0
            s.switch_pending = False
            with self._lock:
                self.precision_switches += 1
        best = None
        if s.server is not None and s.active:
            best = (min(s.inflight_arrival.values(), default=now), 0, "step")
        if s.waiting:
            idle = s.server is None or not s.active
            probing = s.precision == 1 and s.finished < PROBE and s.submitted >= PROBE
            be = s.break_even()
            if be is None or s.switch_pending or probing or (idle and len(s.waiting) < be):
                c = (s.waiting[0][2], 1, "solo")
            elif len(s.inflight_arrival) < 2 * MAX_SLOTS:
                c = (s.waiting[0][2], 1, "submit")
            else:
                c = None
            if c is not None and (best is None or c < best):
                best = c
        return best

    @staticmethod
    def _worker_stream():
        """for the calling thread: opens a CUDA stream of its own on the caller's device
        for the library's work (cpm_set_thread_stream); returns the function that
        waits for it and hands the thread back to the library stream"""
        import torch

        from . import set_thread_stream

        dev = torch.cuda.current_device()

        def open_stream():
            torch.cuda.set_device(dev)
            st = torch.cuda.Stream()
            set_thread_stream(st.cuda_stream)

            def close():
                set_thread_stream(None)
                st.synchronize()

            return close

        return open_stream

    def run_concurrent(self, requests, keep_solutions=False):
        """run() with one worker thread per surface, each queueing its surface's work
        on a CUDA stream of its own (cpm_set_thread_stream), so the surfaces' solves
        overlap on the device.  Within a surface: earliest arrival first, with the same
        batching, probe and precision rules as run()."""
        order = sorted(requests, key=lambda r: r["t"])
        by = {name: [r for r in order if r["surface"] == name] for name in self.surfaces}
        out = {}
        t0 = time.perf_counter()
        errors = []
        open_stream = self._worker_stream()

        def worker(s, reqs):
            try:
                close_stream = open_stream()
                s.inflight_arrival = {}
                geo, i = [], 0
                want = [r["id"] for r in reqs]
                # membership tests only: other workers insert into `out` meanwhile
                while any(rid not in out for rid in want):
                    now = time.perf_counter() - t0
                    while i < len(reqs) and reqs[i]["t"] <= now:
                        r = reqs[i]
                        i += 1
                        if r["kind"] == "laplace":
                            s.waiting.append((r["id"], s.rhs(r["values"]), r["t"]))
                        else:
                            geo.append(r)
                    c = self._candidate(s, now)
                    if geo and (c is None or geo[0]["t"] < c[0]):
                        take = self._geo_take(geo)
                        geo = geo[len(take):]
                        self._geodesics(s, take, keep_solutions, t0, out)
                        continue
                    if c is None:
                        wait = reqs[i]["t"] - (time.perf_counter() - t0) if i < len(reqs) else 0.0
                        time.sleep(max(0.0001, min(0.002, wait)))
                        continue
                    self._unit(s, c[2], keep_solutions, t0, out)
                close_stream()
            except BaseException as e:  # reported on the calling thread
                errors.append(e)

        threads = [threading.Thread(target=worker, args=(self.surfaces[name], reqs), daemon=True)
                   for name, reqs in by.items() if reqs]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        if errors:
            raise errors[0]
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


def serve_fp64_one_at_a_time(surfaces, requests, dt_scale=1.0, keep_solutions=False):
    """The plain FP64 path serving the same stream: requests in arrival order,
    each solved alone once it has arrived (one right-hand side, the reference's
    algorithm; geodesics in FP64).  Returns {id: record} like ServingLoop.run."""
    by = {s.name: s for s in surfaces}
    solvers = {}
    out = {}
    t0 = time.perf_counter()
    for r in sorted(requests, key=lambda q: q["t"]):
        wait = r["t"] - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        s = by[r["surface"]]
        if r["kind"] == "laplace":
            if s.name not in solvers:
                solvers[s.name] = Solver(s.opset, s.m, s.n, kslots=1)
            x, st = solvers[s.name].solve(s.rhs(r["values"]), tol=s.tol, precision=0, precond=DIAGONAL)
            x, stats = x[0], st[0]
        else:
            x, its = Geodesic(s.tube, r["source"]).run(dt_scale * s.tube.dx ** 2, precision=0, tol=s.tol)
            stats = dict(iterations=its)
        done = time.perf_counter() - t0
        rec = dict(kind=r["kind"], surface=s.name, arrival=r["t"], completion=done, latency=done - r["t"], stats=stats)
        if keep_solutions:
            rec["x"] = x
        out[r["id"]] = rec
    return out


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
