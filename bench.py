"""Benchmark of the closest-point solve path on one GB300 (replicas on N GPUs).

Workload (the configuration the headline metric is quoted on): Laplace
-Delta_S u = 0 on the unit sphere with interior Dirichlet conditions on the
circles z = 0.3 and z = -0.5, dx = 0.025 (~166k tube nodes, 215,662 rows with
the IBC DOF and Dirichlet value rows), tricubic extension, 2nd-order IBCs.
Requests are right-hand sides with random circle values U[0,1] (seeded).

A step is 64 requests served by the continuous-batching server over two
32-slot batches on their own streams (--batches): FP32 BiCGStab inside FP64
iterative refinement to ||b - A x|| <= 1e-10 ||b|| (the reference's relative
residual), slots refilled as solves finish.
`value` is solves/s with every right-hand side resident in HBM (CUDA events on
the library stream).  Reported beside it: the plain FP64 one-request-at-a-time
GPU path (the reference algorithm on the device), latencies, the error against
the FP64 solutions, one static batch of 32, the end-to-end number through the
C-ABI with host buffers, the L.E apply roofline and the CPU baseline (the
oracle, the C++ restatement of the reference's custom solver, on the host's
cores).  `--impl reference` times the CPU restatement alone.

`--workload torus-geodesic | mesh-curves | serving-mix` prints one line for
the other configurations instead: the heat-method geodesic on the torus
R = 1, r = 0.4 at dx = 0.01; diffusion curves on the perturbed icosphere mesh
(327,680 triangles, 16 polyline IBCs, 3 right-hand sides) at dx = 0.005; and
a seeded Poisson stream of requests over the sphere, torus and mesh.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "cpm-ibc_gb300"))
sys.path.insert(0, os.path.join(ROOT, "cpm-ibc_gb300", "python"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

METRIC = "solves/s + p50/p99 latency: batched FP32-refined vs plain FP64 GPU at 1e-8 rel"
UNIT = "solves/s"
DX = 0.025
KSLOTS = 32
TOL = 1e-10
WORKLOAD = "sphere R=1 + Circle3D Dirichlet IBCs z=0.3 (u=U[0,1]) and z=-0.5 (u=U[0,1]), Laplace m=0 n=-1, dx=0.025, p=3, order-2 IBCs"


def circles(mod, dx):
    if hasattr(mod, "circle3d_desc"):
        mk = lambda R, c: mod.circle3d_desc(R, c, (0, 0, 1), dx, 2)
    else:
        mk = lambda R, c: mod.desc(mod.CIRCLE3D, [R, *c, 0, 0, 1], (-1.0, 1.0), boundary_order=2,
                                   on_ibc_tolerance=0.1 * dx * dx)
    return [mk(math.sqrt(1 - 0.09), (0, 0, 0.3)), mk(math.sqrt(1 - 0.25), (0, 0, -0.5))]


def rhs_from_rows(rows, vals):
    """PoissonWithIBC::GetRHS with f = 0 and Dirichlet value vals[c] on IBC c."""
    b = np.zeros(len(rows["kind"]))
    d = rows["kind"] == 2
    b[d] = np.asarray(vals)[rows["ibc"][d]]
    return b


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.lines = []
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms",
                                       "200", "-i", str(self.index)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                      text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.p = None
        return self

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def ranks():
    """(world, rank, local rank) from the launcher's environment"""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def dist_setup(backend=None):
    """one replica per GPU: the process group over the launcher's ranks (NCCL on the
    rank's GPU by default), or None for a single process"""
    world, rank, local = ranks()
    if world > 1:
        import torch
        import torch.distributed as dist

        if backend is None:
            torch.cuda.set_device(local)
            backend = "nccl"
        dist.init_process_group(backend)
        return world, rank, local, dist
    return 1, 0, local, None


def max_over_ranks(t, dist, device="cpu"):
    """the slowest replica's time (the job ends when every replica has)"""
    if dist is None:
        return float(t)
    import torch

    tt = torch.tensor([float(t)], device=device, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def replicas_value(world, n_per_rank, t_max):
    """whole-job solves/s: every replica serves n_per_rank requests, no data-path collective"""
    return world * n_per_rank / t_max


def cpu_model():
    """the host CPU's model name (lscpu, else /proc/cpuinfo, else the platform string)"""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform

    return platform.processor() or platform.machine()


EBCG_NOTE = "unavailable on this box (Eigen not installed, no network): the reference's Eigen BiCGSTAB path is not timed"


def bench_config(D, N, ibc_dofs, world):
    """the workload's config dict, shared by the GPU arm and the reference arm"""
    return {"workload": WORKLOAD, "rows": int(D), "tube_nodes": int(N), "ibc_dofs": int(ibc_dofs), "tol": TOL,
            "requests": "Laplace right-hand sides with circle values U[0,1] (seeded)",
            "l2": "no flush: the solve's working set (the GPU arm's 10 FP32 + 4 FP64 [D][32] arrays, "
                  f"{(10 * 4 + 4 * 8) * D * KSLOTS / 1e6:.0f} MB) exceeds the 129 MB L2",
            "parallelism": f"replicas x{world}"}


def oracle_c2():
    """the oracle's C2 problem (the reference's custom-solver path restated on the host)"""
    import oracle_lib as ol

    ol.build()
    return ol, ol.RefProblem(ol.sphere_desc(), circles(ol, DX), 3, DX)


def timed_oracle_solve(P, b, threads, tol=TOL):
    """one whole oracle BiCGStab solve of b on `threads` OpenMP threads: (x, stats)"""
    import oracle_lib as ol

    os.environ["OMP_NUM_THREADS"] = str(threads)
    ol.lib().cpmref_set_num_threads(int(threads))
    x, st = P.solve(0.0, -1.0, b, tol=tol)
    return x, st


def run_reference(args):
    """The reference arm: whole solves of the C2 system by the oracle (the C++17
    restatement of the reference's custom BiCGStab path) on the host's cores,
    one right-hand side per step, no extrapolation."""
    # rank 0 alone runs it (no process group needed); other ranks exit
    world, rank, _ = ranks()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ol, P = oracle_c2()
    setup_s = time.perf_counter() - t0
    rows = P.rows()
    rng = np.random.default_rng(1234)
    for _ in range(args.warmup):
        timed_oracle_solve(P, rhs_from_rows(rows, rng.uniform(0, 1, 2)), threads)
    times, iters = [], []
    t_run = time.perf_counter()
    for _ in range(args.steps):
        _, st = timed_oracle_solve(P, rhs_from_rows(rows, rng.uniform(0, 1, 2)), threads)
        times.append(st["seconds"])
        iters.append(st["iterations"])
    wall = time.perf_counter() - t_run
    sec_per_solve = float(np.mean(times))
    v = 1.0 / sec_per_solve
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sec_per_solve * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(P.D, P.N, P.total_ibc_dofs, world),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "cpu_model": cpu_model(),
                         "sample": f"{args.steps} whole solves (tol {TOL}, x0 = 0, diagonal preconditioner) of the "
                                   f"two-circle sphere system by the oracle (C++17 restatement of the reference's custom "
                                   f"BiCGStab: SpMV serial, vector ops OpenMP), one right-hand side per step",
                         "ebcg": EBCG_NOTE},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "latency_ms": {"p50": float(np.percentile(times, 50) * 1e3), "p99": float(np.percentile(times, 99) * 1e3)},
        "reference_note": "the reference (nathandking/cpm-ibc) needs Eigen3, fcpw and LBFGS++, absent here; "
                          "its custom solve path is timed through the oracle restatement",
        "iterations_per_solve": int(np.median(iters)), "setup_s": setup_s, "timed_wall_s": wall,
    }
    print(json.dumps(line), flush=True)


def run_profile(what):
    """Short, self-contained workload runs for ncu captures: 3 + 5 FP32 32-RHS
    applies and 3 + 5 FP64 1-RHS applies, or one batched mixed-precision solve."""
    import torch

    import build_ext

    build_ext.build()
    import cpm_gb300 as cg

    cg.set_device(0)
    dev = torch.device("cuda", 0)
    T = cg.Tube(cg.desc(cg.SPHERE, [1.0]), 3, DX)
    O = cg.OpSet(T, circles(cg, DX))
    D = O.D
    if what == "apply":
        for k, fp32 in ((KSLOTS, True), (1, False)):
            dt = torch.float32 if fp32 else torch.float64
            x = torch.randn((D, k), dtype=dt, device=dev)
            t = torch.empty_like(x)
            y = torch.empty_like(x)
            for _ in range(8):
                O.apply_device(0.0, -1.0, k, fp32, x.data_ptr(), t.data_ptr(), y.data_ptr())
            cg.sync()
    else:
        rows = O.rows()
        rng = np.random.default_rng(5)
        B = np.stack([rhs_from_rows(rows, rng.uniform(0, 1, 2)) for _ in range(KSLOTS)], axis=1)
        b = torch.from_numpy(B).to(dev)
        x = torch.zeros_like(b)
        st = cg.Solver(O, 0.0, -1.0, kslots=KSLOTS).solve_device(b.data_ptr(), x.data_ptr(), KSLOTS, tol=TOL, precision=1)
        print(json.dumps({"iterations": max(s["iterations"] for s in st)}))
    torch.cuda.synchronize()


def serving_mix(cg, requests, rate, seed=11, concurrent=True):
    """The serving stream over the three resident surfaces (the sphere with two circles at
    dx 0.025, the torus at dx 0.01, the perturbed icosphere at dx 0.005): `requests` seeded
    Poisson arrivals at `rate` per second, one in 32 a geodesic, the rest IBC Laplace solves
    with values U[0,1]; served by the serving loop (continuous batching, mixed precision; with
    `concurrent`, one worker thread and CUDA stream per surface) and, on the same stream and
    arrival times, one request at a time by the plain FP64 path.
    Returns the summary (solves/s, p50/p99 latency of both)."""
    from cpm_gb300 import serving as SV
    from cpm_gb300 import workloads as W

    t = time.perf_counter()
    surfaces = W.serving_surfaces(cg)
    t_setup = time.perf_counter() - t
    loop = SV.ServingLoop(surfaces)
    reqs = SV.poisson_stream(surfaces, requests, rate=rate, geodesic_every=32, seed=seed)
    warm = SV.poisson_stream(surfaces, 12, rate=0.0, geodesic_every=0, seed=seed + 1)
    for r in warm:
        r["id"] = -1 - r["id"]
    serve = loop.run_concurrent if concurrent else loop.run
    serve(warm)
    t = time.perf_counter()
    out = serve(reqs)
    span = time.perf_counter() - t
    lat = {k: [o["latency"] for o in out.values() if o["kind"] == k] for k in ("laplace", "geodesic")}
    fb = sum(1 for o in out.values() if o["kind"] == "laplace" and o["stats"].get("fp64_fallback"))
    geo_batched = sum(1 for o in out.values() if o["kind"] == "geodesic" and o["stats"].get("batched", 1) > 1)
    t = time.perf_counter()
    out64 = SV.serve_fp64_one_at_a_time(surfaces, reqs)
    span64 = time.perf_counter() - t
    lat64 = {k: [o["latency"] for o in out64.values() if o["kind"] == k] for k in ("laplace", "geodesic")}
    all_lat = [o["latency"] for o in out.values()]
    all_lat64 = [o["latency"] for o in out64.values()]

    def pct(v):
        return {k: {"p50": float(np.percentile(x, 50) * 1e3), "p99": float(np.percentile(x, 99) * 1e3), "n": len(x)}
                for k, x in v.items() if x}

    return {
        "config": {"surfaces": {s.name: {"tube_nodes": s.tube.N, "rows": s.opset.D, "curves": s.n_ibc,
                                         "server_bytes": s.bytes} for s in surfaces},
                   "requests": requests, "rate_per_s": rate, "geodesic_every": 32, "arrivals": "seeded Poisson process",
                   "workers": "one thread and CUDA stream per surface" if concurrent else "one loop for all surfaces",
                   "slots_per_surface": 32, "tol": TOL},
        "setup_s": t_setup, "makespan_s": span, "solves_per_s": len(out) / span,
        "latency_ms": {"p50": float(np.percentile(all_lat, 50) * 1e3), "p99": float(np.percentile(all_lat, 99) * 1e3),
                       "by_kind": pct(lat)},
        "laplace_fp64_fallbacks": fb, "geodesics_batched": geo_batched, "admissions": loop.admissions,
        "evictions": loop.evictions,
        "precision_switches": loop.precision_switches,
        "final_precision": {s.name: ("mixed" if s.precision else "fp64") for s in surfaces},
        "solo_fp64_solves": loop.solo_solves,
        "fp64_one_at_a_time": {"makespan_s": span64, "solves_per_s": len(out64) / span64,
                               "latency_ms": {"p50": float(np.percentile(all_lat64, 50) * 1e3),
                                              "p99": float(np.percentile(all_lat64, 99) * 1e3), "by_kind": pct(lat64)},
                               "path": "the same stream and arrival times, each request solved alone in FP64"},
        "speedup_solves_per_s": (len(out) / span) / (len(out64) / span64),
    }


def run_workload(args):
    """One JSON line for a configuration other than the headline one."""
    import build_ext

    build_ext.build()
    import cpm_gb300 as cg
    from cpm_gb300 import serving as SV
    from cpm_gb300 import workloads as W

    cg.set_device(0)
    line = {"workload": args.workload, "n_gpus": 1, "data": "synthetic"}
    if args.workload == "torus-geodesic":
        dx = 0.01
        t = time.perf_counter()
        T = cg.Tube(cg.desc(cg.TORUS, [1.0, 0.4], (-1.4, 1.4)), 3, dx)
        cg.sync()
        t_tube = time.perf_counter() - t
        cp = T.export()["cp"]
        rng = np.random.default_rng(12)
        srcs = cp[rng.choice(T.N, args.sources, replace=False)]
        # one source at a time (the reference's way: its own point-IBC operator per source), FP64
        n_solo = min(args.solo, args.sources)
        solo, t_solo_setup, t_solo = [], 0.0, 0.0
        for k in range(n_solo):
            t = time.perf_counter()
            G = cg.Geodesic(T, srcs[k])
            t_solo_setup += time.perf_counter() - t
            if k == 0:
                G.run(dx * dx, precision=0)  # warm-up (graph capture)
            t = time.perf_counter()
            phi, its = G.run(dx * dx, precision=0)
            t_solo += time.perf_counter() - t
            solo.append((G.D, phi, its))
        # all sources at once on one slot-patched operator
        t = time.perf_counter()
        B = cg.GeodesicBatch(T, srcs)
        t_batch_setup = time.perf_counter() - t
        t = time.perf_counter()
        phib, itsb = B.run(dx * dx)
        t_batch = time.perf_counter() - t
        err = max(float(np.max(np.abs(phib[k][:Dk] - phi)) / np.max(np.abs(phi))) for k, (Dk, phi, _) in enumerate(solo))
        line.update({
            "config": {"surface": "torus R=1 r=0.4", "dx": dx, "tube_nodes": T.N, "sources": args.sources,
                       "source": "seeded random tube nodes' closest points", "dt": dx * dx,
                       "heat_step": "FP64, 2000 damped Jacobi sweeps per preconditioner call", "poisson_steps": "FP64"},
            "tube_build_s": t_tube,
            "one_at_a_time": {"sources": n_solo, "seconds": t_solo, "solves_per_s": n_solo / t_solo,
                              "setup_s_per_source": t_solo_setup / n_solo,
                              "iterations": [list(map(int, x[2])) for x in solo]},
            "batched": {"sources": args.sources, "seconds": t_batch, "solves_per_s": args.sources / t_batch,
                        "setup_s": t_batch_setup, "iterations_first": [int(v) for v in itsb[0]]},
            "speedup_batched_vs_one_at_a_time": (args.sources / t_batch) / (n_solo / t_solo),
            "batched_rel_err_vs_one_at_a_time": err,
        })
    elif args.workload == "mesh-curves":
        dx = 0.005
        t = time.perf_counter()
        v, f = W.perturbed_icosphere(7, seed=3)
        bb = W.mesh_bbox(v)
        T = cg.Tube(cg.desc(cg.TRIANGULATION, (), bb, verts=v, prims=f), 3, dx)
        cg.sync()
        t_tube = time.perf_counter() - t
        curves, _ = W.parallel_plane_curves(v, f, 16, seed=4)
        t = time.perf_counter()
        O = cg.OpSet(T, [cg.desc(cg.POLYLINE, (), bb, boundary_order=2, on_ibc_tolerance=0.1 * dx * dx, verts=p,
                                 prims=sg) for p, sg in curves])
        cg.sync()
        t_ops = time.perf_counter() - t
        rows = O.rows()
        rgb = np.random.default_rng(9).uniform(0, 1, (16, 3))
        B = np.zeros((3, O.D))
        d = rows["kind"] == 2
        for ch in range(3):
            B[ch][d] = rgb[rows["ibc"][d], ch]
        S32 = cg.Solver(O, 0.0, -1.0, kslots=32)
        S32.solve(B, tol=TOL, precision=1)
        t = time.perf_counter()
        X32, st32 = S32.solve(B, tol=TOL, precision=1)
        t_mixed = time.perf_counter() - t
        S1 = cg.Solver(O, 0.0, -1.0, kslots=1)
        t = time.perf_counter()
        X64, st64 = [], []
        for ch in range(3):
            x, st = S1.solve(B[ch], tol=TOL, precision=0)
            X64.append(x[0])
            st64.append(st[0])
        t_fp64 = time.perf_counter() - t
        line.update({
            "config": {"surface": "perturbed icosphere level 7 (327,680 triangles), 8 real SH l<=6, amplitude 0.1",
                       "dx": dx, "tube_nodes": T.N, "rows": O.D, "ibc_dofs": O.total_ibc_dofs, "curves": 16,
                       "rhs": 3},
            "tube_build_s": t_tube, "operator_build_s": t_ops,
            "mixed_batched_3": {"seconds": t_mixed, "solves_per_s": 3 / t_mixed,
                                "iterations": [s_["iterations"] for s_ in st32],
                                "fp64_fallbacks": sum(s_["fp64_fallback"] for s_ in st32)},
            "fp64_one_at_a_time": {"seconds": t_fp64, "solves_per_s": 3 / t_fp64,
                                   "iterations": [s_["iterations"] for s_ in st64]},
            "mixed_rel_err_vs_fp64": float(max(np.max(np.abs(X32[c] - X64[c])) / np.max(np.abs(X64[c]))
                                               for c in range(3))),
        })
    else:  # serving-mix
        line.update(serving_mix(cg, args.requests, args.rate, concurrent=args.serve == "concurrent"))
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--plain-solves", type=int, default=8)
    ap.add_argument("--profile", choices=["apply", "solve"], default=None,
                    help="run only a few applies (or one batched solve) of the workload, for ncu")
    ap.add_argument("--workload", choices=["torus-geodesic", "mesh-curves", "serving-mix"], default=None,
                    help="one line for another configuration instead of the headline benchmark")
    ap.add_argument("--requests", type=int, default=160, help="serving-mix: requests in the stream")
    ap.add_argument("--sources", type=int, default=32, help="torus-geodesic: sources of the batched run")
    ap.add_argument("--solo", type=int, default=2, help="torus-geodesic: sources also run one at a time")
    ap.add_argument("--rate", type=float, default=8.0, help="serving-mix: mean arrivals per second")
    ap.add_argument("--batches", type=int, default=2,
                    help="32-slot batches of the server, run concurrently on their own streams")
    ap.add_argument("--mix-requests", type=int, default=256,
                    help="requests of the serving-stream sample in the default line (0: none)")
    ap.add_argument("--mix-rate", type=float, default=4.0, help="its mean arrivals per second")
    ap.add_argument("--serve", choices=["concurrent", "sequential"], default="concurrent",
                    help="serving stream: one worker thread and CUDA stream per surface, or one loop for all")
    ap.add_argument("--served-tol", type=float, default=TOL,
                    help="relative residual of the served mixed-precision solves (the plain FP64 path keeps 1e-10)")
    ap.add_argument("--refine-every", type=int, default=0,
                    help="mixed precision: reliable-update period in iterations (0: the library default)")
    ap.add_argument("--inner-tol", type=float, default=0.0,
                    help="mixed precision: residual drop that asks for a reliable update (0: the library default)")
    args = ap.parse_args()
    if args.workload:
        return run_workload(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.profile:
        return run_profile(args.profile)
    args.warmup = max(3, args.warmup)

    world, rank, local, dist = dist_setup()
    import torch

    import build_ext

    build_ext.build()
    import cpm_gb300 as cg

    cg.set_device(local)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    st = torch.cuda.ExternalStream(cg.stream_ptr(), device=dev)

    # ---- setup (not part of the metric; reported)
    t0 = time.perf_counter()
    T = cg.Tube(cg.desc(cg.SPHERE, [1.0]), 3, DX)
    O = cg.OpSet(T, circles(cg, DX))
    cg.sync()
    setup_s = time.perf_counter() - t0
    tuning = O.autotune(reps=10, fp64=True)  # launch shapes of the E passes, kept with the operator
    D = O.D
    rows = O.rows()
    rng = np.random.default_rng(1000 + rank)
    per_step = KSLOTS * args.batches  # requests per step: every slot of the server once
    n_warm, n_timed = args.warmup * per_step, args.steps * per_step
    vals = rng.uniform(0, 1, size=(n_warm + n_timed, 2))
    B = np.stack([rhs_from_rows(rows, v) for v in vals])  # [requests][D]
    b_dev = torch.from_numpy(B).to(dev)  # every request's right-hand side resident in HBM
    x_dev = torch.zeros_like(b_dev)
    stol = args.served_tol  # the mixed served path's relative residual (the plain FP64 path keeps the reference's TOL)
    srv = cg.Server(O, 0.0, -1.0, tol=stol, refine_every=args.refine_every, inner_tol=args.inner_tol, batches=args.batches)

    def stream(lo, hi):
        """submit requests lo..hi-1 at once and serve them to completion (continuous batching)"""
        for k in range(lo, hi):
            srv.submit_device(b_dev[k].data_ptr(), x_dev[k].data_ptr(), k)
        return srv.drain(want_x=False)

    stream(0, n_warm)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches0 = cg.launch_count()
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        served = stream(n_warm, n_warm + n_timed)
        e1.record(st)
        e1.synchronize()
        torch.cuda.synchronize()
    launches = cg.launch_count() - launches0
    t_total = max_over_ranks(e0.elapsed_time(e1) * 1e-3, dist, dev)
    value = replicas_value(world, n_timed, t_total)
    st_timed = [served[k][1] for k in range(n_warm, n_warm + n_timed)]
    assert all(x["status"] == 0 for x in st_timed), "a served request did not converge"
    iters = [x["iterations"] for x in st_timed]
    refs = [x["refinements"] for x in st_timed]
    service = [x["service"] for x in st_timed]
    latency = [x["latency"] for x in st_timed]

    # ---- accuracy of the served solutions: FP64 device solves of the first 32 timed requests
    s64 = cg.Solver(O, 0.0, -1.0, kslots=KSLOTS)
    sel = list(range(n_warm, n_warm + KSLOTS))
    x64, _ = s64.solve(B[sel], tol=1e-12, precision=0)
    xs = x_dev[sel].cpu().numpy()
    rel_err = float(max(np.max(np.abs(xs[j] - x64[j])) / np.max(np.abs(x64[j])) for j in range(KSLOTS)))

    # ---- the same requests served to relative residual 1e-8, the metric's error bound (the
    # plain FP64 path keeps the reference's 1e-10): a second server, timed the same way
    tol8 = None
    if stol != 1e-8:
        x8 = torch.zeros_like(b_dev)
        srv8 = cg.Server(O, 0.0, -1.0, tol=1e-8, refine_every=args.refine_every, inner_tol=args.inner_tol,
                         batches=args.batches)

        def stream8(lo, hi):
            for k in range(lo, hi):
                srv8.submit_device(b_dev[k].data_ptr(), x8[k].data_ptr(), k)
            return srv8.drain(want_x=False)

        stream8(0, n_warm)
        torch.cuda.synchronize()
        e8a, e8b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e8a.record(st)
        served8 = stream8(n_warm, n_warm + n_timed)
        e8b.record(st)
        e8b.synchronize()
        torch.cuda.synchronize()
        t8 = max_over_ranks(e8a.elapsed_time(e8b) * 1e-3, dist, dev)
        st8 = [served8[k][1] for k in range(n_warm, n_warm + n_timed)]
        x8s = x8[sel].cpu().numpy()
        tol8 = {"tol": 1e-8, "solves_per_s": replicas_value(world, n_timed, t8),
                "max_rel_err_vs_fp64": float(max(np.max(np.abs(x8s[j] - x64[j])) / np.max(np.abs(x64[j]))
                                                 for j in range(KSLOTS))),
                "err_what": f"relative l_inf against FP64 solves (tol 1e-12) of {KSLOTS} of the requests",
                "latency_ms": {"p50": float(np.percentile([x["service"] for x in st8], 50) * 1e3),
                               "p99": float(np.percentile([x["service"] for x in st8], 99) * 1e3)},
                "iterations_p50": float(np.median([x["iterations"] for x in st8])),
                "fp64_fallbacks": int(sum(x.get("fp64_fallback", 0) for x in st8)),
                "converged": bool(all(x["status"] == 0 for x in st8)),
                "what": "the same requests through a server at relative residual 1e-8 (the metric's error bound); "
                        "the plain FP64 path keeps the reference's 1e-10"}
        del srv8, x8

    # ---- one static batch of 32 (all slots start together; the batch ends with its slowest solve)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2
    bstat = torch.from_numpy(np.ascontiguousarray(B[sel].T)).to(dev)
    xstat = torch.zeros_like(bstat)
    s64.solve_device(bstat.data_ptr(), xstat.data_ptr(), KSLOTS, tol=stol, precision=1)
    with torch.cuda.stream(st):
        flush.zero_()
    e0s, e1s = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0s.record(st)
    sst = s64.solve_device(bstat.data_ptr(), xstat.data_ptr(), KSLOTS, tol=stol, precision=1)
    e1s.record(st)
    e1s.synchronize()
    static_s = e0s.elapsed_time(e1s) * 1e-3

    # ---- plain FP64 path, one request at a time (the reference algorithm on the device)
    s1 = cg.Solver(O, 0.0, -1.0, kslots=1)
    bp = torch.from_numpy(np.ascontiguousarray(B[sel[0]][:, None])).to(dev)
    xp = torch.zeros((D, 1), dtype=torch.float64, device=dev)
    s1.solve_device(bp.data_ptr(), xp.data_ptr(), 1, tol=TOL, precision=0)
    plain_t, plain_iters = [], []
    for j in range(args.plain_solves):
        bp.copy_(torch.from_numpy(np.ascontiguousarray(B[sel[j % KSLOTS]][:, None])))
        with torch.cuda.stream(st):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        stp = s1.solve_device(bp.data_ptr(), xp.data_ptr(), 1, tol=TOL, precision=0)
        e1.record(st)
        e1.synchronize()
        plain_t.append(e0.elapsed_time(e1) * 1e-3)
        plain_iters.append(stp[0]["iterations"])
    plain_sps = 1.0 / float(np.mean(plain_t))

    # ---- end to end through the C-ABI server with host buffers (H2D of b and D2H of x per request),
    # the same requests as the timed device-resident stream
    n_e2e = n_timed
    he = list(range(n_warm, n_warm + n_e2e))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in he:
        srv.submit(B[k], k)
    got = srv.drain(want_x=True)
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, dev)
    assert all(got[k][1]["status"] == 0 for k in he)
    e2e_value = replicas_value(world, n_e2e, e2e_s)

    # ---- roofline of the L.E apply (FP32, 32 RHS): E pass, IBC patch rows and L pass on the library stream
    xf = torch.randn((D, KSLOTS), dtype=torch.float32, device=dev)
    tf = torch.empty_like(xf)
    yf = torch.empty_like(xf)
    for _ in range(3):
        O.apply_device(0.0, -1.0, KSLOTS, True, xf.data_ptr(), tf.data_ptr(), yf.data_ptr())
    reps = 20
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        O.apply_device(0.0, -1.0, KSLOTS, True, xf.data_ptr(), tf.data_ptr(), yf.data_ptr())
    e1.record(st)
    e1.synchronize()
    apply_s = e0.elapsed_time(e1) * 1e-3 / reps
    n_ident = int(rows["identity"].sum())
    stencil_rows = D - n_ident
    # algorithmic bytes per apply: base index + 12 FP32 weights per stencil row, x read + y written per row and RHS
    alg_bytes = stencil_rows * (4 + 12 * 4) + D * KSLOTS * (4 + 4)
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        peak, peak_src = float(json.load(open(peaks_path))["hbm_gbs"]), "measured"
    achieved = alg_bytes / apply_s / 1e9
    # FP32 arithmetic of the same apply: the separable E sum is 143 flops per stencil row and RHS
    # (per plane i: 4 x (1 mul + 3 fma) over k, 1 mul + 3 fma over j, 1 mul by wx_i, 1 add into the row
    # sum, less the first add; fma = 2 flops), the L row 16 flops per row and RHS
    fp32_flops = stencil_rows * KSLOTS * 143 + D * KSLOTS * 16
    traffic = None
    prof = os.path.join(ROOT, "profiles", "apply_traffic.json")
    if os.path.exists(prof):
        traffic = json.load(open(prof)).get("bytes_per_apply")

    # ---- the serving stream over three surfaces (bounded sample; rank 0, N = 1 only)
    mix = None
    if rank == 0 and world == 1 and args.mix_requests > 0:
        mix = serving_mix(cg, args.mix_requests, args.mix_rate, concurrent=args.serve == "concurrent")

    # ---- CPU baseline and the error against the oracle (rank 0, N = 1 only): whole oracle solves
    cpu, rel_err_oracle = None, None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        ol, P = oracle_c2()
        oracle_setup_s = time.perf_counter() - t0
        prow = P.rows()
        k0 = sel[0]
        # the served solution of request k0 against the oracle's solve of the same system to tol 1e-12,
        # compared on the tube rows (matched by grid index)
        g_rec, r_rec = T.export()["rec"], P.tube()["rec"]
        o = np.argsort(g_rec)
        pos = np.searchsorted(g_rec[o], r_rec)
        if P.N == O.N and np.array_equal(g_rec[o][pos], r_rec):
            m = o[pos]
            x_ref, _ = timed_oracle_solve(P, rhs_from_rows(prow, vals[k0]), threads, tol=1e-12)
            xs0 = x_dev[k0].cpu().numpy()[m]
            rel_err_oracle = float(np.max(np.abs(xs0 - x_ref[:P.N])) / np.max(np.abs(x_ref[:P.N])))
        b_cpu = rhs_from_rows(prow, vals[sel[1]])
        _, st_all = timed_oracle_solve(P, b_cpu, threads)
        _, st_one = timed_oracle_solve(P, b_cpu, 1)
        cpu = {"value": 1.0 / st_all["seconds"], "unit": UNIT, "cores": threads, "kind": "port", "cpu_model": cpu_model(),
               "sample": f"one whole solve (tol {TOL}, {st_all['iterations']} iterations) of the two-circle sphere system "
                         f"(dx 0.025) by the oracle on {threads} threads (SpMV serial, vector ops OpenMP, as the "
                         f"reference runs); setup {oracle_setup_s:.1f} s not included",
               "one_thread": {"value": 1.0 / st_one["seconds"], "unit": UNIT, "cores": 1,
                              "iterations": st_one["iterations"]},
               "ebcg": EBCG_NOTE}

    clocks = clk.summary()
    # nominal FP32 peak at the SM clock seen under load: 152 SMs x 128 FP32 lanes x 2 flops per fma
    sm_mhz = (clocks or {}).get("sm_mhz") or 2070.0
    props = torch.cuda.get_device_properties(dev)
    fp32_peak = props.multi_processor_count * 128 * 2 * sm_mhz * 1e6 / 1e12
    fp32_achieved = fp32_flops / apply_s / 1e12
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_total / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32-inner/f64-refine", "data": "synthetic",
            "config": bench_config(D, O.N, O.total_ibc_dofs, world),
            "serving": {"slots": per_step, "batches": args.batches, "requests_per_step": per_step, "tol": stol,
                        "refine_every": args.refine_every or 32, "inner_tol": args.inner_tol or 0.1,
                        "how": f"continuous batching over {args.batches} 32-slot batches on their own streams: every "
                               f"step's {per_step} requests submitted at once with their right-hand sides resident in "
                               "HBM; slots refill as solves finish"},
            "latency_ms": {"p50": float(np.percentile(service, 50) * 1e3), "p99": float(np.percentile(service, 99) * 1e3),
                           "what": "admission into a slot to result (service time)"},
            "queue_order_ms": {"p50": float(np.percentile(latency, 50) * 1e3),
                               "p99": float(np.percentile(latency, 99) * 1e3),
                               "what": "submit to result with all of a step's requests submitted at once: the order "
                                       "in the queue, not a serving latency"},
            "fp64_plain": {"solves_per_s": plain_sps, "p50_ms": float(np.percentile(plain_t, 50) * 1e3),
                           "p99_ms": float(np.percentile(plain_t, 99) * 1e3),
                           "iterations": int(np.median(plain_iters)),
                           "tube_node_iterations_per_s": float(O.N * np.sum(plain_iters) / np.sum(plain_t))},
            "speedup_vs_fp64_plain": value / world / plain_sps,
            "served_tol_1e-8": (dict(tol8, speedup_vs_fp64_plain=tol8["solves_per_s"] / world / plain_sps)
                                if tol8 else None),
            # tube nodes x BiCGStab iterations (per right-hand side) per second, the whole job
            "tube_node_iterations_per_s": float(world * O.N * np.sum(iters) / t_total),
            "static_batch_32": {"solves_per_s": KSLOTS / static_s, "ms": static_s * 1e3,
                                "iterations_max": int(max(x["iterations"] for x in sst))},
            "rel_err_vs_fp64": rel_err,
            "rel_err_vs_oracle": rel_err_oracle,
            "rel_err_vs_oracle_what": "relative l_inf on the tube rows of one served (mixed) solution against the "
                                      "oracle's FP64 solve of the same right-hand side to tol 1e-12",
            "iterations_p50": float(np.median(iters)), "iterations_max": int(max(iters)),
            "refinements_p50": float(np.median(refs)),
            "fp64_fallbacks": int(sum(int(x.get("fp64_fallback", 0)) for x in st_timed)),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(D * per_step * 8),
                    "d2h_bytes_per_step": int(D * per_step * 8),
                    "path": f"cpm_server_submit / cpm_server_step / cpm_server_poll with host arrays, {n_e2e} requests"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "kernel": "L.E apply (E pass + IBC patch rows + L pass), FP32, 32 RHS",
                         "apply_us": apply_s * 1e6, "alg_bytes_per_apply": alg_bytes, "peak_source": peak_src,
                         "fp32": {"achieved": fp32_achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                                  "frac": fp32_achieved / fp32_peak, "flops_per_apply": int(fp32_flops),
                                  "peak_source": "nominal: SMs x 128 FP32 lanes x 2 flops x median SM clock under load"}},
            "cpu_baseline": cpu,
            "serving_mix": mix,
            "launch_shapes": {k: (round(v, 2) if isinstance(v, float) else v) for k, v in tuning.items()},
            "gpu_launches": int(launches),
            "clocks": clocks,
            "setup_s": setup_s,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
