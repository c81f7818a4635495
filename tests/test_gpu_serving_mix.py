"""The serving mix at reduced size: three device-resident surfaces with their
IBC curves, a seeded Poisson stream of IBC-Laplace and geodesic requests, and
an HBM budget that holds only two servers at a time (so servers are released
and admitted while the stream runs).

Tolerances: every Laplace result within 1e-8 relative l_inf of the plain FP64
device solve of the same right-hand side; every geodesic within 1e-8 of the
FP64 geodesic from the same source."""
import numpy as np
import pytest

from cpm_gb300 import serving as SV
from cpm_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_serving_mix_results_and_admission(gpu):
    surfaces = W.serving_surfaces(gpu, dx_scale=5.0, mesh_level=3, n_curves=2)
    by = {s.name: s for s in surfaces}
    sizes = sorted(s.bytes for s in surfaces)
    loop = SV.ServingLoop(surfaces, hbm_budget=sizes[-1] + sizes[-2])
    reqs = SV.poisson_stream(surfaces, 48, rate=400.0, geodesic_every=16, seed=2)
    out = loop.run(reqs, keep_solutions=True)
    assert sorted(out) == [r["id"] for r in reqs]
    assert loop.admissions >= 3
    for r in reqs:
        rec = out[r["id"]]
        s = by[r["surface"]]
        assert rec["latency"] >= 0
        if r["kind"] == "laplace":
            assert rec["stats"]["status"] == 0
            x64, _ = gpu.Solver(s.opset, 0.0, -1.0).solve(s.rhs(r["values"]), tol=1e-12, precision=0)
            assert np.max(np.abs(rec["x"] - x64[0])) / np.max(np.abs(x64[0])) <= 1e-8
        else:
            g = gpu.Geodesic(s.tube, r["source"])
            p64, _ = g.run(s.tube.dx ** 2, precision=0)
            p64 = p64[:s.tube.N]
            assert np.max(np.abs(rec["x"] - p64)) / np.max(np.abs(p64)) <= 1e-8


def test_sparse_stream_solves_alone_in_fp64(gpu):
    """A stream slow enough that requests arrive one by one: each is solved
    alone by the plain FP64 path (a 32-slot batch of one costs a full batch),
    with the same results as the FP64 device solve."""
    surfaces = W.serving_surfaces(gpu, dx_scale=5.0, mesh_level=3, n_curves=2)
    by = {s.name: s for s in surfaces}
    loop = SV.ServingLoop(surfaces)
    reqs = SV.poisson_stream(surfaces, 12, rate=8.0, geodesic_every=0, seed=4)
    out = loop.run(reqs, keep_solutions=True)
    assert sorted(out) == [r["id"] for r in reqs]
    assert loop.solo_solves >= 1
    assert any(o["mode"] == "solo" for o in out.values())
    for r in reqs:
        rec = out[r["id"]]
        s = by[r["surface"]]
        x64, _ = gpu.Solver(s.opset, 0.0, -1.0).solve(s.rhs(r["values"]), tol=1e-12, precision=0)
        assert np.max(np.abs(rec["x"] - x64[0])) / np.max(np.abs(x64[0])) <= 1e-8
    base = SV.serve_fp64_one_at_a_time(surfaces, reqs)
    assert sorted(base) == sorted(out)


def test_concurrent_workers_results_and_admission(gpu):
    """run_concurrent: one worker thread and CUDA stream per surface
    (cpm_set_thread_stream), with the same HBM budget of two servers. Every
    result within 1e-8 of the FP64 device solve (Laplace) or the FP64 geodesic."""
    surfaces = W.serving_surfaces(gpu, dx_scale=5.0, mesh_level=3, n_curves=2)
    by = {s.name: s for s in surfaces}
    sizes = sorted(s.bytes for s in surfaces)
    loop = SV.ServingLoop(surfaces, hbm_budget=sizes[-1] + sizes[-2])
    reqs = SV.poisson_stream(surfaces, 64, rate=400.0, geodesic_every=16, seed=6)
    lib_stream = gpu.stream_ptr()
    out = loop.run_concurrent(reqs, keep_solutions=True)
    assert sorted(out) == sorted(r["id"] for r in reqs)
    assert gpu.stream_ptr() == lib_stream  # the calling thread keeps the library stream
    for r in reqs:
        rec = out[r["id"]]
        s = by[r["surface"]]
        assert rec["latency"] >= 0
        if r["kind"] == "laplace":
            assert rec["stats"]["status"] == 0
            x64, _ = gpu.Solver(s.opset, 0.0, -1.0).solve(s.rhs(r["values"]), tol=1e-12, precision=0)
            assert np.max(np.abs(rec["x"] - x64[0])) / np.max(np.abs(x64[0])) <= 1e-8
        else:
            g = gpu.Geodesic(s.tube, r["source"])
            p64, _ = g.run(s.tube.dx ** 2, precision=0)
            p64 = p64[:s.tube.N]
            assert np.max(np.abs(rec["x"] - p64)) / np.max(np.abs(p64)) <= 1e-8


def test_thread_stream_orders_the_calling_threads_work(gpu):
    """cpm_set_thread_stream: an apply queued from a thread on its own stream
    gives the same bits as on the library stream; the library stream is back
    after the thread resets it."""
    import threading

    import torch

    T = gpu.Tube(gpu.desc(gpu.SPHERE, [1.0]), 3, 0.1)
    O = gpu.OpSet(T)
    x = torch.rand((O.D, 32), dtype=torch.float64, device="cuda")
    t0, y0 = torch.empty_like(x), torch.empty_like(x)
    t1, y1 = torch.empty_like(x), torch.empty_like(x)
    lib_stream = gpu.stream_ptr()
    torch.cuda.synchronize()
    O.apply_device(1.0, -1.0, 32, False, x.data_ptr(), t0.data_ptr(), y0.data_ptr())
    gpu.sync()
    seen = {}

    def work():
        st = torch.cuda.Stream()
        gpu.set_thread_stream(st.cuda_stream)
        seen["stream"] = gpu.stream_ptr()
        seen["own"] = st.cuda_stream
        O.apply_device(1.0, -1.0, 32, False, x.data_ptr(), t1.data_ptr(), y1.data_ptr())
        gpu.sync()
        gpu.set_thread_stream(None)
        seen["after"] = gpu.stream_ptr()

    th = threading.Thread(target=work)
    th.start()
    th.join()
    assert seen["stream"] == seen["own"] and seen["after"] == lib_stream
    assert torch.equal(y0, y1)


@pytest.mark.parametrize("concurrent", [False, True])
def test_waiting_geodesics_run_as_one_batch(gpu, concurrent):
    """Geodesics waiting on one surface run together on a slot-patched operator
    (GeodesicBatch); each distance within 1e-8 of its FP64 geodesic alone."""
    surfaces = W.serving_surfaces(gpu, dx_scale=5.0, mesh_level=3, n_curves=2)
    s = surfaces[0]
    cp = s.closest_points()
    rng = np.random.default_rng(8)
    reqs = [dict(id=k, t=0.0, surface=s.name, kind="geodesic", source=cp[int(rng.integers(len(cp)))]) for k in range(4)]
    loop = SV.ServingLoop(surfaces, geodesic_batch_min=2)
    out = (loop.run_concurrent if concurrent else loop.run)(reqs, keep_solutions=True)
    assert sorted(out) == list(range(4))
    assert max(o["stats"]["batched"] for o in out.values()) >= 2
    for r in reqs:
        p64, _ = gpu.Geodesic(s.tube, r["source"]).run(s.tube.dx ** 2, precision=0)
        p64 = p64[:s.tube.N]
        assert np.max(np.abs(out[r["id"]]["x"] - p64)) / np.max(np.abs(p64)) <= 1e-8
