"""cpm_apply_device_noalloc: the operator apply for callers that cannot
allocate device memory when they call it (applications whose device memory
is owned by their own pool, latency-critical loops where cudaMalloc/cudaFree
would synchronise the device).  Its scratch is a fixed 32 MiB device array
inside the library.

Checked through the C-ABI against cpm_apply_device (caller-provided scratch),
on two calls in a row: both run the same kernels in the same order, so the
results are equal bit for bit (tolerance 0); and an input too large for the
fixed array is rejected.
This file is collected last so that a failure here leaves every other test run.
"""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ibcs(cg, dx):
    mk = lambda R, c: cg.desc(cg.CIRCLE3D, [R, *c, 0, 0, 1], (-1.0, 1.0), boundary_order=2, on_ibc_tolerance=0.1 * dx * dx)
    return [mk(math.sqrt(1 - 0.09), (0, 0, 0.3)), mk(math.sqrt(1 - 0.25), (0, 0, -0.5))]


@pytest.mark.parametrize("kslots,fp32", [(1, False), (32, True)])
def test_noalloc_apply_matches_apply_device_twice(gpu, kslots, fp32):
    torch = pytest.importorskip("torch")
    cg = gpu
    dx = 0.05
    T = cg.Tube(cg.desc(cg.SPHERE, [1.0]), 3, dx)
    O = cg.OpSet(T, _ibcs(cg, dx))
    L = cg.lib()
    L.cpm_apply_device_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                          ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    dev = torch.device("cuda", 0)
    dt = torch.float32 if fp32 else torch.float64
    gen = torch.Generator(device="cpu").manual_seed(3)
    for call in range(2):  # two calls in a row through the shared scratch array
        x = torch.randn((O.D, kslots), generator=gen, dtype=torch.float64).to(dt).to(dev)
        m, n = (1.0, -1.0) if call == 0 else (0.0, -1.0)
        t = torch.empty_like(x)
        y_ref = torch.empty_like(x)
        O.apply_device(m, n, kslots, fp32, x.data_ptr(), t.data_ptr(), y_ref.data_ptr())
        cg.sync()
        y = torch.full_like(x, float("nan"))
        rc = L.cpm_apply_device_noalloc(O.h, m, n, kslots, int(fp32), x.data_ptr(), y.data_ptr())
        assert rc == 0, L.cpm_last_error().decode()
        cg.sync()
        a, b = y.cpu().double().numpy(), y_ref.cpu().double().numpy()
        assert np.all(np.isfinite(a))
        assert np.array_equal(a, b)  # the same kernels on the same inputs: bit for bit


def test_noalloc_rejects_inputs_beyond_the_fixed_array(gpu):
    torch = pytest.importorskip("torch")
    cg = gpu
    dx = 0.025  # 215,662 rows: FP64 x 32 right-hand sides needs 55 MB > 32 MiB
    T = cg.Tube(cg.desc(cg.SPHERE, [1.0]), 3, dx)
    O = cg.OpSet(T, _ibcs(cg, dx))
    L = cg.lib()
    L.cpm_apply_device_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                          ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    x = torch.zeros((O.D, 32), dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    rc = L.cpm_apply_device_noalloc(O.h, 0.0, -1.0, 32, 0, x.data_ptr(), y.data_ptr())
    assert rc == -1
    assert b"exceeds" in L.cpm_last_error()
