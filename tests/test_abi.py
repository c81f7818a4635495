"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/cpm_gpu.h declares (no GPU needed: no compute call is made)."""
import ctypes
import os
import re
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "cpm_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cpm_[a-z0-9_]+)\s*\(", txt)))


def test_library_builds_and_exports_every_declared_symbol():
    sys.path.insert(0, os.path.join(ROOT, "cpm-ibc_gb300"))
    import build_ext

    path = build_ext.build()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_binds_every_symbol():
    sys.path.insert(0, os.path.join(ROOT, "cpm-ibc_gb300", "python"))
    import cpm_gb300

    L = cpm_gb300.lib()
    for s in declared_symbols():
        getattr(L, s)


def test_error_string_without_gpu_call():
    sys.path.insert(0, os.path.join(ROOT, "cpm-ibc_gb300", "python"))
    import cpm_gb300

    L = cpm_gb300.lib()
    h = ctypes.c_void_p()
    # invalid arguments are rejected on the host before any device work
    rc = L.cpm_tube_build(None, 3, 0.1, ctypes.byref(h))
    assert rc == -1
    assert b"invalid" in L.cpm_last_error()


def test_new_entry_points_reject_invalid_arguments_on_the_host():
    """cpm_closest_points and cpm_geodesic_nearest_* validate their arguments before any
    device work (status -1, CPM_ERR_INVALID_ARG)."""
    sys.path.insert(0, os.path.join(ROOT, "cpm-ibc_gb300", "python"))
    import cpm_gb300

    L = cpm_gb300.lib()
    vp = ctypes.c_void_p
    L.cpm_closest_points.argtypes = [vp, ctypes.c_int64, vp, ctypes.c_double, vp, vp]
    L.cpm_geodesic_nearest_create.argtypes = [vp, ctypes.c_int64, vp, ctypes.c_int64, vp, vp, vp]
    L.cpm_geodesic_nearest_run.argtypes = [vp, ctypes.c_double, ctypes.c_int32, ctypes.c_double, ctypes.c_int32, vp, vp]
    x = (ctypes.c_double * 3)()
    out = (ctypes.c_double * 3)()
    d = cpm_gb300.desc(cpm_gb300.SPHERE, [1.0])
    assert L.cpm_closest_points(None, 1, x, 0.0, out, out) == -1
    assert L.cpm_closest_points(ctypes.byref(d), -1, x, 0.0, out, out) == -1
    assert L.cpm_closest_points(ctypes.byref(d), 1, None, 0.0, out, out) == -1
    assert L.cpm_closest_points(ctypes.byref(d), 0, None, 0.0, None, None) == 0  # nothing to do
    h = vp()
    assert L.cpm_geodesic_nearest_create(None, 0, None, 0, None, None, ctypes.byref(h)) == -1
    assert L.cpm_geodesic_nearest_run(None, 0.01, 0, 1e-10, 0, out, None) == -1
    assert b"invalid" in L.cpm_last_error()
