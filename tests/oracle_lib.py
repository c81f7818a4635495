"""ctypes binding of the oracle (the CPU restatement of the reference's solve path).

Test infrastructure only: the product library never imports this module.  It
is used by the tests and by ``bench.py``'s CPU baseline / reference legs.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "_build", "libcpmref.so")

SPHERE, TORUS, CIRCLE3D, POINT, TRIANGULATION, POLYLINE = range(6)

_lock = threading.Lock()
_lib = None


class SurfaceDesc(ctypes.Structure):
    """Surface / IBC descriptor; the same field layout is used by the oracle and the C-ABI."""

    _fields_ = [
        ("kind", ctypes.c_int32),
        ("nparams", ctypes.c_int32),
        ("params", ctypes.c_double * 8),
        ("bbox", ctypes.c_double * 2),
        ("nverts", ctypes.c_int64),
        ("verts", ctypes.POINTER(ctypes.c_double)),
        ("nprims", ctypes.c_int64),
        ("prims", ctypes.POINTER(ctypes.c_int64)),
        ("boundary_order", ctypes.c_int32),
        ("boundary_type", ctypes.c_int32 * 2),
        ("is_oriented", ctypes.c_int32),
        ("has_point_on_side1", ctypes.c_int32),
        ("use_cp_diff_directions", ctypes.c_int32),
        ("use_Jcp_surface_normals", ctypes.c_int32),
        ("pad0", ctypes.c_int32),
        ("on_ibc_tolerance", ctypes.c_double),
        ("point_on_side1", ctypes.c_double * 3),
        ("dof_radius_scale", ctypes.c_double),
    ]


def make_desc(kind, params=(), bbox=(-1.0, 1.0), boundary_order=1, on_ibc_tolerance=0.0,
              verts=None, prims=None, boundary_type=(0, 0)):
    d = SurfaceDesc()
    d.kind = kind
    d.nparams = len(params)
    for i, p in enumerate(params):
        d.params[i] = float(p)
    d.bbox[0], d.bbox[1] = bbox
    d.boundary_order = boundary_order
    d.boundary_type[0], d.boundary_type[1] = boundary_type
    d.use_Jcp_surface_normals = 1
    d.on_ibc_tolerance = on_ibc_tolerance
    d.dof_radius_scale = 1.0
    d._keep = []
    if verts is not None:
        v = np.ascontiguousarray(verts, dtype=np.float64)
        p = np.ascontiguousarray(prims, dtype=np.int64)
        d._keep += [v, p]
        d.nverts = v.shape[0]
        d.verts = v.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.nprims = p.shape[0]
        d.prims = p.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    return d


def sphere_desc(R=1.0, bbox=(-1.0, 1.0)):
    """SurfaceSpecifier("Sphere") defaults: R = 1, bbox [-1, 1] (src/SurfaceSpecifier.cpp:120-126)."""
    return make_desc(SPHERE, [R], bbox)


def torus_desc(R=2.0, r=1.0, bbox=(-3.0, 3.0)):
    return make_desc(TORUS, [R, r], bbox)


def circle3d_desc(R, centre, normal, dx, boundary_order=2, bbox=(-1.0, 1.0)):
    return make_desc(CIRCLE3D, [R, *centre, *normal], bbox, boundary_order=boundary_order,
                     on_ibc_tolerance=0.1 * dx * dx)


def point_desc(p, dx, boundary_order=1, bbox=(-1.0, 1.0)):
    return make_desc(POINT, list(p), bbox, boundary_order=boundary_order, on_ibc_tolerance=0.1 * dx * dx)


def build():
    """Compile the oracle with its Makefile (seconds)."""
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "-j8"], check=True)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                build()
            L = ctypes.CDLL(LIB_PATH)
            vp = ctypes.c_void_p
            P = ctypes.POINTER
            L.cpmref_last_error.restype = ctypes.c_char_p
            L.cpmref_problem_create.argtypes = [P(SurfaceDesc), ctypes.c_int32, P(SurfaceDesc), ctypes.c_int32,
                                                ctypes.c_double, ctypes.c_int32, P(vp)]
            L.cpmref_problem_create_from_cp.argtypes = [P(SurfaceDesc), ctypes.c_int32, ctypes.c_double, ctypes.c_int64,
                                                        vp, vp, vp, P(vp)]
            L.cpmref_problem_destroy.argtypes = [vp]
            L.cpmref_problem_sizes.argtypes = [vp, vp]
            L.cpmref_problem_grid.argtypes = [vp, vp]
            L.cpmref_setup_seconds.argtypes = [vp]
            L.cpmref_setup_seconds.restype = ctypes.c_double
            L.cpmref_tube_export.argtypes = [vp] * 7
            L.cpmref_visited_export.argtypes = [vp] * 4
            L.cpmref_weights_export.argtypes = [vp, vp]
            L.cpmref_csr_nnz.argtypes = [vp, ctypes.c_int32]
            L.cpmref_csr_nnz.restype = ctypes.c_int64
            L.cpmref_csr_rows.argtypes = [vp, ctypes.c_int32]
            L.cpmref_csr_rows.restype = ctypes.c_int64
            L.cpmref_csr_export.argtypes = [vp, ctypes.c_int32, vp, vp, vp]
            L.cpmref_rows_export.argtypes = [vp] * 5
            L.cpmref_xp_export.argtypes = [vp, vp]
            L.cpmref_row_sides.argtypes = [vp, vp]
            L.cpmref_ibc_sizes.argtypes = [vp, ctypes.c_int32, vp]
            L.cpmref_ibc_export.argtypes = [vp, ctypes.c_int32] + [vp] * 7
            L.cpmref_apply.argtypes = [vp, ctypes.c_double, ctypes.c_double, vp, vp]
            L.cpmref_solve.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_int32, ctypes.c_int32, vp, vp,
                                       ctypes.c_double, ctypes.c_int32, vp]
            L.cpmref_geodesic.argtypes = [vp, ctypes.c_double, ctypes.c_int32, vp, vp]
            L.cpmref_geodesic_nearest.argtypes = [vp, ctypes.c_int64, vp, ctypes.c_int64, vp, vp, ctypes.c_double,
                                                  ctypes.c_int32, vp, vp]
            L.cpmref_set_parallel_rows.argtypes = [ctypes.c_int32]
            L.cpmref_set_num_threads.argtypes = [ctypes.c_int32]
            L.cpmref_csr_multiply.argtypes = [vp, ctypes.c_int32, vp, vp]
            L.cpmref_heat_nearest.argtypes = [vp, ctypes.c_int64, vp, ctypes.c_int64, vp, vp, ctypes.c_double,
                                              ctypes.c_int32, vp]
            L.cpmref_closest_points.argtypes = [P(SurfaceDesc), ctypes.c_int64, vp, vp, vp]
            _lib = L
        return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def _check(rc):
    if rc != 0:
        raise RuntimeError(lib().cpmref_last_error().decode())


class RefProblem:
    """A surface (+ interior boundaries) assembled exactly as the reference does."""

    def __init__(self, surface, ibcs=(), p=3, dx=0.1, record_visited=False, _handle=None):
        L = lib()
        if _handle is not None:
            self.h = _handle
        else:
            h = ctypes.c_void_p()
            arr = (SurfaceDesc * max(1, len(ibcs)))(*ibcs) if ibcs else None
            _check(L.cpmref_problem_create(ctypes.byref(surface), len(ibcs), arr, p, dx, int(record_visited),
                                           ctypes.byref(h)))
            self.h = h
        s = np.zeros(10, np.int64)
        L.cpmref_problem_sizes(self.h, _ptr(s))
        (self.N, self.D, self.N1d, self.total_ibc_dofs, self.num2, self.n_ibc, self.n_visited, self.nnzL,
         self.nnzE, self.n_plot) = [int(v) for v in s]
        g = np.zeros(3)
        L.cpmref_problem_grid(self.h, _ptr(g))
        self.dx, self.xstart, self.radius = [float(v) for v in g]
        self.setup_seconds = float(L.cpmref_setup_seconds(self.h))

    @classmethod
    def from_cp(cls, surface, p, dx, keys, cp, dist):
        L = lib()
        h = ctypes.c_void_p()
        keys = np.ascontiguousarray(keys, np.int64)
        order = np.argsort(keys, kind="stable")
        k = np.ascontiguousarray(keys[order])
        c = np.ascontiguousarray(np.asarray(cp, np.float64)[order])
        d = np.ascontiguousarray(np.asarray(dist, np.float64)[order])
        _check(L.cpmref_problem_create_from_cp(ctypes.byref(surface), p, dx, len(k), _ptr(k), _ptr(c), _ptr(d),
                                               ctypes.byref(h)))
        return cls(surface, _handle=h)

    def __del__(self):
        try:
            lib().cpmref_problem_destroy(self.h)
        except Exception:
            pass

    def tube(self):
        N = self.N
        rec = np.zeros(N, np.int64)
        x = np.zeros((N, 3))
        cp = np.zeros((N, 3))
        dist = np.zeros(N)
        bpt = np.zeros(N, np.int64)
        nbr = np.zeros((N, 6), np.int64)
        lib().cpmref_tube_export(self.h, _ptr(rec), _ptr(x), _ptr(cp), _ptr(dist), _ptr(bpt), _ptr(nbr))
        return dict(rec=rec, x=x, cp=cp, dist=dist, bpt=bpt, nbr=nbr)

    def visited(self):
        n = self.n_visited
        rec = np.zeros(n, np.int64)
        cp = np.zeros((n, 3))
        dist = np.zeros(n)
        lib().cpmref_visited_export(self.h, _ptr(rec), _ptr(cp), _ptr(dist))
        return rec, cp, dist

    def weights(self):
        w = np.zeros((self.N, 3, 4))
        lib().cpmref_weights_export(self.h, _ptr(w))
        return w

    def csr(self, which):
        """which: 0 Lfull, 1 Efull, 2 L, 3 E, 4 plot interpolation (with IBC columns),
        5 / 6 / 7 the whole-tube gradient matrices Dc_x / Dc_y / Dc_z."""
        L = lib()
        nnz = int(L.cpmref_csr_nnz(self.h, which))
        rows = int(L.cpmref_csr_rows(self.h, which))
        ptr = np.zeros(rows + 1, np.int64)
        idx = np.zeros(nnz, np.int64)
        val = np.zeros(nnz)
        L.cpmref_csr_export(self.h, which, _ptr(ptr), _ptr(idx), _ptr(val))
        return ptr, idx, val

    def csr_multiply(self, which, x):
        """y = A x for the exported matrix `which` (see csr), in the oracle."""
        x = np.ascontiguousarray(x, np.float64)
        rows = int(lib().cpmref_csr_rows(self.h, which))
        y = np.zeros(rows)
        _check(lib().cpmref_csr_multiply(self.h, which, _ptr(x), _ptr(y)))
        return y

    def rows(self):
        D = self.D
        ident = np.zeros(D, np.uint8)
        kind = np.zeros(D, np.int32)
        ibc = np.zeros(D, np.int32)
        point = np.zeros((D, 3))
        lib().cpmref_rows_export(self.h, _ptr(ident), _ptr(kind), _ptr(ibc), _ptr(point))
        side = np.zeros(D, np.int32)
        lib().cpmref_row_sides(self.h, _ptr(side))
        return dict(identity=ident.astype(bool), kind=kind, ibc=ibc, point=point, side=side)

    def xp(self):
        xp = np.zeros((self.n_plot, 3))
        lib().cpmref_xp_export(self.h, _ptr(xp))
        return xp

    def ibc_subsets(self, c):
        s = np.zeros(5, np.int64)
        lib().cpmref_ibc_sizes(self.h, c, _ptr(s))
        nt, nd = int(s[0]), int(s[1])
        tag_set = np.zeros(nt, np.int64)
        tag_dist = np.zeros(nt)
        tag_dir = np.zeros((nt, 3))
        tag_cpdiff = np.zeros((nt, 3))
        dof_set = np.zeros(nd, np.int64)
        dof_cp = np.zeros((nd, 3))
        dof_cpbar = np.zeros((nd, 3))
        lib().cpmref_ibc_export(self.h, c, _ptr(tag_set), _ptr(tag_dist), _ptr(tag_dir), _ptr(dof_set), _ptr(dof_cp),
                                _ptr(dof_cpbar), _ptr(tag_cpdiff))
        return dict(tag_set=tag_set, tag_dist=tag_dist, tag_dir=tag_dir, tag_cpdiff=tag_cpdiff, dof_set=dof_set,
                    dof_cp=dof_cp, dof_cpbar=dof_cpbar, col_start=int(s[2]), dcol_start=int(s[3]),
                    identity_rows_start=int(s[4]))

    def apply(self, m, n, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.D)
        lib().cpmref_apply(self.h, m, n, _ptr(x), _ptr(y))
        return y

    def solve(self, m, n, b, precond=1, precond_iters=0, tol=1e-10, max_iters=100000):
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros(self.D)
        st = np.zeros(4)
        _check(lib().cpmref_solve(self.h, m, n, precond, precond_iters, _ptr(b), _ptr(x), tol, max_iters, _ptr(st)))
        return x, dict(iterations=int(st[0]), restarts=int(st[1]), rel_res2=float(st[2]), seconds=float(st[3]))

    def geodesic(self, dt, step1_jacobi_iters=0):
        phi = np.zeros(self.D)
        its = np.zeros(8, np.int32)
        _check(lib().cpmref_geodesic(self.h, dt, step1_jacobi_iters, _ptr(phi), _ptr(its)))
        return phi, its[:4].tolist()

    def heat_nearest(self, ibc_idx, inside_idx, inside_dist, dt, step1_jacobi_iters=0):
        """GeodesicDistanceNearest's heat step: the solution of the transposed implicit-Euler
        system (before u = E u)."""
        a = np.ascontiguousarray(ibc_idx, np.int64)
        b = np.ascontiguousarray(inside_idx, np.int64)
        d = np.ascontiguousarray(inside_dist, np.float64)
        u = np.zeros(self.N)
        _check(lib().cpmref_heat_nearest(self.h, len(a), _ptr(a), len(b), _ptr(b), _ptr(d), dt, step1_jacobi_iters,
                                         _ptr(u)))
        return u

    def geodesic_nearest(self, ibc_idx, inside_idx, inside_dist, dt, step1_jacobi_iters=0):
        """GeodesicDistanceNearest::ComputeDistance on this (IBC-free) problem; phi on the tube
        rows.  step1_jacobi_iters = 0 solves the heat step directly (dense LU, small tubes)."""
        a = np.ascontiguousarray(ibc_idx, np.int64)
        b = np.ascontiguousarray(inside_idx, np.int64)
        d = np.ascontiguousarray(inside_dist, np.float64)
        phi = np.zeros(self.N)
        its = np.zeros(8, np.int32)
        _check(lib().cpmref_geodesic_nearest(self.h, len(a), _ptr(a), len(b), _ptr(b), _ptr(d), dt, step1_jacobi_iters,
                                             _ptr(phi), _ptr(its)))
        return phi, its[:4].tolist()


def csr_matvec(ptr, idx, val, x):
    """y = A x for an exported CSR matrix (numpy; summation order irrelevant at test tolerance)."""
    rows = len(ptr) - 1
    r = np.repeat(np.arange(rows), np.diff(ptr))
    return np.bincount(r, weights=val * x[idx], minlength=rows)


def set_parallel_rows(on):
    """Row loops of the oracle's sparse products on OpenMP threads (results unchanged;
    the default, serial, is what the CPU baseline times)."""
    lib().cpmref_set_parallel_rows(1 if on else 0)


def closest_points(surface, x):
    x = np.ascontiguousarray(x, np.float64)
    n = x.shape[0]
    cp = np.zeros((n, 3))
    dist = np.zeros(n)
    _check(lib().cpmref_closest_points(ctypes.byref(surface), n, _ptr(x), _ptr(cp), _ptr(dist)))
    return cp, dist
