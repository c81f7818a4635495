"""ctypes binding of libcpmgpu.so, the C-ABI of the GB300 closest-point solve path.

Class and method names follow the reference's C++ interface (Tube, Solver,
problems) so that tests read like the reference's drivers.  There is no CPU
fallback: if the CUDA library is missing or no GPU is present the calls fail.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(os.path.dirname(HERE))  # .../cpm-ibc_gb300
LIB_PATH = os.path.join(PKG, "_build", "libcpmgpu.so")

SPHERE, TORUS, CIRCLE3D, POINT, TRIANGULATION, POLYLINE = range(6)
STATUS = {0: "OK", -1: "INVALID_ARG", -2: "CUDA_ERROR", -3: "OOM", -4: "BASEPOINT_OUTSIDE_TUBE", -5: "NOT_CONVERGED",
          -6: "BREAKDOWN", -7: "UNSUPPORTED", -8: "ADMISSION", -9: "TIMEOUT"}


class CpmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class SurfaceDesc(ctypes.Structure):
    """struct cpm_surface_desc (include/cpm_gpu.h)."""

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


class CpTable(ctypes.Structure):
    """struct cpm_cp_table: caller-computed closest points at query points"""

    _fields_ = [("n", ctypes.c_int64), ("x", ctypes.c_void_p), ("cp", ctypes.c_void_p), ("dist", ctypes.c_void_p)]


def cp_table(x, cp, dist=None):
    """a CpTable over numpy arrays (kept alive on the returned object)"""
    x = np.ascontiguousarray(x, np.float64).reshape(-1, 3)
    cp = np.ascontiguousarray(cp, np.float64).reshape(-1, 3)
    t = CpTable(n=len(x), x=x.ctypes.data, cp=cp.ctypes.data)
    t._keep = [x, cp]
    if dist is not None:
        d = np.ascontiguousarray(dist, np.float64).reshape(-1)
        t.dist = d.ctypes.data
        t._keep.append(d)
    return t


class TubeInfo(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_int64), ("n1d", ctypes.c_int64), ("n_bricks", ctypes.c_int64),
                ("n_visited", ctypes.c_int64), ("dx", ctypes.c_double), ("xstart", ctypes.c_double),
                ("radius", ctypes.c_double), ("p", ctypes.c_int32), ("pad", ctypes.c_int32)]


class TuneResult(ctypes.Structure):
    _fields_ = [("e32_blocks_per_sm", ctypes.c_int32), ("patch_blocks_per_sm", ctypes.c_int32),
                ("e64_blocks_per_sm", ctypes.c_int32), ("e32_us", ctypes.c_float), ("patch_us", ctypes.c_float),
                ("e64_us", ctypes.c_float), ("e32_default_us", ctypes.c_float), ("patch_default_us", ctypes.c_float),
                ("e64_default_us", ctypes.c_float)]


class SolveOpts(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("max_iters", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("precond", ctypes.c_int32), ("precond_iters", ctypes.c_int32), ("inner_tol", ctypes.c_double),
                ("max_refine", ctypes.c_int32), ("refine_every", ctypes.c_int32)]


class SolveStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("refinements", ctypes.c_int32), ("restarts", ctypes.c_int32),
                ("status", ctypes.c_int32), ("rel_residual", ctypes.c_double), ("seconds", ctypes.c_double),
                ("fp64_fallback", ctypes.c_int32), ("pad", ctypes.c_int32)]


def ibc_plot_points(d):
    """Surface::xp() of an IBC curve: a Circle3D's 100 parameter points, a Point, or a polyline's vertices"""
    n = ctypes.c_int64()
    _check(lib().cpm_ibc_plot_points(ctypes.byref(d), ctypes.byref(n), None))
    xp = np.zeros((n.value, 3))
    _check(lib().cpm_ibc_plot_points(ctypes.byref(d), ctypes.byref(n), _p(xp)))
    return xp


def closest_points(d, x, max_dist=0.0):
    """Surface::ClosestPoint (src/Surface.cpp:61-190) on the device for the points x (n, 3):
    (cp (n, 3), dist (n,)).  max_dist > 0 bounds mesh and polyline searches."""
    x = np.ascontiguousarray(np.atleast_2d(x), np.float64)
    L = lib()
    L.cpm_closest_points.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p,
                                     ctypes.c_void_p]
    cp = np.zeros_like(x)
    dist = np.zeros(len(x))
    _check(L.cpm_closest_points(ctypes.byref(d), len(x), _p(x), float(max_dist), _p(cp), _p(dist)))
    return cp, dist


def desc(kind, params=(), bbox=(-1.0, 1.0), boundary_order=1, on_ibc_tolerance=0.0, verts=None, prims=None,
         boundary_type=(0, 0)):
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


_lib = None


def lib():
    """Load the CUDA library; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise CpmError(-2, f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        L = ctypes.CDLL(LIB_PATH)
        vp, P = ctypes.c_void_p, ctypes.POINTER
        L.cpm_last_error.restype = ctypes.c_char_p
        L.cpm_device_info.argtypes = [ctypes.c_char_p, ctypes.c_int64, vp, vp, vp]
        L.cpm_tube_build.argtypes = [P(SurfaceDesc), ctypes.c_int32, ctypes.c_double, P(vp)]
        L.cpm_tube_build_from_cp.argtypes = [P(SurfaceDesc), ctypes.c_int32, ctypes.c_double, ctypes.c_int64, vp, vp, vp,
                                             P(vp)]
        L.cpm_tube_info_get.argtypes = [vp, P(TubeInfo)]
        L.cpm_tube_export.argtypes = [vp] * 8
        L.cpm_tube_reference_order.argtypes = [vp, vp]
        L.cpm_interp_query.argtypes = [vp, ctypes.c_int64, vp, vp, vp]
        L.cpm_tube_destroy.argtypes = [vp]
        L.cpm_opset_create.argtypes = [vp, ctypes.c_int32, P(SurfaceDesc), P(vp)]
        L.cpm_opset_create_identity.argtypes = [vp, ctypes.c_int64, vp, P(vp)]
        L.cpm_opset_create_from_cp.argtypes = [vp, ctypes.c_int32, P(SurfaceDesc), P(CpTable), P(CpTable), P(vp)]
        L.cpm_tube_nearest.argtypes = [vp, ctypes.c_int64, vp, vp]
        L.cpm_ibc_plot_points.argtypes = [P(SurfaceDesc), vp, vp]
        L.cpm_opset_sizes.argtypes = [vp, vp]
        L.cpm_opset_rows.argtypes = [vp] * 5
        L.cpm_opset_row_sides.argtypes = [vp, vp]
        L.cpm_opset_ibc_sizes.argtypes = [vp, ctypes.c_int32, vp]
        L.cpm_opset_ibc_export.argtypes = [vp, ctypes.c_int32, vp, vp, vp]
        L.cpm_opset_export_csr.argtypes = [vp, ctypes.c_int32, vp, vp, vp, vp]
        L.cpm_opset_plot_interp.argtypes = [vp, ctypes.c_int64, vp, vp, vp]
        L.cpm_opset_plot_interp_csr.argtypes = [vp, ctypes.c_int64, vp, vp, vp, vp, vp]
        L.cpm_explicit_step.argtypes = [vp, ctypes.c_double, ctypes.c_int32, vp, vp]
        L.cpm_gray_scott_step.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_double, vp, vp]
        L.cpm_opset_destroy.argtypes = [vp]
        L.cpm_apply.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_int32, vp, vp]
        L.cpm_apply_device.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_int32, ctypes.c_int32, vp, vp, vp]
        L.cpm_get_stream.restype = ctypes.c_void_p
        L.cpm_launch_count.restype = ctypes.c_int64
        L.cpm_sync.restype = ctypes.c_int
        L.cpm_set_thread_stream.argtypes = [vp]
        L.cpm_opset_autotune.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, P(TuneResult)]
        L.cpm_opset_set_launch.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]
        L.cpm_solver_create.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_int32, P(vp)]
        L.cpm_solve.argtypes = [vp, ctypes.c_int32, vp, vp, P(SolveOpts), P(SolveStats)]
        L.cpm_solve_device.argtypes = [vp, ctypes.c_int32, vp, vp, P(SolveOpts), P(SolveStats)]
        L.cpm_solver_destroy.argtypes = [vp]
        L.cpm_server_create.argtypes = [vp, ctypes.c_double, ctypes.c_double, P(SolveOpts), P(vp)]
        L.cpm_server_create_batches.argtypes = [vp, ctypes.c_double, ctypes.c_double, P(SolveOpts), ctypes.c_int32, P(vp)]
        L.cpm_server_submit.argtypes = [vp, vp, ctypes.c_int64]
        L.cpm_server_submit_device.argtypes = [vp, vp, vp, ctypes.c_int64]
        L.cpm_server_step.argtypes = [vp, vp, vp, vp]
        L.cpm_server_step_async.argtypes = [vp, vp, vp, vp]
        L.cpm_server_poll.argtypes = [vp, vp, vp, P(SolveStats), vp]
        L.cpm_server_destroy.argtypes = [vp]
        L.cpm_server_device_bytes.argtypes = [vp]
        L.cpm_server_device_bytes.restype = ctypes.c_int64
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise CpmError(rc, lib().cpm_last_error().decode())


def _p(a):
    return None if a is None else a.ctypes.data


def device_info():
    name = ctypes.create_string_buffer(256)
    fr, to, sm = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32()
    _check(lib().cpm_device_info(name, 256, ctypes.byref(fr), ctypes.byref(to), ctypes.byref(sm)))
    return dict(name=name.value.decode(), free=fr.value, total=to.value, sms=sm.value)


class Tube:
    """Tube(SurfaceSpecifier&, p, dx) (src/Tube.h:45) built on the device."""

    def __init__(self, surface, p=3, dx=0.1, _handle=None):
        self.surface = surface
        if _handle is None:
            h = ctypes.c_void_p()
            _check(lib().cpm_tube_build(ctypes.byref(surface), p, dx, ctypes.byref(h)))
            _handle = h
        self.h = _handle
        info = TubeInfo()
        _check(lib().cpm_tube_info_get(self.h, ctypes.byref(info)))
        self.N, self.N1d, self.n_bricks, self.n_visited = info.n_nodes, info.n1d, info.n_bricks, info.n_visited
        self.dx, self.xstart, self.radius, self.p = info.dx, info.xstart, info.radius, info.p

    @classmethod
    def from_closest_points(cls, surface, p, dx, keys, cp, dist):
        keys = np.asarray(keys, np.int64)
        o = np.argsort(keys, kind="stable")
        k = np.ascontiguousarray(keys[o])
        c = np.ascontiguousarray(np.asarray(cp, np.float64)[o])
        d = np.ascontiguousarray(np.asarray(dist, np.float64)[o])
        h = ctypes.c_void_p()
        _check(lib().cpm_tube_build_from_cp(ctypes.byref(surface), p, dx, len(k), _p(k), _p(c), _p(d), ctypes.byref(h)))
        return cls(surface, _handle=h)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().cpm_tube_destroy(self.h)
        except Exception:
            pass

    def export(self):
        N = self.N
        out = dict(rec=np.zeros(N, np.int64), x=np.zeros((N, 3)), cp=np.zeros((N, 3)), dist=np.zeros(N),
                   bpt=np.zeros(N, np.int64), nbr=np.zeros((N, 6), np.int64), w=np.zeros((N, 3, 4)))
        _check(lib().cpm_tube_export(self.h, _p(out["rec"]), _p(out["x"]), _p(out["cp"]), _p(out["dist"]),
                                     _p(out["bpt"]), _p(out["nbr"]), _p(out["w"])))
        return out

    def reference_order(self):
        """Device index of each node in the reference's tube numbering (its BFS flood order)."""
        order = np.zeros(self.N, np.int64)
        _check(lib().cpm_tube_reference_order(self.h, _p(order)))
        return order

    def nearest(self, x):
        """Tube::NearestTubeIndex: device index of the node at each point's nearest grid point, or -1"""
        x = np.ascontiguousarray(np.atleast_2d(x), np.float64)
        idx = np.zeros(x.shape[0], np.int64)
        _check(lib().cpm_tube_nearest(self.h, x.shape[0], _p(x), _p(idx)))
        return idx

    def interp_query(self, xq):
        """Interpolation(Tube&, xq) rows: 64 (column, value) per query point."""
        xq = np.ascontiguousarray(xq, np.float64)
        n = xq.shape[0]
        cols = np.zeros((n, 64), np.int64)
        vals = np.zeros((n, 64))
        _check(lib().cpm_interp_query(self.h, n, _p(xq), _p(cols), _p(vals)))
        return cols, vals


class OpSet:
    """Lfull / Efull / identity rows (Helpers::SetupMatrices + IBCMatrixManipulations) on the device."""

    def __init__(self, tube, ibcs=(), identity_rows=None, ibc_cp=None, surface_cp=None):
        """identity_rows (device tube indices): the nearest-node baselines' operator,
        plain L and E with Dirichlet rows there (no IBC columns; ibcs must be empty).
        ibc_cp (one CpTable per IBC) and surface_cp (a CpTable): closest points
        computed by the caller (cpm_opset_create_from_cp)"""
        self.tube = tube
        self.ibcs = list(ibcs)
        h = ctypes.c_void_p()
        if ibc_cp is not None or surface_cp is not None:
            arr = (SurfaceDesc * max(1, len(ibcs)))(*ibcs) if ibcs else None
            tabs = (CpTable * max(1, len(ibcs)))(*(ibc_cp or [CpTable() for _ in ibcs])) if ibcs else None
            _check(lib().cpm_opset_create_from_cp(tube.h, len(ibcs), arr, tabs,
                                                  ctypes.byref(surface_cp) if surface_cp is not None else None,
                                                  ctypes.byref(h)))
        elif identity_rows is not None:
            if ibcs:
                raise ValueError("identity_rows and IBC curves are exclusive")
            rows = np.ascontiguousarray(identity_rows, np.int64)
            _check(lib().cpm_opset_create_identity(tube.h, len(rows), _p(rows), ctypes.byref(h)))
        else:
            arr = (SurfaceDesc * max(1, len(ibcs)))(*ibcs) if ibcs else None
            _check(lib().cpm_opset_create(tube.h, len(ibcs), arr, ctypes.byref(h)))
        self.h = h
        s = np.zeros(9, np.int64)
        _check(lib().cpm_opset_sizes(self.h, _p(s)))
        (self.D, self.N, self.total_ibc_dofs, self.num2, self.n_ibc, self.n_patched, self.n_moved, self.n_patch_rows,
         self.n_patch_entries) = [int(v) for v in s]

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().cpm_opset_destroy(self.h)
        except Exception:
            pass

    def rows(self):
        D = self.D
        ident = np.zeros(D, np.uint8)
        kind = np.zeros(D, np.int32)
        ibc = np.zeros(D, np.int32)
        point = np.zeros((D, 3))
        _check(lib().cpm_opset_rows(self.h, _p(ident), _p(kind), _p(ibc), _p(point)))
        side = np.zeros(D, np.int32)
        _check(lib().cpm_opset_row_sides(self.h, _p(side)))
        return dict(identity=ident.astype(bool), kind=kind, ibc=ibc, point=point, side=side)

    def ibc_subsets(self, c):
        s = np.zeros(5, np.int64)
        _check(lib().cpm_opset_ibc_sizes(self.h, c, _p(s)))
        tag = np.zeros(int(s[0]), np.int64)
        dof = np.zeros(int(s[1]), np.int64)
        cp = np.zeros((int(s[1]), 3))
        _check(lib().cpm_opset_ibc_export(self.h, c, _p(tag), _p(dof), _p(cp)))
        return dict(tag_set=tag, dof_set=dof, dof_cp=cp, col_start=int(s[2]), dcol_start=int(s[3]),
                    identity_rows_start=int(s[4]))

    def csr(self, which):
        nnz = ctypes.c_int64()
        _check(lib().cpm_opset_export_csr(self.h, which, ctypes.byref(nnz), None, None, None))
        ptr = np.zeros(self.D + 1, np.int64)
        idx = np.zeros(nnz.value, np.int64)
        val = np.zeros(nnz.value)
        _check(lib().cpm_opset_export_csr(self.h, which, ctypes.byref(nnz), _p(ptr), _p(idx), _p(val)))
        return ptr, idx, val

    def plot_interp(self, xp):
        """GetPlotInterpMatrix + AddIBCPlotInterpolation: per evaluation point 64
        (column, value) entries in the operator's column layout."""
        xp = np.ascontiguousarray(xp, np.float64)
        n = xp.shape[0]
        cols = np.zeros((n, 64), np.int64)
        vals = np.zeros((n, 64))
        _check(lib().cpm_opset_plot_interp(self.h, n, _p(xp), _p(cols), _p(vals)))
        return cols, vals

    def explicit_step(self, dt, u):
        """HeatWithIBC explicit step: Efull (u + dt Lfull u); u: (D,) or (k, D)."""
        u = np.ascontiguousarray(np.atleast_2d(u), np.float64)
        out = np.zeros_like(u)
        _check(lib().cpm_explicit_step(self.h, dt, u.shape[0], _p(u), _p(out)))
        return out

    def gray_scott_step(self, dt, u, v, F=0.054, k=0.063):
        """ReactionDiffusionWithIBC step (before the Dirichlet values): new (u, v)."""
        u = np.array(u, np.float64)
        v = np.array(v, np.float64)
        _check(lib().cpm_gray_scott_step(self.h, dt, F, k, _p(u), _p(v)))
        return u, v

    def plot_interp_csr(self, xp):
        """The evaluation rows as CSR (ptr, cols, vals): each point's 64 entries, then the
        further copies of entries that lie across several IBCs."""
        xp = np.ascontiguousarray(xp, np.float64)
        n = xp.shape[0]
        nnz = ctypes.c_int64(0)
        _check(lib().cpm_opset_plot_interp_csr(self.h, n, _p(xp), ctypes.byref(nnz), None, None, None))
        ptr = np.zeros(n + 1, np.int64)
        cols = np.zeros(nnz.value, np.int64)
        vals = np.zeros(nnz.value)
        _check(lib().cpm_opset_plot_interp_csr(self.h, n, _p(xp), ctypes.byref(nnz), _p(ptr), _p(cols), _p(vals)))
        return ptr, cols, vals

    def evaluate(self, x, xp):
        """u at evaluation points xp from a solution x on the operator's rows"""
        ptr, cols, vals = self.plot_interp_csr(xp)
        prod = vals * np.asarray(x, np.float64)[cols]
        return np.add.reduceat(prod, ptr[:-1]) if len(prod) else np.zeros(len(ptr) - 1)

    def apply(self, m, n, x):
        """Solver::Multiply (src/Solver.cpp:122-138); x: (D,) or (k, D)."""
        x = np.ascontiguousarray(np.atleast_2d(x), np.float64)
        y = np.zeros_like(x)
        _check(lib().cpm_apply(self.h, m, n, x.shape[0], _p(x), _p(y)))
        return y

    def apply_device(self, m, n, kslots, fp32, x_ptr, t_ptr, y_ptr):
        """Asynchronous device apply on the calling thread's library stream ([D][kslots] arrays)."""
        _check(lib().cpm_apply_device(self.h, m, n, kslots, int(fp32), x_ptr, t_ptr, y_ptr))

    def autotune(self, reps=20, fp64=False):
        """Time the 32-slot E passes over candidate launch shapes, keep the fastest with
        this operator (cpm_opset_autotune) and return the chosen shapes and times."""
        r = TuneResult()
        _check(lib().cpm_opset_autotune(self.h, int(reps), int(bool(fp64)), ctypes.byref(r)))
        return {k: getattr(r, k) for k, _ in TuneResult._fields_}

    def set_launch(self, e32_blocks_per_sm=0, patch_blocks_per_sm=0, e64_blocks_per_sm=0):
        """Set the 32-slot E passes' launch shapes by hand (0: the defaults)."""
        _check(lib().cpm_opset_set_launch(self.h, int(e32_blocks_per_sm), int(patch_blocks_per_sm),
                                          int(e64_blocks_per_sm)))


class Geodesic:
    """GeodesicDistance::ComputeDistance (problems/GeodesicDistance.cpp:11-69) from a point source."""

    def __init__(self, tube, source):
        L = lib()
        L.cpm_geodesic_create.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                                          ctypes.POINTER(ctypes.c_int64)]
        L.cpm_geodesic_run.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int32, ctypes.c_double,
                                       ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
        L.cpm_geodesic_destroy.argtypes = [ctypes.c_void_p]
        self.tube = tube
        src = np.ascontiguousarray(source, np.float64)
        h, D = ctypes.c_void_p(), ctypes.c_int64()
        _check(L.cpm_geodesic_create(tube.h, _p(src), ctypes.byref(h), ctypes.byref(D)))
        self.h, self.D = h, D.value

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().cpm_geodesic_destroy(self.h)
        except Exception:
            pass

    def run(self, dt, precision=0, tol=1e-10, heat_sweeps=2000):
        phi = np.zeros(self.D)
        its = np.zeros(4, np.int32)
        _check(lib().cpm_geodesic_run(self.h, dt, precision, tol, heat_sweeps, _p(phi), _p(its)))
        return phi, its.tolist()


class GeodesicBatch:
    """The heat-method geodesic distance from up to 32 sources at once on one
    operator (each source's point IBC applied to its own slot only)."""

    def __init__(self, tube, sources):
        L = lib()
        L.cpm_geodesic_batch_create.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                                ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_int64)]
        L.cpm_geodesic_batch_run.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                             ctypes.c_void_p, ctypes.c_void_p]
        L.cpm_geodesic_batch_destroy.argtypes = [ctypes.c_void_p]
        self.tube = tube
        src = np.ascontiguousarray(np.atleast_2d(sources), np.float64)
        self.n = src.shape[0]
        h, D = ctypes.c_void_p(), ctypes.c_int64()
        _check(L.cpm_geodesic_batch_create(tube.h, self.n, _p(src), ctypes.byref(h), ctypes.byref(D)))
        self.h, self.D = h, D.value

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().cpm_geodesic_batch_destroy(self.h)
        except Exception:
            pass

    def run(self, dt, tol=1e-10, heat_sweeps=2000):
        """phi (n, D): tube rows, then each source's own DOF rows; iterations (n, 4)"""
        phi = np.zeros((self.n, self.D))
        its = np.zeros((self.n, 4), np.int32)
        _check(lib().cpm_geodesic_batch_run(self.h, dt, tol, heat_sweeps, _p(phi), _p(its)))
        return phi, its


class GeodesicNearest:
    """GeodesicDistanceNearest::ComputeDistance (problems/GeodesicDistanceNearest.cpp:11-53):
    identity rows at the constraint nodes `ibc_rows`, smoothed heat sources at
    `inside_rows` (distances `inside_dist`), all device row indices."""

    def __init__(self, tube, ibc_rows, inside_rows=(), inside_dist=()):
        L = lib()
        L.cpm_geodesic_nearest_create.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
        L.cpm_geodesic_nearest_run.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int32, ctypes.c_double,
                                               ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
        L.cpm_geodesic_nearest_destroy.argtypes = [ctypes.c_void_p]
        self.tube = tube
        a = np.ascontiguousarray(ibc_rows, np.int64)
        b = np.ascontiguousarray(inside_rows, np.int64)
        d = np.ascontiguousarray(inside_dist, np.float64)
        if len(b) != len(d):
            raise ValueError("inside_rows and inside_dist differ in length")
        h = ctypes.c_void_p()
        _check(L.cpm_geodesic_nearest_create(tube.h, len(a), _p(a), len(b), _p(b), _p(d), ctypes.byref(h)))
        self.h = h

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().cpm_geodesic_nearest_destroy(self.h)
        except Exception:
            pass

    def run(self, dt, precision=0, tol=1e-10, heat_sweeps=2000):
        """phi on the tube rows (device order) and the 4 iteration counts."""
        phi = np.zeros(self.tube.N)
        its = np.zeros(4, np.int32)
        _check(lib().cpm_geodesic_nearest_run(self.h, dt, precision, tol, heat_sweeps, _p(phi), _p(its)))
        return phi, its.tolist()


def set_device(dev):
    lib().cpm_set_device.argtypes = [ctypes.c_int32]
    _check(lib().cpm_set_device(int(dev)))


def stream_ptr():
    """The calling thread's library cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
    return lib().cpm_get_stream()


def set_thread_stream(ptr):
    """Queue this thread's library work on the cudaStream_t `ptr` (an integer, e.g.
    torch.cuda.Stream().cuda_stream); None or 0 goes back to the library stream."""
    _check(lib().cpm_set_thread_stream(ptr or None))


def launch_count():
    return int(lib().cpm_launch_count())


def sync():
    _check(lib().cpm_sync())


# preconditioners (src/Defines.h:13-18)
IDENTITY, DIAGONAL, JACOBI = 0, 1, 2


class Solver:
    """Solver::Init(m, n, ...) + Solve (src/Solver.cpp:8-114), k right-hand sides per call."""

    def __init__(self, opset, m, n, kslots=1):
        self.opset = opset
        self.m, self.n, self.kslots = m, n, kslots
        h = ctypes.c_void_p()
        _check(lib().cpm_solver_create(opset.h, m, n, kslots, ctypes.byref(h)))
        self.h = h

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().cpm_solver_destroy(self.h)
        except Exception:
            pass

    def solve(self, b, tol=1e-10, precision=0, max_iters=100000, inner_tol=0.0, max_refine=400, raise_on_error=True,
              precond=DIAGONAL, precond_iters=0, refine_every=0):
        b = np.ascontiguousarray(np.atleast_2d(b), np.float64)
        k = b.shape[0]
        x = np.zeros_like(b)
        o = SolveOpts(tol=tol, max_iters=max_iters, precision=precision, precond=precond, precond_iters=precond_iters,
                      inner_tol=inner_tol, max_refine=max_refine, refine_every=refine_every)
        st = (SolveStats * k)()
        rc = lib().cpm_solve(self.h, k, _p(b), _p(x), ctypes.byref(o), st)
        stats = [dict(iterations=s.iterations, refinements=s.refinements, restarts=s.restarts, status=s.status,
                      rel_residual=s.rel_residual, seconds=s.seconds,
                      fp64_fallback=s.fp64_fallback) for s in st]
        if rc != 0 and raise_on_error:
            raise CpmError(rc, lib().cpm_last_error().decode() + f" stats={stats}")
        return x, stats

    def solve_device(self, b_ptr, x_ptr, k, tol=1e-10, precision=0, max_iters=100000, inner_tol=0.0, max_refine=400,
                     precond=DIAGONAL, precond_iters=0, refine_every=0):
        o = SolveOpts(tol=tol, max_iters=max_iters, precision=precision, precond=precond, precond_iters=precond_iters,
                      inner_tol=inner_tol, max_refine=max_refine, refine_every=refine_every)
        st = (SolveStats * k)()
        rc = lib().cpm_solve_device(self.h, k, b_ptr, x_ptr, ctypes.byref(o), st)
        stats = [dict(iterations=s.iterations, refinements=s.refinements, restarts=s.restarts, status=s.status,
                      rel_residual=s.rel_residual, seconds=s.seconds,
                      fp64_fallback=s.fp64_fallback) for s in st]
        if rc != 0:
            raise CpmError(rc, lib().cpm_last_error().decode() + f" stats={stats}")
        return stats


class Server:
    """Continuous batching of right-hand sides on one operator (m, n): up to 32
    in flight in a 32-slot solver (precision 1: FP32 with FP64 reliable
    updates; 0: plain FP64), admitted as slots free up."""

    def __init__(self, opset, m, n, tol=1e-10, inner_tol=0.0, max_refine=400, refine_every=0, max_iters=100000,
                 precision=1, batches=1):
        """batches: 32-slot solvers run concurrently, each on its own stream"""
        self.opset, self.D, self.precision, self.batches = opset, opset.D, precision, batches
        o = SolveOpts(tol=tol, max_iters=max_iters, precision=precision, precond=DIAGONAL, precond_iters=0,
                      inner_tol=inner_tol, max_refine=max_refine, refine_every=refine_every)
        h = ctypes.c_void_p()
        _check(lib().cpm_server_create_batches(opset.h, m, n, ctypes.byref(o), int(batches), ctypes.byref(h)))
        self.h = h

    @staticmethod
    def device_bytes(opset, batches=1):
        return batches * int(lib().cpm_server_device_bytes(opset.h))

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().cpm_server_destroy(self.h)
        except Exception:
            pass

    def submit(self, b, tag):
        b = np.ascontiguousarray(b, np.float64)
        assert b.shape == (self.D,)
        _check(lib().cpm_server_submit(self.h, _p(b), int(tag)))

    def submit_device(self, b_ptr, x_ptr, tag):
        """device right-hand side and solution destination (D doubles each)"""
        _check(lib().cpm_server_submit_device(self.h, b_ptr, x_ptr, int(tag)))

    def step(self, pipelined=False):
        """one admission + iteration-graph + harvest round: (active, queued, finished).
        pipelined: harvest the previous call's graphs, launch the next ones and return
        without waiting (cpm_server_step_async)"""
        a, q, f = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        fn = lib().cpm_server_step_async if pipelined else lib().cpm_server_step
        _check(fn(self.h, ctypes.byref(a), ctypes.byref(q), ctypes.byref(f)))
        return a.value, q.value, f.value

    def poll(self, want_x=True):
        """pop one finished request: (tag, x or None, stats) or None"""
        tag = ctypes.c_int64()
        x = np.empty(self.D) if want_x else None
        st = SolveStats()
        lat = ctypes.c_double()
        got = lib().cpm_server_poll(self.h, ctypes.byref(tag), _p(x) if want_x else None, ctypes.byref(st),
                                    ctypes.byref(lat))
        if got < 0:
            _check(got)
        if got == 0:
            return None
        return tag.value, x, dict(iterations=st.iterations, refinements=st.refinements, restarts=st.restarts,
                                  status=st.status, rel_residual=st.rel_residual, service=st.seconds,
                                  latency=lat.value, fp64_fallback=st.fp64_fallback)

    def drain(self, want_x=True, pipelined=True):
        """step until every submitted request has finished; returns {tag: (x, stats)}.
        Pipelined steps (the default) copy each round's results out while the next
        round's graphs run."""
        out = {}
        while True:
            a, q, _ = self.step(pipelined)
            while True:
                r = self.poll(want_x)
                if r is None:
                    break
                out[r[0]] = (r[1], r[2])
            if a == 0 and q == 0:
                return out
