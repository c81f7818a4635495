"""Synthetic surfaces and boundary curves of the benchmark configurations.

The reference's examples read meshes and curves from files (OBJ and CSV,
src/SimplePolygonMesh.cpp:139, src/Helpers.cpp:11-82); the configurations here
are generated instead, from seeds:

* ``perturbed_icosphere``: an icosphere subdivided ``level`` times, each vertex
  moved radially by a seeded sum of real spherical harmonics of degree <= lmax,
  then scaled into a unit bounding box centred at the origin.
* ``plane_loops``: closed polylines where a plane cuts a closed triangle mesh
  (the curve's vertices lie on mesh edges, so the curve lies on the surface).
* ``mesh_bbox``: the bounding interval the reference derives from a mesh
  (SurfaceSpecifier::SetSurface, src/SurfaceSpecifier.cpp:346-361).
"""
import math

import numpy as np

# ---------------------------------------------------------------- icosphere


def icosphere(level):
    """Unit icosphere: the icosahedron with every triangle split into four
    ``level`` times, new vertices projected to the sphere.  Returns
    (vertices [V,3] float64, faces [F,3] int64); F = 20 * 4**level."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    verts = np.array(v, dtype=np.float64)
    verts /= np.linalg.norm(verts, axis=1, keepdims=True)
    faces = np.array(f, dtype=np.int64)
    for _ in range(level):
        # one midpoint per undirected edge
        e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
        key = np.minimum(e[:, 0], e[:, 1]) * len(verts) + np.maximum(e[:, 0], e[:, 1])
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = uniq // len(verts), uniq % len(verts)
        mid = verts[a] + verts[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(verts)
        verts = np.concatenate([verts, mid])
        nf = len(faces)
        m01, m12, m20 = (base + inv[:nf], base + inv[nf:2 * nf], base + inv[2 * nf:])
        v0, v1, v2 = faces[:, 0], faces[:, 1], faces[:, 2]
        faces = np.concatenate([np.stack([v0, m01, m20], 1), np.stack([v1, m12, m01], 1), np.stack([v2, m20, m12], 1),
                                np.stack([m01, m12, m20], 1)])
    return verts, faces


# ---------------------------------------------------------------- spherical harmonics


def _legendre(l, m, x):
    """Associated Legendre P_l^m(x), m >= 0, with the Condon-Shortley phase (recurrence in l)."""
    pmm = np.ones_like(x)
    if m > 0:
        s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
        fact = 1.0
        for _ in range(m):
            pmm = -pmm * fact * s
            fact += 2.0
    if l == m:
        return pmm
    pm1 = x * (2 * m + 1) * pmm
    if l == m + 1:
        return pm1
    for ll in range(m + 2, l + 1):
        pll = ((2 * ll - 1) * x * pm1 - (ll + m - 1) * pmm) / (ll - m)
        pmm, pm1 = pm1, pll
    return pm1


def real_sph_harm(l, m, theta, phi):
    """Orthonormal real spherical harmonic Y_lm at polar angle theta, azimuth phi."""
    am = abs(m)
    k = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
    p = _legendre(l, am, np.cos(theta))
    if m > 0:
        return math.sqrt(2.0) * k * p * np.cos(m * phi)
    if m < 0:
        return math.sqrt(2.0) * k * p * np.sin(am * phi)
    return k * p


def perturbed_icosphere(level=7, n_harmonics=8, lmax=6, amplitude=0.1, seed=0):
    """Icosphere with vertices at radius 1 + amplitude * S / max|S|, S a seeded
    sum of n_harmonics real spherical harmonics (degrees 1..lmax, orders and
    N(0,1) coefficients drawn from the seed), then scaled so the bounding box's
    largest side is 1 and centred at the origin."""
    rng = np.random.default_rng(seed)
    verts, faces = icosphere(level)
    theta = np.arccos(np.clip(verts[:, 2], -1.0, 1.0))
    phi = np.arctan2(verts[:, 1], verts[:, 0])
    s = np.zeros(len(verts))
    for _ in range(n_harmonics):
        l = int(rng.integers(1, lmax + 1))
        m = int(rng.integers(-l, l + 1))
        s += rng.standard_normal() * real_sph_harm(l, m, theta, phi)
    r = 1.0 + amplitude * s / np.max(np.abs(s))
    verts = verts * r[:, None]
    lo, hi = verts.min(axis=0), verts.max(axis=0)
    verts = (verts - 0.5 * (lo + hi)) / np.max(hi - lo)
    return verts, faces


def mesh_bbox(verts):
    """SurfaceSpecifier::SetSurface: [min(0, all coordinates), max(0, all coordinates)]."""
    return (float(min(0.0, verts.min())), float(max(0.0, verts.max())))


# ---------------------------------------------------------------- curves on a mesh


def plane_loops(verts, faces, normal, offset):
    """Closed polylines where the plane normal . x = offset cuts the mesh.

    Vertex heights that are exactly zero are moved off the plane so every
    crossing is on an edge interior; each triangle with vertices on both sides
    contributes one segment between its two crossed edges, and segments are
    chained through shared edges.  Returns a list of loops, each
    (points [n,3], segments [n,2])."""
    n = np.asarray(normal, np.float64)
    n = n / np.linalg.norm(n)
    h = verts @ n - offset
    h = np.where(h == 0.0, 1e-300, h)
    pos = h > 0
    cnt = pos[faces].sum(axis=1)
    cut = np.nonzero((cnt == 1) | (cnt == 2))[0]
    edge_pt = {}

    def point(a, b):
        k = (min(a, b), max(a, b))
        if k not in edge_pt:
            t = h[k[0]] / (h[k[0]] - h[k[1]])
            edge_pt[k] = verts[k[0]] + t * (verts[k[1]] - verts[k[0]])
        return k

    adj = {}
    for fi in cut:
        f = faces[fi]
        ks = [point(f[a], f[b]) for a, b in ((0, 1), (1, 2), (2, 0)) if pos[f[a]] != pos[f[b]]]
        assert len(ks) == 2
        adj.setdefault(ks[0], []).append(ks[1])
        adj.setdefault(ks[1], []).append(ks[0])
    loops = []
    seen = set()
    for start in adj:
        if start in seen:
            continue
        chain = [start]
        seen.add(start)
        prev, cur = None, start
        while True:
            nxt = [k for k in adj[cur] if k != prev]
            if not nxt or nxt[0] == start:
                break
            prev, cur = cur, nxt[0]
            if cur in seen:
                break
            seen.add(cur)
            chain.append(cur)
        pts = np.array([edge_pt[k] for k in chain])
        m = len(pts)
        segs = np.stack([np.arange(m), (np.arange(m) + 1) % m], axis=1).astype(np.int64)
        loops.append((pts, segs))
    return loops


def parallel_plane_curves(verts, faces, count, seed=0, spread=0.8):
    """``count`` closed curves on a mesh from parallel planes with a seeded
    normal, offsets evenly spaced over ``spread`` times the mesh's extent along
    it (with a seeded jitter of a tenth of the spacing); the largest loop of
    each cut.  Parallel cuts keep the curves apart."""
    rng = np.random.default_rng(seed)
    n = rng.standard_normal(3)
    n /= np.linalg.norm(n)
    h = verts @ n
    lo, hi = h.min(), h.max()
    c0 = 0.5 * (lo + hi) - 0.5 * spread * (hi - lo)
    step = spread * (hi - lo) / count
    curves = []
    for k in range(count):
        off = c0 + (k + 0.5) * step + 0.1 * step * (rng.random() - 0.5)
        loops = plane_loops(verts, faces, n, off)
        curves.append(max(loops, key=lambda lp: len(lp[0])))
    return curves, n


# ---------------------------------------------------------------- the serving mix


def serving_surfaces(cg, dx_scale=1.0, mesh_level=7, n_curves=16, seed=3):
    """The three surfaces of the serving stream, each with fixed Dirichlet IBC
    curves (order 2, on_ibc_tolerance 0.1 dx^2):

    * the unit sphere at dx = 0.025 with the circles z = 0.3 and z = -0.5;
    * the torus R = 1, r = 0.4 at dx = 0.01 with its outer and inner equators;
    * the perturbed icosphere (``perturbed_icosphere(mesh_level)``) at
      dx = 0.005 with ``n_curves`` parallel plane cuts.

    dx_scale multiplies every dx (smaller configurations for tests)."""
    from .serving import ServedSurface

    def circ(R, z, dx, bb):
        return cg.desc(cg.CIRCLE3D, [R, 0, 0, z, 0, 0, 1], bb, boundary_order=2, on_ibc_tolerance=0.1 * dx * dx)

    out = []
    dx = 0.025 * dx_scale
    T = cg.Tube(cg.desc(cg.SPHERE, [1.0]), 3, dx)
    out.append(ServedSurface("sphere", T, [circ(math.sqrt(1 - 0.09), 0.3, dx, (-1.0, 1.0)),
                                           circ(math.sqrt(1 - 0.25), -0.5, dx, (-1.0, 1.0))]))
    dx = 0.01 * dx_scale
    bb = (-1.4, 1.4)
    T = cg.Tube(cg.desc(cg.TORUS, [1.0, 0.4], bb), 3, dx)
    out.append(ServedSurface("torus", T, [circ(1.4, 0.0, dx, bb), circ(0.6, 0.0, dx, bb)]))
    dx = 0.005 * dx_scale
    v, f = perturbed_icosphere(mesh_level, seed=seed)
    bb = mesh_bbox(v)
    T = cg.Tube(cg.desc(cg.TRIANGULATION, (), bb, verts=v, prims=f), 3, dx)
    curves, _ = parallel_plane_curves(v, f, n_curves, seed=seed + 1)
    out.append(ServedSurface("mesh", T, [cg.desc(cg.POLYLINE, (), bb, boundary_order=2, on_ibc_tolerance=0.1 * dx * dx,
                                                 verts=p, prims=s) for p, s in curves]))
    return out
