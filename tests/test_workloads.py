"""Synthetic workload generators (CPU): the icosphere is a closed 2-manifold of
the stated size, the spherical harmonics are orthonormal, and plane cuts give
closed loops lying on the cutting plane."""
import numpy as np

from cpm_gb300 import workloads as W


def test_icosphere_sizes_and_manifold():
    for level in (0, 2, 4):
        v, f = W.icosphere(level)
        assert len(f) == 20 * 4 ** level and len(v) == 10 * 4 ** level + 2
        e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
        _, c = np.unique(e, axis=0, return_counts=True)
        assert np.all(c == 2)
        assert np.allclose(np.linalg.norm(v, axis=1), 1.0)


def test_real_spherical_harmonics_orthonormal():
    # Gauss-Legendre in cos(theta) x uniform phi integrates degree <= 12 products exactly
    xg, wg = np.polynomial.legendre.leggauss(16)
    phi = np.linspace(0, 2 * np.pi, 32, endpoint=False)
    th, ph = np.meshgrid(np.arccos(xg), phi, indexing="ij")
    w = wg[:, None] * np.full(len(phi), 2 * np.pi / len(phi))[None, :]
    lm = [(1, -1), (2, 1), (3, -2), (4, 0), (6, 4), (6, -6)]
    Y = [W.real_sph_harm(l, m, th, ph) for l, m in lm]
    G = np.array([[np.sum(a * b * w) for b in Y] for a in Y])
    assert np.allclose(G, np.eye(len(lm)), atol=1e-12)


def test_perturbed_icosphere_bbox():
    v, f = W.perturbed_icosphere(3, seed=1)
    lo, hi = v.min(0), v.max(0)
    assert np.isclose(np.max(hi - lo), 1.0) and np.allclose(lo + hi, 0.0)
    assert W.mesh_bbox(v) == (float(min(0, v.min())), float(max(0, v.max())))


def test_plane_loops_closed_on_plane():
    v, f = W.perturbed_icosphere(4, seed=2)
    curves, n = W.parallel_plane_curves(v, f, 4, seed=5)
    for pts, segs in curves:
        h = pts @ n
        assert np.ptp(h) < 1e-12  # on one plane
        assert np.array_equal(segs[:, 1], np.roll(segs[:, 0], -1))  # closed chain
        assert len(np.unique(np.round(pts, 14), axis=0)) == len(pts)


def test_break_even_count():
    """Requests waiting from which a 32-slot batch beats one-by-one FP64 solves:
    unknown until the surface's FP64 iteration count is measured; then the
    32-slot iteration cost (in one-RHS FP64 iterations) times the ratio of
    mixed to FP64 iterations (2 until measured), at least 2."""
    from cpm_gb300 import serving as SV

    s = object.__new__(SV.ServedSurface)
    s.precision, s.fp64_iters, s.mixed_iters = 1, None, None
    assert s.break_even() is None
    s.fp64_iters = 247.0
    assert s.break_even() == int(np.ceil(SV.K32_MIXED * 2.0))
    s.mixed_iters = 466.0
    assert s.break_even() == int(np.ceil(SV.K32_MIXED * 466.0 / 247.0))
    s.mixed_iters = 100.0
    assert s.break_even() == 2
    s.precision = 0
    assert s.break_even() == int(np.ceil(SV.K32_FP64))
