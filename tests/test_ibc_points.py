"""IBC curve plot points (Surface::xp(), host code, no GPU): a Circle3D's 100
parameter points lie on the circle in its plane, start where the IBC subset's
breadth-first search starts and close the loop at theta = 2 pi; a Point is
itself; a polyline is its vertices."""
import math

import numpy as np

import cpm_gb300 as cg


def test_circle_points():
    R, c, n = math.sqrt(0.91), np.array([0.0, 0.0, 0.3]), np.array([0.0, 0.0, 1.0])
    xp = cg.ibc_plot_points(cg.desc(cg.CIRCLE3D, [R, *c, *n]))
    assert xp.shape == (100, 3)
    assert np.allclose(np.linalg.norm(xp - c, axis=1), R, atol=1e-14)
    assert np.allclose((xp - c) @ n, 0.0, atol=1e-14)
    assert np.allclose(xp[0], xp[-1], atol=1e-14)
    ang = np.unwrap(np.arctan2(xp[:, 1] - c[1], xp[:, 0] - c[0]))
    assert np.allclose(np.diff(ang), np.diff(ang)[0], atol=1e-12)
    assert abs(abs(ang[-1] - ang[0]) - 2 * math.pi) < 1e-12


def test_point_and_polyline_points():
    assert np.array_equal(cg.ibc_plot_points(cg.desc(cg.POINT, [0.36, 0.48, 0.8])), [[0.36, 0.48, 0.8]])
    v = np.array([[1.0, 0, 0], [0, 1.0, 0], [-1.0, 0, 0]])
    s = np.array([[0, 1], [1, 2]])
    assert np.array_equal(cg.ibc_plot_points(cg.desc(cg.POLYLINE, (), verts=v, prims=s)), v)
