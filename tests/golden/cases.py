"""Shared definitions of the small parity cases (cutters, degenerate meshes,
paths) used by the golden-fixture generator and the tests."""
from __future__ import annotations

import math

import numpy as np

from opencamlib_gb300 import cutters as cu

# The five cutters of the precision workload plus the other composite presets.
CUTTERS = {
    "cyl": lambda: cu.CylCutter(6.0, 20.0),
    "ball": lambda: cu.BallCutter(6.0, 20.0),
    "bull": lambda: cu.BullCutter(6.0, 1.0, 20.0),
    "cone": lambda: cu.ConeCutter(6.0, math.pi / 4, 20.0),
    "ballcone": lambda: cu.BallConeCutter(2.0, 6.0, math.pi / 4),
    "bullcone": lambda: cu.BullConeCutter(4.0, 1.0, 8.0, math.pi / 4),
    "cylcone": lambda: cu.CylConeCutter(2.0, 6.0, math.pi / 4),
    "conecone": lambda: cu.ConeConeCutter(2.0, math.pi / 3, 6.0, math.pi / 5),
}


def degenerate_mesh() -> np.ndarray:
    """Hand-made triangles that hit the special cases of the contact code:
    a horizontal square (facet special case), a vertical wall (no facet
    drop), a triangle with a vertical edge, a steep facet, a 4-triangle tent
    sharing an apex (shared vertices/edges), a nearly horizontal facet (near
    the 1e-7 tolerance), and a triangle with a horizontal edge."""
    T = [
        (0, 0, 5, 10, 0, 5, 10, 10, 5),
        (0, 0, 5, 10, 10, 5, 0, 10, 5),
        (20, 0, 0, 30, 0, 0, 25, 0, 8),
        (40, 0, 0, 40, 0, 6, 48, 5, 2),
        (60, 0, 0, 61, 10, 12, 70, 0, 1),
        (80, 0, 2, 90, 0, 2, 85, 5, 8),
        (90, 0, 2, 90, 10, 2, 85, 5, 8),
        (90, 10, 2, 80, 10, 2, 85, 5, 8),
        (80, 10, 2, 80, 0, 2, 85, 5, 8),
        (0, 20, 3, 10, 20, 3 + 1e-8, 0, 30, 3),
        (100, 0, 3, 110, 0, 3, 105, 8, 0),
        (20, 20, 1, 35, 22, 9, 24, 33, 4),
    ]
    return np.array(T, dtype=np.float64)


def degenerate_points() -> np.ndarray:
    """CL points on vertices, edges, bbox boundaries, and a raster."""
    P = [(0, 0), (10, 10), (5, 5), (5, 0), (-3, 5), (13, 5), (25, 0), (25, 0.5), (40, 0), (40, 3),
         (85, 5), (85, 0), (80, 5), (61, 10), (105, 0), (105, 4), (5, 25), (200, 200), (27, 27), (-3.0000001, 5)]
    pts = [(x, y, -50.0) for x, y in P] + [(5.0, 5.0, 100.0), (85.0, 5.0, 7.999)]
    xs = np.arange(-4.0, 114.0, 1.7)
    ys = np.arange(-4.0, 36.0, 1.3)
    X, Y = np.meshgrid(xs, ys)
    raster = np.stack([X.ravel(), Y.ravel(), np.full(X.size, -50.0)], axis=1)
    return np.concatenate([np.array(pts, dtype=np.float64), raster], axis=0)


def path_spans() -> np.ndarray:
    """Lines and arcs (both directions, one nearly full circle); rows are
    [type, p1.xyz, p2.xyz, c.xyz, dir]."""
    return np.array([
        [0, 5, 5, 0, 90, 20, 0, 0, 0, 0, 0],
        [0, 90, 20, 3, 60, 80, -1, 0, 0, 0, 0],
        [1, 60, 80, 0, 40, 60, 0, 40, 80, 0, 1],
        [1, 40, 60, 0, 20, 40, 0, 30, 50, 0, 0],
        [1, 20, 40, 0, 20, 40.000001, 0, 30, 40, 0, 1],
    ], dtype=np.float64)
