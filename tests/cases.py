"""Seeded scenes shared by the golden-fixture generator, the parity tests,
__graft_entry__.smoke() and bench.py.  Every field comes from the
deterministic generator in contour3d_gb300/csrc/fieldgen.h, so the same case
yields the same input bytes on every machine."""
from __future__ import annotations

import numpy as np

from contour3d_gb300 import _abi, fields

CAM0 = (2.5, 2.0, 1.5)
CENTRE = (0.5, 0.5, 0.5)


def blobs_small():
    f = fields.blobs((24, 20, 28), nblobs=6, seed=3)
    s = _abi.make_scene(CAM0, CENTRE, 160, 120)
    s.contours = [_abi.Contour(f, 0.5, (0, 255, 255))]
    s.lines = _abi.cube_edges(nitems=5, width=2.0)
    return s


def modes_warp(width=128, height=96):
    f, std = fields.modes((17, 13, 21), nmodes=16, kmin=1, kmax=4, power=5.0 / 6.0, seed=7)
    s = _abi.make_scene((2.2, -1.6, 1.8), CENTRE, width, height, light=(1.0, 0.5, -0.5))
    s.contours = [_abi.Contour(f, -0.5 * std, (255, 128, 0), converter="warp"),
                  _abi.Contour(f, 0.5 * std, (64, 200, 255), converter="warp")]
    return s


def degenerate():
    """Node values equal to the threshold: coincident vertices, zero-area
    triangles, NaN face normals (triangulate.c:89-91)."""
    k, j, i = np.meshgrid(np.arange(14), np.arange(12), np.arange(13), indexing="ij")
    f = ((i + 2 * j + 3 * k) % 4).astype(np.float64)
    s = _abi.make_scene(CAM0, CENTRE, 96, 80)
    s.contours = [_abi.Contour(f, 1.0, (255, 255, 0)), _abi.Contour(f, 2.0, (0, 255, 0))]
    return s


def empty():
    f = fields.blobs((16, 16, 16), nblobs=4, seed=5)
    s = _abi.make_scene(CAM0, CENTRE, 64, 48, bg=(10, 20, 30))
    s.contours = [_abi.Contour(f, 10.0, (255, 0, 0))]
    s.lines = _abi.cube_edges(nitems=3, width=3.0, color=(200, 200, 200))
    return s


def tiny():
    rng = np.random.default_rng(11)
    a = rng.random((4, 4, 4))
    b = rng.random((3, 3, 3))
    s = _abi.make_scene(CAM0, CENTRE, 64, 64)
    s.contours = [_abi.Contour(a, 0.5, (255, 0, 255)), _abi.Contour(b, 0.5, (0, 0, 255))]
    return s


def camera_inside():
    """Camera inside the volume: vertices behind it or beyond the screen plane fail
    projection and their triangles are dropped (render.c:62-72, project.c:39-46)."""
    f = fields.blobs((22, 22, 22), nblobs=8, seed=9)
    s = _abi.make_scene((0.5, 0.45, 0.55), (0.5, 0.5, 0.0), 100, 100, view_height=0.8)
    s.contours = [_abi.Contour(f, 0.4, (220, 220, 220))]
    s.lines = _abi.cube_edges(nitems=9, width=1.5)
    return s


def nonuniform_multi():
    """Stretched grids, two fields, three objects, lines of several widths."""
    def stretched(n):
        u = np.arange(n, dtype=np.float64) / float(n - 1)
        return u + 0.3 * u * (1.0 - u) * (u - 0.5)
    a = fields.blobs((18, 21, 19), nblobs=5, seed=21)
    b, std = fields.modes((20, 16, 24), nmodes=8, kmin=1, kmax=3, power=1.0, seed=22)
    s = _abi.make_scene((-1.2, 2.4, 1.9), CENTRE, 150, 110)
    g = (stretched(19), stretched(21), stretched(18))
    s.contours = [_abi.Contour(a, 0.45, (255, 80, 80), grids=g),
                  _abi.Contour(b, 0.0, (80, 255, 80)),
                  _abi.Contour(a, 0.7, (80, 80, 255), grids=g)]
    s.lines = [_abi.Line((0, 0, 0), (1, 1, 1), 2, (255, 255, 255), 1.5),
               _abi.Line((1, 0, 0), (0, 1, 1), 17, (255, 0, 255), 5.0),
               _abi.Line((0, 1, 0), (0, 1, 1), 4, (0, 255, 255), 0.5)]
    return s


SMALL_CASES = {
    "blobs_small": blobs_small,
    "modes_warp": modes_warp,
    "degenerate": degenerate,
    "empty": empty,
    "tiny": tiny,
    "camera_inside": camera_inside,
    "nonuniform_multi": nonuniform_multi,
}


def config0():
    """Plain method, small: 128^3 f64 Gaussian blobs (8), one threshold 0.5,
    camera (2.5, 2.0, 1.5) looking at the cube centre, 1024 x 1024."""
    f = fields.blobs((128, 128, 128), nblobs=8, seed=0)
    s = _abi.make_scene(CAM0, CENTRE, 1024, 1024)
    s.contours = [_abi.Contour(f, 0.5, (0, 255, 255))]
    return s


def config1_params():
    """Plain method at scale: 512^3 f64, 64 Fourier modes |k| in 1..16,
    amplitude |k|^(-5/6), thresholds +-0.5 std, 1920 x 1080."""
    return dict(shape=(512, 512, 512), nmodes=64, kmin=1, kmax=16, power=5.0 / 6.0, seed=1,
                width=1920, height=1080)


def config1_scene(std: float, shape=(512, 512, 512)):
    s = _abi.make_scene(CAM0, CENTRE, 1920, 1080)
    s.contours = []
    return s, [(-0.5 * std, (0, 255, 255)), (0.5 * std, (255, 255, 0))]
