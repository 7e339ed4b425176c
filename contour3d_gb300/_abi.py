"""ctypes mirror of include/contour3d.h plus scene helpers.

The structures below have the layout of the reference's public types
(reference include/contour3d.h:10-56), so a `Scene` can be handed to any
library exporting the `contour3d_execute` signature: this package's CUDA
library, or the CPU checkers used by the tests.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np


class Vector(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class Color(C.Structure):
    _fields_ = [("r", C.c_uint8), ("g", C.c_uint8), ("b", C.c_uint8)]


CONVERTER = C.CFUNCTYPE(Vector, Vector)


class ContourObj(C.Structure):
    _fields_ = [
        ("pencil", C.c_int),
        ("glsizes", C.c_size_t * 3),
        ("grids", C.POINTER(C.c_double) * 3),
        ("converter", C.c_void_p),
        ("threshold", C.c_double),
        ("color", Color),
        ("array", C.POINTER(C.c_double)),
    ]


class LineObj(C.Structure):
    _fields_ = [
        ("edges", Vector * 2),
        ("nitems", C.c_size_t),
        ("converter", C.c_void_p),
        ("color", Color),
        ("width", C.c_double),
    ]


def vec(v: Sequence[float]) -> Vector:
    return Vector(float(v[0]), float(v[1]), float(v[2]))


def col(c: Sequence[int]) -> Color:
    return Color(int(c[0]), int(c[1]), int(c[2]))


@dataclass
class Contour:
    """One iso-surface: field[k, j, i] (x fastest in memory), node grids, level."""

    field: np.ndarray
    threshold: float
    color: Tuple[int, int, int] = (0, 255, 255)
    grids: Optional[Tuple[np.ndarray, np.ndarray, np.ndarray]] = None
    converter: str = "identity"  # "identity" or "warp" (a smooth test map)

    def node_grids(self):
        if self.grids is not None:
            return tuple(np.ascontiguousarray(g, dtype=np.float64) for g in self.grids)
        nz, ny, nx = self.field.shape
        return tuple(unit_grid(n) for n in (nx, ny, nz))


@dataclass
class Line:
    start: Tuple[float, float, float]
    end: Tuple[float, float, float]
    nitems: int = 2
    color: Tuple[int, int, int] = (255, 255, 255)
    width: float = 2.0
    converter: str = "identity"


@dataclass
class Scene:
    camera: Tuple[float, float, float]
    look_at: Tuple[float, float, float]
    light: Tuple[float, float, float]
    width: int
    height: int
    center: Tuple[float, float, float]
    local_x: Tuple[float, float, float]
    local_y: Tuple[float, float, float]
    bg: Tuple[int, int, int] = (0, 0, 0)
    contours: List[Contour] = field(default_factory=list)
    lines: List[Line] = field(default_factory=list)


def unit_grid(n: int) -> np.ndarray:
    """Uniform nodes i / (n - 1) on [0, 1], computed as one IEEE division each."""
    return np.arange(n, dtype=np.float64) / float(n - 1)


def look_at_screen(camera, look_at, width, height, view_height=1.0, up=(0.0, 0.0, 1.0)):
    """Screen centre and local axes for a camera looking at `look_at`.

    The screen plane sits half-way between camera and focal point; local_y is
    world `up` made orthogonal to the view direction and scaled to
    `view_height`, local_x = view x up scaled so |local_x| / |local_y| equals
    width / height.  local_x x local_y then points back at the camera, so
    depths (screen normal . ray) are negative and larger means nearer.
    """
    cam = np.asarray(camera, dtype=np.float64)
    tgt = np.asarray(look_at, dtype=np.float64)
    view = tgt - cam
    view = view / np.linalg.norm(view)
    upv = np.asarray(up, dtype=np.float64)
    right = np.cross(view, upv)
    right = right / np.linalg.norm(right)
    upo = np.cross(right, view)
    center = cam + 0.5 * (tgt - cam)
    ly = upo * view_height
    lx = right * view_height * (width / height)
    return tuple(center.tolist()), tuple(lx.tolist()), tuple(ly.tolist())


def make_scene(camera, look_at, width, height, light=(0.0, 2.0, -1.0), view_height=1.0,
               bg=(0, 0, 0)) -> Scene:
    center, lx, ly = look_at_screen(camera, look_at, width, height, view_height)
    return Scene(tuple(camera), tuple(look_at), tuple(light), int(width), int(height),
                 center, lx, ly, tuple(bg))


class ExecuteArgs:
    """ctypes argument pack for a `contour3d_execute`-shaped call.

    `converters` maps "identity"/"warp" to function addresses inside the
    target library.  The pack keeps every buffer it points at alive.
    """

    def __init__(self, scene: Scene, converters: dict, fname: str = "",
                 sdecomp_info: Optional[int] = None):
        self._keep = []
        self.info = C.c_void_p(sdecomp_info)
        self.camera = vec(scene.camera)
        self.look_at = vec(scene.look_at)
        self.light = vec(scene.light)
        self.sizes = (C.c_size_t * 2)(scene.width, scene.height)
        self.center = vec(scene.center)
        self.local = (Vector * 2)(vec(scene.local_x), vec(scene.local_y))
        self.bg = col(scene.bg)
        n = len(scene.contours)
        self.contours = (ContourObj * max(n, 1))()
        for idx, c in enumerate(scene.contours):
            arr = np.ascontiguousarray(c.field, dtype=np.float64)
            g = c.node_grids()
            self._keep += [arr, *g]
            o = self.contours[idx]
            o.pencil = 0
            nz, ny, nx = arr.shape
            o.glsizes[0], o.glsizes[1], o.glsizes[2] = nx, ny, nz
            for d in range(3):
                o.grids[d] = g[d].ctypes.data_as(C.POINTER(C.c_double))
            o.converter = converters[c.converter]
            o.threshold = float(c.threshold)
            o.color = col(c.color)
            o.array = arr.ctypes.data_as(C.POINTER(C.c_double))
        m = len(scene.lines)
        self.lines = (LineObj * max(m, 1))()
        for idx, l in enumerate(scene.lines):
            o = self.lines[idx]
            o.edges[0] = vec(l.start)
            o.edges[1] = vec(l.end)
            o.nitems = int(l.nitems)
            o.converter = converters[l.converter]
            o.color = col(l.color)
            o.width = float(l.width)
        self.num_contours = n
        self.num_lines = m
        self.fname = fname.encode()

    def execute_tuple(self):
        return (self.info, C.byref(self.camera), C.byref(self.look_at), C.byref(self.light),
                self.sizes, C.byref(self.center), self.local, C.byref(self.bg),
                C.c_size_t(self.num_contours), self.contours, C.c_size_t(self.num_lines),
                self.lines, C.c_char_p(self.fname))


def declare_execute(fn) -> None:
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.POINTER(Vector), C.POINTER(Vector), C.POINTER(Vector),
                   C.POINTER(C.c_size_t), C.POINTER(Vector), C.POINTER(Vector),
                   C.POINTER(Color), C.c_size_t, C.POINTER(ContourObj), C.c_size_t,
                   C.POINTER(LineObj), C.c_char_p]


def read_ppm(path: str) -> Tuple[int, int, np.ndarray]:
    with open(path, "rb") as fp:
        data = fp.read()
    parts = data.split(b"\n", 3)
    assert parts[0] == b"P6", parts[0]
    w, h = (int(x) for x in parts[1].split())
    assert parts[2] == b"255"
    body = np.frombuffer(parts[3], dtype=np.uint8)
    assert body.size == w * h * 3, (body.size, w, h)
    return w, h, body.reshape(h, w, 3)


def cube_edges(nitems: int = 2, color=(255, 255, 255), width: float = 2.0) -> List[Line]:
    """The 12 edges of the unit cube as line objects."""
    out = []
    for a in range(3):
        b, c = [d for d in range(3) if d != a]
        for u in (0.0, 1.0):
            for v in (0.0, 1.0):
                s = [0.0, 0.0, 0.0]
                s[b], s[c] = u, v
                e = list(s)
                e[a] = 1.0
                out.append(Line(tuple(s), tuple(e), nitems, color, width))
    return out
