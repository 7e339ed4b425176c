"""ctypes bindings of the native library (see include/contour3d.h and
include/contour3d_gb300.h for the C declarations)."""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Tuple

import numpy as np

from . import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcontour3d_gb300.so")
FIELDGEN_PATH = os.path.join(HERE, "_build", "libc3d_fieldgen.so")


class NativeLibraryMissing(RuntimeError):
    pass


class Stats(C.Structure):
    _fields_ = [("cells", C.c_uint64), ("triangles", C.c_uint64), ("candidates", C.c_uint64),
                ("candidate_overflows", C.c_uint64), ("tiny", C.c_uint64), ("winners", C.c_uint64),
                ("normals", C.c_uint64), ("slabs", C.c_uint64), ("kernel_launches", C.c_uint64),
                ("ms_total", C.c_double), ("ms_classify", C.c_double), ("ms_scan", C.c_double),
                ("ms_emit", C.c_double), ("ms_cover", C.c_double), ("ms_exact", C.c_double),
                ("ms_shade", C.c_double), ("filter_violations", C.c_uint64 * 5)]


class Field(C.Structure):
    """contour3d_gb300_field_t: a field resident in device memory."""
    _fields_ = [("device_array", C.c_void_p), ("dtype", C.c_int), ("sizes", C.c_size_t * 3),
                ("grids", C.POINTER(C.c_double) * 3), ("converter", C.c_void_p),
                ("threshold", C.c_double), ("color", _abi.Color)]


F64, F32 = 0, 1

# every symbol declared in include/contour3d.h and include/contour3d_gb300.h
EXPORTS = [
    "contour3d_execute", "contour3d_gb300_identity", "contour3d_gb300_declare_identity",
    "contour3d_gb300_render", "contour3d_gb300_render_device", "contour3d_gb300_last_stats",
    "contour3d_gb300_set_stage_timing", "contour3d_gb300_set_slab_cells", "contour3d_gb300_set_filter_check",
    "contour3d_gb300_debug_triangles", "contour3d_gb300_debug_cell_counts",
    "contour3d_gb300_install_transport", "contour3d_gb300_extend", "contour3d_gb300_release",
    "contour3d_gb300_cell_offsets_noalloc",
    "c3d_comm_world", "sdecomp",
]


class Library:
    def __init__(self, path: str = LIB_PATH):
        if not os.path.exists(path):
            raise NativeLibraryMissing(
                f"{path} is not built; run `python -m contour3d_gb300.build` (there is no CPU fallback)")
        self.path = path
        self.lib = C.CDLL(path)
        L = self.lib
        _abi.declare_execute(L.contour3d_execute)
        L.contour3d_gb300_render.restype = C.c_int
        L.contour3d_gb300_render_device.restype = C.c_int
        L.contour3d_gb300_last_stats.restype = C.c_int
        L.contour3d_gb300_last_stats.argtypes = [C.POINTER(Stats)]
        L.contour3d_gb300_set_stage_timing.argtypes = [C.c_int]
        L.contour3d_gb300_set_slab_cells.argtypes = [C.c_uint64]
        L.contour3d_gb300_debug_triangles.restype = C.c_long
        L.contour3d_gb300_debug_triangles.argtypes = [C.POINTER(_abi.ContourObj), C.c_void_p, C.c_long,
                                                      C.POINTER(C.c_long)]
        L.contour3d_gb300_debug_cell_counts.restype = C.c_long
        L.contour3d_gb300_debug_cell_counts.argtypes = [C.POINTER(_abi.ContourObj), C.c_void_p]
        L.c3d_fieldgen_modes_device.restype = C.c_double
        L.c3d_fieldgen_modes_device.argtypes = [C.c_void_p, C.c_int, C.c_long * 3, C.c_long * 3, C.c_long * 3,
                                                C.c_int, C.c_int, C.c_int, C.c_double, C.c_uint64]
        L.c3d_fieldgen_blobs_device.restype = C.c_int
        identity = C.cast(L.contour3d_gb300_identity, C.c_void_p).value
        self.converters = {"identity": identity}
        if os.path.exists(FIELDGEN_PATH):
            fg = C.CDLL(FIELDGEN_PATH)
            self.converters["warp"] = C.cast(fg.c3d_example_warp, C.c_void_p).value
            self._fieldgen = fg

    # ---- the drop-in entry point ----
    def execute(self, scene: _abi.Scene, fname: str, sdecomp_info: Optional[int] = None) -> int:
        a = _abi.ExecuteArgs(scene, self.converters, fname, sdecomp_info)
        return self.lib.contour3d_execute(*a.execute_tuple())

    # ---- extensions ----
    def render(self, scene: _abi.Scene, with_depth: bool = False):
        """ppm-ordered RGB (H, W, 3) [and canvas-ordered depth] of one process."""
        a = _abi.ExecuteArgs(scene, self.converters)
        rgb = np.zeros((scene.height, scene.width, 3), dtype=np.uint8)
        depth = np.zeros((scene.height, scene.width), dtype=np.float64) if with_depth else None
        rc = self.lib.contour3d_gb300_render(
            C.byref(a.camera), C.byref(a.light), a.sizes, C.byref(a.center), a.local, C.byref(a.bg),
            C.c_size_t(a.num_contours), a.contours, C.c_size_t(a.num_lines), a.lines,
            rgb.ctypes.data_as(C.c_void_p), depth.ctypes.data_as(C.c_void_p) if with_depth else None)
        if rc != 0:
            raise RuntimeError("contour3d_gb300_render failed")
        return (rgb, depth) if with_depth else rgb

    def render_device(self, scene: _abi.Scene, fields, rgb_dev_ptr: int, stream: int = 0) -> int:
        """Render device-resident fields: `fields` is a list of
        (device_ptr, dtype, (nx, ny, nz), grids(host arrays), threshold, color)."""
        keep = []
        arr = (Field * max(len(fields), 1))()
        for n, (ptr, dt, sizes, grids, thr, color) in enumerate(fields):
            f = arr[n]
            f.device_array = ptr
            f.dtype = dt
            for d in range(3):
                f.sizes[d] = sizes[d]
                g = np.ascontiguousarray(grids[d], dtype=np.float64)
                keep.append(g)
                f.grids[d] = g.ctypes.data_as(C.POINTER(C.c_double))
            f.converter = self.converters["identity"]
            f.threshold = float(thr)
            f.color = _abi.col(color)
        a = _abi.ExecuteArgs(scene, self.converters)
        return self.lib.contour3d_gb300_render_device(
            C.byref(a.camera), C.byref(a.light), a.sizes, C.byref(a.center), a.local, C.byref(a.bg),
            C.c_size_t(len(fields)), arr, C.c_size_t(a.num_lines), a.lines, C.c_void_p(rgb_dev_ptr),
            C.c_void_p(stream))

    def stats(self) -> Stats:
        s = Stats()
        self.lib.contour3d_gb300_last_stats(C.byref(s))
        return s

    def set_stage_timing(self, on: bool) -> None:
        self.lib.contour3d_gb300_set_stage_timing(1 if on else 0)

    def set_filter_check(self, on: bool) -> None:
        self.lib.contour3d_gb300_set_filter_check(1 if on else 0)

    def set_slab_cells(self, n: int) -> int:
        return self.lib.contour3d_gb300_set_slab_cells(C.c_uint64(n))

    def triangles(self, contour: _abi.Contour) -> Tuple[np.ndarray, int]:
        """Rendered triangles in drawing order (224-byte records) and the triangulated count."""
        from .records import TRI_DTYPE
        sc = _abi.Scene((0, 0, 0), (0, 0, 0), (0, 0, 1), 1, 1, (0, 0, 0), (1, 0, 0), (0, 1, 0),
                        contours=[contour])
        a = _abi.ExecuteArgs(sc, self.converters)
        total = C.c_long(0)
        n = self.lib.contour3d_gb300_debug_triangles(a.contours, None, 0, C.byref(total))
        if n < 0:
            raise RuntimeError("contour3d_gb300_debug_triangles failed")
        out = np.zeros(max(n, 1), dtype=TRI_DTYPE)
        n2 = self.lib.contour3d_gb300_debug_triangles(a.contours, out.ctypes.data_as(C.c_void_p), n,
                                                      C.byref(total))
        assert n2 == n
        return out[:n], int(total.value)

    def cell_counts(self, field: np.ndarray, threshold: float) -> Tuple[np.ndarray, int]:
        sc = _abi.Scene((0, 0, 0), (0, 0, 0), (0, 0, 1), 1, 1, (0, 0, 0), (1, 0, 0), (0, 1, 0),
                        contours=[_abi.Contour(field, threshold)])
        a = _abi.ExecuteArgs(sc, self.converters)
        nz, ny, nx = field.shape
        counts = np.zeros((nz - 1, ny - 1, nx - 1), dtype=np.uint8)
        total = self.lib.contour3d_gb300_debug_cell_counts(a.contours, counts.ctypes.data_as(C.c_void_p))
        if total < 0:
            raise RuntimeError("contour3d_gb300_debug_cell_counts failed")
        return counts, int(total)

    def fieldgen_modes_device(self, ptr: int, dtype: int, shape, nmodes, kmin, kmax, power, seed,
                              offset=(0, 0, 0), glshape=None) -> float:
        nz, ny, nx = shape
        gl = glshape or shape
        std = self.lib.c3d_fieldgen_modes_device(
            C.c_void_p(ptr), dtype, (C.c_long * 3)(gl[2], gl[1], gl[0]),
            (C.c_long * 3)(offset[2], offset[1], offset[0]), (C.c_long * 3)(nx, ny, nz), nmodes, kmin,
            kmax, power, seed)
        if std < 0:
            raise RuntimeError("device field generation failed")
        return std

    def fieldgen_blobs_device(self, ptr: int, shape, nblobs, seed) -> None:
        nz, ny, nx = shape
        z = (C.c_long * 3)(0, 0, 0)
        rc = self.lib.c3d_fieldgen_blobs_device(C.c_void_p(ptr), (C.c_long * 3)(nx, ny, nz), z,
                                                (C.c_long * 3)(nx, ny, nz), C.c_int(nblobs),
                                                C.c_uint64(seed))
        if rc != 0:
            raise RuntimeError("device blob generation failed")

    def release(self) -> None:
        self.lib.contour3d_gb300_release()


_singleton: Optional[Library] = None


def load() -> Library:
    global _singleton
    if _singleton is None:
        _singleton = Library()
    return _singleton
