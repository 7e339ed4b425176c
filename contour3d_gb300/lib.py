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
                ("ms_shade", C.c_double), ("filter_violations", C.c_uint64 * 5),
                ("cover_triangles", C.c_uint64), ("exact_fragments", C.c_uint64), ("slivers", C.c_uint64),
                ("vertices", C.c_uint64), ("ms_vertices", C.c_double), ("ms_normals", C.c_double),
                ("shade_exact", C.c_uint64), ("shade_violations", C.c_uint64), ("unsynchronised", C.c_uint64),
                ("redone", C.c_uint64), ("graph", C.c_uint64)]


class Field(C.Structure):
    """contour3d_gb300_field_t: a field resident in device memory."""
    _fields_ = [("device_array", C.c_void_p), ("dtype", C.c_int), ("sizes", C.c_size_t * 3),
                ("grids", C.POINTER(C.c_double) * 3), ("converter", C.c_void_p),
                ("threshold", C.c_double), ("color", _abi.Color)]


F64, F32 = 0, 1


class Frame(C.Structure):
    """contour3d_gb300_frame_t."""
    _fields_ = [("camera_position", _abi.Vector), ("light_direction", _abi.Vector),
                ("screen_sizes", C.c_size_t * 2), ("screen_center", _abi.Vector),
                ("screen_local", _abi.Vector * 2), ("bg_color", _abi.Color), ("num_fields", C.c_size_t),
                ("fields", C.POINTER(Field)), ("num_lines", C.c_size_t), ("lines", C.POINTER(_abi.LineObj)),
                ("rgb_out", C.c_void_p)]


class RequestStats(C.Structure):
    _fields_ = [("latency_ms", C.c_double), ("queue_ms", C.c_double), ("device_ms", C.c_double),
                ("estimate_bytes", C.c_uint64), ("held_bytes", C.c_uint64)]


class ServerMemory(C.Structure):
    _fields_ = [("used_bytes", C.c_uint64), ("peak_bytes", C.c_uint64), ("overcommits", C.c_uint64),
                ("trims", C.c_uint64)]


class FramePack:
    """A frame of device-resident fields plus everything its pointers refer to."""

    def __init__(self, lib: "Library", scene: _abi.Scene, fields, rgb_dev_ptr: int):
        self._keep = []
        self.fields = (Field * max(len(fields), 1))()
        for n, (ptr, dt, sizes, grids, thr, color) in enumerate(fields):
            f = self.fields[n]
            f.device_array = ptr
            f.dtype = dt
            for d in range(3):
                f.sizes[d] = sizes[d]
                g = np.ascontiguousarray(grids[d], dtype=np.float64)
                self._keep.append(g)
                f.grids[d] = g.ctypes.data_as(C.POINTER(C.c_double))
            f.converter = lib.converters["identity"]
            f.threshold = float(thr)
            f.color = _abi.col(color)
        a = _abi.ExecuteArgs(scene, lib.converters)
        self._keep.append(a)
        fr = Frame()
        fr.camera_position = a.camera
        fr.light_direction = a.light
        fr.screen_sizes[0], fr.screen_sizes[1] = scene.width, scene.height
        fr.screen_center = a.center
        fr.screen_local[0], fr.screen_local[1] = a.local[0], a.local[1]
        fr.bg_color = a.bg
        fr.num_fields = len(fields)
        fr.fields = C.cast(self.fields, C.POINTER(Field))
        fr.num_lines = a.num_lines
        fr.lines = C.cast(a.lines, C.POINTER(_abi.LineObj))
        fr.rgb_out = rgb_dev_ptr
        self.frame = fr

# every symbol declared in include/contour3d.h and include/contour3d_gb300.h
class SdecompTable(C.Structure):
    """The `sdecomp` function table of include/sdecomp.h (function pointers)."""
    _fields_ = [(n, C.c_void_p) for n in ("construct", "destruct", "get_comm_cart", "get_comm_rank",
                                         "get_nprocs", "get_myrank", "get_neighbours",
                                         "get_pencil_mysize", "get_pencil_offset")]


def sdecomp_table(L: "Library") -> SdecompTable:
    return SdecompTable.in_dll(L.lib, "sdecomp")


EXPORTS = [
    "contour3d_execute", "contour3d_gb300_identity", "contour3d_gb300_declare_identity",
    "contour3d_gb300_render", "contour3d_gb300_render_device", "contour3d_gb300_last_stats",
    "contour3d_gb300_set_stage_timing", "contour3d_gb300_set_slab_cells", "contour3d_gb300_set_filter_check",
    "contour3d_gb300_set_async", "contour3d_gb300_set_server_async", "contour3d_gb300_set_graphs", "contour3d_gb300_set_launch_shape",
    "contour3d_gb300_set_dependent_launch", "contour3d_gb300_set_batch_classify",
    "contour3d_gb300_set_upload_model",
    "contour3d_gb300_debug_triangles", "contour3d_gb300_debug_cell_counts",
    "contour3d_gb300_install_transport", "contour3d_gb300_extend", "contour3d_gb300_release",
    "contour3d_gb300_cell_offsets_noalloc", "contour3d_gb300_render_batch", "contour3d_gb300_server_create",
    "contour3d_gb300_server_submit", "contour3d_gb300_server_wait", "contour3d_gb300_server_destroy",
    "contour3d_gb300_server_memory",
    "contour3d_gb300_device_bytes", "contour3d_gb300_reduce_nearest",
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
                                                C.c_int, C.c_int, C.c_int, C.c_double, C.c_uint64, C.c_double]
        L.c3d_fieldgen_blobs_device.restype = C.c_int
        L.c3d_fieldgen_modes_device_async.restype = C.c_double
        L.c3d_fieldgen_modes_device_async.argtypes = [
            C.c_void_p, C.c_int, C.c_long * 3, C.c_long * 3, C.c_long * 3, C.c_int, C.c_int, C.c_int, C.c_double,
            C.c_uint64, C.c_double, C.c_void_p]
        L.contour3d_gb300_render_device.argtypes = [
            C.POINTER(_abi.Vector), C.POINTER(_abi.Vector), C.POINTER(C.c_size_t), C.POINTER(_abi.Vector),
            C.POINTER(_abi.Vector), C.POINTER(_abi.Color), C.c_size_t, C.POINTER(Field), C.c_size_t,
            C.POINTER(_abi.LineObj), C.c_void_p, C.c_void_p]
        L.contour3d_gb300_render.argtypes = [
            C.POINTER(_abi.Vector), C.POINTER(_abi.Vector), C.POINTER(C.c_size_t), C.POINTER(_abi.Vector),
            C.POINTER(_abi.Vector), C.POINTER(_abi.Color), C.c_size_t, C.POINTER(_abi.ContourObj), C.c_size_t,
            C.POINTER(_abi.LineObj), C.c_void_p, C.c_void_p]
        L.contour3d_gb300_render_batch.restype = C.c_int
        L.contour3d_gb300_render_batch.argtypes = [C.POINTER(Frame), C.c_size_t, C.c_int, C.c_void_p]
        L.contour3d_gb300_server_create.restype = C.c_void_p
        L.contour3d_gb300_server_create.argtypes = [C.c_int, C.c_uint64, C.c_uint64]
        L.contour3d_gb300_server_submit.restype = C.c_int
        L.contour3d_gb300_server_submit.argtypes = [C.c_void_p, C.POINTER(Frame), C.POINTER(C.c_uint64)]
        L.contour3d_gb300_server_wait.restype = C.c_int
        L.contour3d_gb300_server_wait.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(RequestStats)]
        L.contour3d_gb300_server_memory.restype = C.c_int
        L.contour3d_gb300_server_memory.argtypes = [C.c_void_p, C.POINTER(ServerMemory)]
        L.contour3d_gb300_server_destroy.restype = C.c_int
        L.contour3d_gb300_server_destroy.argtypes = [C.c_void_p]
        L.contour3d_gb300_device_bytes.restype = C.c_uint64
        L.contour3d_gb300_cell_offsets_noalloc.restype = C.c_int
        L.contour3d_gb300_cell_offsets_noalloc.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_size_t), C.c_double,
                                                           C.c_void_p, C.c_void_p, C.c_void_p]
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

    def render_pack(self, pack: "FramePack", stream: int = 0) -> int:
        """One FramePack through contour3d_gb300_render_device."""
        fr = pack.frame
        return self.lib.contour3d_gb300_render_device(
            C.byref(fr.camera_position), C.byref(fr.light_direction), fr.screen_sizes, C.byref(fr.screen_center),
            fr.screen_local, C.byref(fr.bg_color), C.c_size_t(fr.num_fields), fr.fields,
            C.c_size_t(fr.num_lines), fr.lines, C.c_void_p(fr.rgb_out), C.c_void_p(stream))

    def frame(self, scene: _abi.Scene, fields, rgb_dev_ptr: int) -> FramePack:
        return FramePack(self, scene, fields, rgb_dev_ptr)

    def render_batch(self, packs, workers: int = 4):
        """Render FramePacks concurrently; returns per-frame device milliseconds."""
        n = len(packs)
        arr = (Frame * max(n, 1))(*[p.frame for p in packs])
        ms = np.zeros(max(n, 1), dtype=np.float64)
        rc = self.lib.contour3d_gb300_render_batch(arr, n, workers, ms.ctypes.data_as(C.c_void_p))
        if rc != 0:
            raise RuntimeError("contour3d_gb300_render_batch failed")
        return ms[:n]

    def server(self, slots: int, budget_bytes: int = 0, resident_bytes: int = 0) -> "Server":
        return Server(self, slots, budget_bytes, resident_bytes)

    def stats(self) -> Stats:
        s = Stats()
        self.lib.contour3d_gb300_last_stats(C.byref(s))
        return s

    def set_stage_timing(self, on: bool) -> None:
        self.lib.contour3d_gb300_set_stage_timing(1 if on else 0)

    def set_filter_check(self, on: bool) -> None:
        self.lib.contour3d_gb300_set_filter_check(1 if on else 0)

    def set_async(self, on: bool) -> None:
        self.lib.contour3d_gb300_set_async(1 if on else 0)

    def set_graphs(self, on: bool) -> None:
        self.lib.contour3d_gb300_set_graphs(1 if on else 0)

    def set_dependent_launch(self, on: bool) -> None:
        self.lib.contour3d_gb300_set_dependent_launch(1 if on else 0)

    def set_batch_classify(self, on: bool) -> None:
        self.lib.contour3d_gb300_set_batch_classify(1 if on else 0)

    def set_upload_model(self, link_gb_per_s: float, slab_ps_per_cell: float, slab_fixed_us: float) -> int:
        f = self.lib.contour3d_gb300_set_upload_model
        f.argtypes = [C.c_double, C.c_double, C.c_double]
        return f(link_gb_per_s, slab_ps_per_cell, slab_fixed_us)

    def set_launch_shape(self, classify_slices: int, emit_blocks_per_sm: int, raster_blocks_per_sm: int) -> None:
        if self.lib.contour3d_gb300_set_launch_shape(int(classify_slices), int(emit_blocks_per_sm),
                                                     int(raster_blocks_per_sm)) != 0:
            raise ValueError("launch shape out of range")

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
                              offset=(0, 0, 0), glshape=None, time: float = 0.0) -> float:
        nz, ny, nx = shape
        gl = glshape or shape
        std = self.lib.c3d_fieldgen_modes_device(
            C.c_void_p(ptr), dtype, (C.c_long * 3)(gl[2], gl[1], gl[0]),
            (C.c_long * 3)(offset[2], offset[1], offset[0]), (C.c_long * 3)(nx, ny, nz), nmodes, kmin,
            kmax, power, seed, time)
        if std < 0:
            raise RuntimeError("device field generation failed")
        return std

    def fieldgen_modes_device_async(self, ptr: int, dtype: int, shape, nmodes, kmin, kmax, power, seed,
                                    time: float, stream: int) -> float:
        nz, ny, nx = shape
        z = (C.c_long * 3)(0, 0, 0)
        std = self.lib.c3d_fieldgen_modes_device_async(
            C.c_void_p(ptr), dtype, (C.c_long * 3)(nx, ny, nz), z, (C.c_long * 3)(nx, ny, nz), nmodes, kmin, kmax,
            power, seed, time, C.c_void_p(stream))
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


class Server:
    """Python face of the served form (contour3d_gb300_server_*)."""

    def __init__(self, lib: Library, slots: int, budget_bytes: int = 0, resident_bytes: int = 0):
        self.lib = lib
        self.h = lib.lib.contour3d_gb300_server_create(slots, budget_bytes, resident_bytes)
        if not self.h:
            raise RuntimeError("contour3d_gb300_server_create failed")
        self._packs = {}

    def submit(self, pack: FramePack) -> int:
        t = C.c_uint64(0)
        if self.lib.lib.contour3d_gb300_server_submit(self.h, C.byref(pack.frame), C.byref(t)) != 0:
            raise RuntimeError("submit failed")
        self._packs[t.value] = pack
        return t.value

    def wait(self, ticket: int) -> RequestStats:
        st = RequestStats()
        rc = self.lib.lib.contour3d_gb300_server_wait(self.h, ticket, C.byref(st))
        self._packs.pop(ticket, None)
        if rc != 0:
            raise RuntimeError(f"request {ticket} failed")
        return st

    def memory(self) -> ServerMemory:
        m = ServerMemory()
        if self.lib.lib.contour3d_gb300_server_memory(self.h, C.byref(m)) != 0:
            raise RuntimeError("contour3d_gb300_server_memory failed")
        return m

    def close(self) -> None:
        if self.h:
            self.lib.lib.contour3d_gb300_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


_singleton: Optional[Library] = None


def load() -> Library:
    global _singleton
    if _singleton is None:
        _singleton = Library()
    return _singleton
