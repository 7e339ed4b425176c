"""ctypes access to the CPU checkers.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  `Oracle` is the C restatement (oracle/c3d_oracle.c, built into
oracle/_build/); `Reference` is the reference library compiled from its own
sources with single-rank shims (oracle/_ref/, built only where the reference
tree exists).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional, Tuple

import numpy as np

from contour3d_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libc3d_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libc3dref.so")
# the reference checkout: $C3D_REFERENCE_TREE, else a directory named
# `reference` beside this repository (absent on GPU hosts: the checker is then
# not built and the tests that need it skip)
REF_TREE = os.environ.get("C3D_REFERENCE_TREE") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")

from contour3d_gb300.records import TRI_DTYPE  # noqa: E402


def build(with_reference: Optional[bool] = None) -> None:
    """Compile the restatement (always) and the reference checker (when its tree exists)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    if with_reference is None:
        with_reference = os.path.isdir(os.path.join(REF_TREE, "src", "contour3d"))
    if with_reference:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_TREE}"], check=True)


class Oracle:
    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build(with_reference=False)
        self.lib = C.CDLL(path)
        L = self.lib
        L.c3d_oracle_render.restype = C.c_int
        L.c3d_oracle_triangles.restype = C.c_long
        L.c3d_oracle_triangles.argtypes = [C.POINTER(_abi.ContourObj), C.c_void_p, C.c_long,
                                           C.POINTER(C.c_long)]
        L.c3d_oracle_cell_counts.restype = C.c_long
        L.c3d_oracle_cell_counts.argtypes = [C.c_void_p, C.POINTER(C.c_size_t), C.c_double,
                                             C.c_void_p]
        _abi.declare_execute(L.c3d_oracle_execute)
        self.converters = {
            "identity": C.cast(L.c3d_oracle_identity, C.c_void_p).value,
            "warp": C.cast(L.c3d_oracle_warp, C.c_void_p).value,
        }

    def render(self, scene: _abi.Scene, nranks: int = 1, with_depth: bool = False):
        """RGB image in ppm row order (H, W, 3) and optionally the depth buffer."""
        a = _abi.ExecuteArgs(scene, self.converters)
        rgb = np.zeros((scene.height, scene.width, 3), dtype=np.uint8)
        depth = np.zeros((scene.height, scene.width), dtype=np.float64) if with_depth else None
        rc = self.lib.c3d_oracle_render(
            C.byref(a.camera), C.byref(a.light), a.sizes, C.byref(a.center), a.local,
            C.byref(a.bg), C.c_size_t(a.num_contours), a.contours, C.c_size_t(a.num_lines),
            a.lines, C.c_int(nranks), rgb.ctypes.data_as(C.c_void_p),
            depth.ctypes.data_as(C.c_void_p) if depth is not None else None)
        if rc != 0:
            raise RuntimeError("oracle render failed")
        return (rgb, depth) if with_depth else rgb

    def execute(self, scene: _abi.Scene, fname: str) -> int:
        a = _abi.ExecuteArgs(scene, self.converters, fname)
        return self.lib.c3d_oracle_execute(*a.execute_tuple())

    def triangles(self, contour: _abi.Contour) -> Tuple[np.ndarray, int]:
        """Rendered triangles in render order, and the triangulated-set count."""
        sc = _abi.Scene((0, 0, 0), (0, 0, 0), (0, 0, 1), 1, 1, (0, 0, 0), (1, 0, 0), (0, 1, 0),
                        contours=[contour])
        a = _abi.ExecuteArgs(sc, self.converters)
        total = C.c_long(0)
        n = self.lib.c3d_oracle_triangles(a.contours, None, 0, C.byref(total))
        out = np.zeros(max(n, 1), dtype=TRI_DTYPE)
        n2 = self.lib.c3d_oracle_triangles(a.contours, out.ctypes.data_as(C.c_void_p), n,
                                           C.byref(total))
        assert n2 == n
        return out[:n], int(total.value)

    def cell_counts(self, field: np.ndarray, threshold: float) -> Tuple[np.ndarray, int]:
        f = np.ascontiguousarray(field, dtype=np.float64)
        nz, ny, nx = f.shape
        sizes = (C.c_size_t * 3)(nx, ny, nz)
        counts = np.zeros((nz - 1, ny - 1, nx - 1), dtype=np.uint8)
        total = self.lib.c3d_oracle_cell_counts(f.ctypes.data_as(C.c_void_p), sizes,
                                                C.c_double(threshold),
                                                counts.ctypes.data_as(C.c_void_p))
        return counts, int(total)


class Reference:
    """The reference library itself (single rank), compiled from its sources."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        L = self.lib
        _abi.declare_execute(L.contour3d_execute)
        L.c3dref_single_rank.restype = C.c_void_p
        L.c3dref_dump_triangles.restype = C.c_long
        L.c3dref_dump_triangles.argtypes = [C.c_void_p, C.POINTER(_abi.ContourObj), C.c_void_p,
                                            C.c_long, C.POINTER(C.c_long)]
        self.info = L.c3dref_single_rank()
        self.converters = {
            "identity": C.cast(L.c3dref_identity, C.c_void_p).value,
            "warp": C.cast(L.c3dref_warp, C.c_void_p).value,
        }

    def execute(self, scene: _abi.Scene, fname: str) -> int:
        a = _abi.ExecuteArgs(scene, self.converters, fname, sdecomp_info=self.info)
        return self.lib.contour3d_execute(*a.execute_tuple())

    def render(self, scene: _abi.Scene, tmpdir: str) -> np.ndarray:
        path = os.path.join(tmpdir, "ref.ppm")
        rc = self.execute(scene, path)
        if rc != 0:
            raise RuntimeError("reference execute failed")
        return _abi.read_ppm(path)[2]

    def triangles(self, contour: _abi.Contour) -> Tuple[np.ndarray, int]:
        sc = _abi.Scene((0, 0, 0), (0, 0, 0), (0, 0, 1), 1, 1, (0, 0, 0), (1, 0, 0), (0, 1, 0),
                        contours=[contour])
        a = _abi.ExecuteArgs(sc, self.converters)
        total = C.c_long(0)
        n = self.lib.c3dref_dump_triangles(self.info, a.contours, None, 0, C.byref(total))
        out = np.zeros(max(n, 1), dtype=TRI_DTYPE)
        n2 = self.lib.c3dref_dump_triangles(self.info, a.contours, out.ctypes.data_as(C.c_void_p),
                                            n, C.byref(total))
        assert n2 == n
        return out[:n], int(total.value)


def reference_available() -> bool:
    return os.path.exists(REF_SO)
