"""Seeded synthetic fields (host generator; see csrc/fieldgen.h).

The same seed yields the same bytes on every host and on the device
generator, so workloads are regenerated rather than shipped.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIELDGEN_SO = os.path.join(HERE, "_build", "libc3d_fieldgen.so")
_lib = None


def build_fieldgen() -> str:
    os.makedirs(os.path.dirname(FIELDGEN_SO), exist_ok=True)
    src = os.path.join(HERE, "csrc", "fieldgen_cpu.c")
    subprocess.run(["gcc", "-std=c99", "-O2", "-ffp-contract=off", "-fPIC", "-Wall", "-shared",
                    "-o", FIELDGEN_SO, src, "-lm"], check=True)
    return FIELDGEN_SO


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(FIELDGEN_SO):
            build_fieldgen()
        L = C.CDLL(FIELDGEN_SO)
        L.c3d_fieldgen_blobs_f64.restype = None
        L.c3d_fieldgen_modes_f64.restype = C.c_double
        L.c3d_fieldgen_modes_f32.restype = C.c_double
        _lib = L
    return _lib


def _block(shape, offset, glshape):
    nz, ny, nx = shape
    gl = glshape if glshape is not None else shape
    off = offset if offset is not None else (0, 0, 0)
    return ((C.c_long * 3)(gl[2], gl[1], gl[0]), (C.c_long * 3)(off[2], off[1], off[0]),
            (C.c_long * 3)(nx, ny, nz))


def blobs(shape, nblobs=8, seed=0, offset=None, glshape=None) -> np.ndarray:
    """Sum of Gaussian blobs on the unit cube; shape = (nz, ny, nx), float64."""
    L = _load()
    out = np.empty(shape, dtype=np.float64)
    gl, off, my = _block(shape, offset, glshape)
    L.c3d_fieldgen_blobs_f64(out.ctypes.data_as(C.c_void_p), gl, off, my, C.c_int(nblobs),
                             C.c_uint64(seed))
    return out


def modes(shape, nmodes=64, kmin=1, kmax=16, power=5.0 / 6.0, seed=0, dtype=np.float64,
          offset=None, glshape=None):
    """Sum of Fourier modes; returns (field, analytic std)."""
    L = _load()
    out = np.empty(shape, dtype=dtype)
    gl, off, my = _block(shape, offset, glshape)
    fn = L.c3d_fieldgen_modes_f64 if dtype == np.float64 else L.c3d_fieldgen_modes_f32
    std = fn(out.ctypes.data_as(C.c_void_p), gl, off, my, C.c_int(nmodes), C.c_int(kmin),
             C.c_int(kmax), C.c_double(power), C.c_uint64(seed))
    return out, float(std)


def _zsplit(nz, parts):
    parts = max(1, min(parts, nz))
    step = (nz + parts - 1) // parts
    return [(z, min(z + step, nz)) for z in range(0, nz, step)]


def modes_threaded(shape, nmodes=64, kmin=1, kmax=16, power=5.0 / 6.0, seed=0, dtype=np.float64,
                   threads=None, offset=None, glshape=None):
    """modes() computed in z-slabs on `threads` host threads (default: every
    core); the bytes are the same as modes() gives, since every value depends
    on its global node index only."""
    from concurrent.futures import ThreadPoolExecutor
    L = _load()
    nz, ny, nx = shape
    o = offset if offset is not None else (0, 0, 0)
    gshape = glshape if glshape is not None else shape
    out = np.empty(shape, dtype=dtype)
    fn = L.c3d_fieldgen_modes_f64 if dtype == np.float64 else L.c3d_fieldgen_modes_f32
    stds = []

    def part(zr):
        z0, z1 = zr
        gl, off, my = _block((z1 - z0, ny, nx), (o[0] + z0, o[1], o[2]), gshape)
        view = out[z0:z1]
        stds.append(fn(view.ctypes.data_as(C.c_void_p), gl, off, my, C.c_int(nmodes), C.c_int(kmin),
                       C.c_int(kmax), C.c_double(power), C.c_uint64(seed)))

    with ThreadPoolExecutor(max_workers=threads or os.cpu_count() or 1) as ex:
        list(ex.map(part, _zsplit(nz, threads or os.cpu_count() or 1)))
    return out, float(stds[0])


def blobs_threaded(shape, nblobs=8, seed=0, threads=None) -> np.ndarray:
    """blobs() computed in z-slabs on `threads` host threads (same bytes)."""
    from concurrent.futures import ThreadPoolExecutor
    L = _load()
    nz, ny, nx = shape
    out = np.empty(shape, dtype=np.float64)

    def part(zr):
        z0, z1 = zr
        gl, off, my = _block((z1 - z0, ny, nx), (z0, 0, 0), shape)
        L.c3d_fieldgen_blobs_f64(out[z0:z1].ctypes.data_as(C.c_void_p), gl, off, my, C.c_int(nblobs),
                                 C.c_uint64(seed))

    with ThreadPoolExecutor(max_workers=threads or os.cpu_count() or 1) as ex:
        list(ex.map(part, _zsplit(nz, threads or os.cpu_count() or 1)))
    return out


def modes_std(nmodes=64, kmin=1, kmax=16, power=5.0 / 6.0, seed=0) -> float:
    L = _load()
    z = (C.c_long * 3)(2, 2, 2)
    return float(L.c3d_fieldgen_modes_f64(None, z, (C.c_long * 3)(0, 0, 0), z, C.c_int(nmodes),
                                          C.c_int(kmin), C.c_int(kmax), C.c_double(power),
                                          C.c_uint64(seed)))
