"""Multi-rank host path on CPU: gloo process groups of 2, 3, 4 and 6 ranks
(powers of two and not, one- and two-dimensional process grids) drive the
library's point-to-point transport (the stand-in for MPI_Sendrecv).

  * contour3d_gb300_extend: each rank's pencil block widened by two layers
    towards its neighbours and clipped at the global boundary
    (src/contour3d/contour/extend.c:150-282) must equal that window of the
    global field;
  * contour3d_gb300_reduce_nearest: the per-pixel nearest-depth reduction to
    rank 0 (src/contour3d/output.c:10-30, 82) must keep, per pixel, the
    larger depth, the lowest rank winning ties.

No GPU is involved: both functions are host code."""
import ctypes as C
import datetime
import os
import socket

import numpy as np
import pytest

SENDRECV = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_size_t, C.c_int, C.c_void_p, C.c_size_t, C.c_int)
PROC_NULL = -2
GLOBAL = (11, 13, 17)  # nx, ny, nz
NPIX = 997


class Transport(C.Structure):
    _fields_ = [("size", C.c_int), ("rank", C.c_int), ("sendrecv", SENDRECV), ("user", C.c_void_p)]


def _global_field():
    nx, ny, nz = GLOBAL
    return np.random.default_rng(5).standard_normal((nz, ny, nx))


def _pixels(rank):
    rng = np.random.default_rng(100 + rank)
    depth = np.round(rng.uniform(0.0, 4.0, NPIX) * 2.0) / 2.0  # coarse values: many ties across ranks
    depth[::7] = -np.finfo(np.float64).max                       # background
    rgb = rng.integers(0, 256, size=(NPIX, 3), dtype=np.uint8)
    return depth, rgb


def _worker(rank, world, port, periodic=False):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=60))
    from contour3d_gb300 import _abi, lib
    L = lib.Library()

    def sendrecv(user, sbuf, sbytes, dest, rbuf, rbytes, src):
        try:
            req = None
            if dest != PROC_NULL:
                out = torch.frombuffer(bytearray(C.string_at(sbuf, sbytes)), dtype=torch.uint8)
                req = dist.isend(out, dst=dest)
            if src != PROC_NULL:
                got = torch.empty(rbytes, dtype=torch.uint8)
                dist.recv(got, src=src)
                C.memmove(rbuf, got.data_ptr(), rbytes)
            if req is not None:
                req.wait()
            return 0
        except Exception:  # reported to the library as a failed exchange
            return 1

    cb = SENDRECV(sendrecv)
    t = Transport(world, rank, cb, None)
    assert L.lib.contour3d_gb300_install_transport(C.byref(t)) == 0
    try:
        sd = lib.sdecomp_table(L)
        world_comm = C.CFUNCTYPE(C.c_void_p)(C.cast(L.lib.c3d_comm_world, C.c_void_p).value)()
        construct = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(C.c_bool),
                                C.POINTER(C.c_void_p))(sd.construct)
        info = C.c_void_p()
        assert construct(world_comm, 3, (C.c_size_t * 3)(0, 0, 0), (C.c_bool * 3)(periodic, periodic, periodic),
                         C.byref(info)) == 0
        mysize = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_size_t, C.POINTER(C.c_size_t))(
            sd.get_pencil_mysize)
        offset = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_size_t, C.POINTER(C.c_size_t))(
            sd.get_pencil_offset)
        size, off = [], []
        for d, g in enumerate(GLOBAL):
            m, o = C.c_size_t(), C.c_size_t()
            assert mysize(info, 0, d, g, C.byref(m)) == 0 and offset(info, 0, d, g, C.byref(o)) == 0
            size.append(m.value)
            off.append(o.value)
        G = _global_field()
        local = np.ascontiguousarray(G[off[2]:off[2] + size[2], off[1]:off[1] + size[1], off[0]:off[0] + size[0]])
        grids = [np.linspace(0.0, 1.0, g)[o:o + s].copy() for g, o, s in zip(GLOBAL, off, size)]
        obj = _abi.ContourObj()
        obj.pencil = 0
        obj.glsizes = (C.c_size_t * 3)(*GLOBAL)
        for d in range(3):
            obj.grids[d] = grids[d].ctypes.data_as(C.POINTER(C.c_double))
        obj.converter = None
        obj.threshold = 0.0
        obj.array = local.ctypes.data_as(C.POINTER(C.c_double))
        esz, eof = (C.c_size_t * 3)(), (C.c_size_t * 3)()
        ext_fn = L.lib.contour3d_gb300_extend
        ext_fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        assert ext_fn(info, C.byref(obj), esz, eof, None) == 0
        for d in range(3):
            lo = max(off[d] - 2, 0)
            hi = min(off[d] + size[d] + 2, GLOBAL[d])
            assert (eof[d], esz[d]) == (lo, hi - lo), (rank, d, off, size, list(eof), list(esz))
        ext = np.empty(esz[2] * esz[1] * esz[0])
        assert ext_fn(info, C.byref(obj), esz, eof, ext.ctypes.data) == 0
        want = G[eof[2]:eof[2] + esz[2], eof[1]:eof[1] + esz[1], eof[0]:eof[0] + esz[0]]
        assert np.array_equal(ext.reshape(esz[2], esz[1], esz[0]), want), f"rank {rank}: extension differs"

        depth, rgb = _pixels(rank)
        red = L.lib.contour3d_gb300_reduce_nearest
        red.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t]
        assert red(info, depth.ctypes.data, rgb.ctypes.data, NPIX) == 0
        if rank == 0:
            all_d = np.stack([_pixels(r)[0] for r in range(world)])
            all_c = np.stack([_pixels(r)[1] for r in range(world)])
            win = np.argmax(all_d, axis=0)  # first maximum: the lowest rank wins ties
            assert np.array_equal(depth, all_d[win, np.arange(NPIX)])
            assert np.array_equal(rgb, all_c[win, np.arange(NPIX)])
        C.CFUNCTYPE(C.c_int, C.c_void_p)(sd.destruct)(info)
    finally:
        L.lib.contour3d_gb300_install_transport(None)
        dist.barrier()
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world", [2, 3, 4, 6])
def test_extend_and_reduce_over_gloo(built, world):
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(world, _free_port()), nprocs=world, join=True)


@pytest.mark.parametrize("world", [2, 4])
def test_extend_periodic_grid(built, world):
    """A periodic process grid: the halos are exchanged with the wrapped
    neighbours too, and the global-boundary layers are clipped by rank
    position as in extend.c:223-252, so every rank's extended block is still
    the clipped window of the global field."""
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(world, _free_port(), True), nprocs=world, join=True)


def _failing_exchange_script(root):
    return f"""
import ctypes as C, sys
import numpy as np
sys.path.insert(0, {root!r})
from tests.test_multirank_cpu import SENDRECV, Transport, GLOBAL
from contour3d_gb300 import _abi, lib
L = lib.Library()
calls = []
def sendrecv(user, sbuf, sbytes, dest, rbuf, rbytes, src):
    calls.append((dest, src))
    return 1  # the exchange failed (a peer that left, a dropped message)
cb = SENDRECV(sendrecv)
t = Transport(2, 0, cb, None)
assert L.lib.contour3d_gb300_install_transport(C.byref(t)) == 0
sd = lib.sdecomp_table(L)
world = C.CFUNCTYPE(C.c_void_p)(C.cast(L.lib.c3d_comm_world, C.c_void_p).value)()
construct = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(C.c_bool),
                        C.POINTER(C.c_void_p))(sd.construct)
info = C.c_void_p()
assert construct(world, 3, (C.c_size_t * 3)(0, 0, 0), (C.c_bool * 3)(False, False, False), C.byref(info)) == 0
mysize = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_size_t, C.POINTER(C.c_size_t))(sd.get_pencil_mysize)
size = []
for d, g in enumerate(GLOBAL):
    m = C.c_size_t()
    assert mysize(info, 0, d, g, C.byref(m)) == 0
    size.append(m.value)
local = np.zeros((size[2], size[1], size[0]))
grids = [np.linspace(0.0, 1.0, g)[:s].copy() for g, s in zip(GLOBAL, size)]
obj = _abi.ContourObj()
obj.pencil = 0
obj.glsizes = (C.c_size_t * 3)(*GLOBAL)
for d in range(3):
    obj.grids[d] = grids[d].ctypes.data_as(C.POINTER(C.c_double))
obj.converter = None
obj.threshold = 0.0
obj.array = local.ctypes.data_as(C.POINTER(C.c_double))
esz, eof = (C.c_size_t * 3)(), (C.c_size_t * 3)()
ext_fn = L.lib.contour3d_gb300_extend
ext_fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
assert ext_fn(info, C.byref(obj), esz, eof, None) == 0  # sizes only: no exchange
ext = np.empty(esz[2] * esz[1] * esz[0])
print("extend", ext_fn(info, C.byref(obj), esz, eof, ext.ctypes.data))
depth = np.zeros(16)
rgb = np.zeros((16, 3), dtype=np.uint8)
red = L.lib.contour3d_gb300_reduce_nearest
red.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t]
print("reduce", red(info, depth.ctypes.data, rgb.ctypes.data, 16))
print("calls", len(calls))
L.lib.contour3d_gb300_install_transport(None)
"""


def test_failed_exchange_is_reported(built):
    """Failure on the host: a transport whose exchange reports an error (a
    rank that left, a dropped message) makes the halo extension and the
    depth reduction return 1 with a [CONTOUR3D ERROR] line; nothing waits."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _failing_exchange_script(root)], capture_output=True, text=True,
                       timeout=120, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "extend 1" in r.stdout and "reduce 1" in r.stdout, r.stdout
    assert "calls 0" not in r.stdout
    assert "[CONTOUR3D ERROR]" in r.stderr
