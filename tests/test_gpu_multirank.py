"""Rank invariance of the drop-in entry point on the GPU.

A multi-rank caller gives each rank its pencil-local block of every field
and calls contour3d_execute collectively (include/contour3d.h:58-86).  Each
rank widens its block by the two-layer halo from its neighbours
(src/contour3d/contour/extend.c:10-282), renders it on the GPU, and the
per-pixel nearest-depth reduction to rank 0 (src/contour3d/output.c:10-30,
77-82) precedes the ppm write.  Rank 0's file must equal the reference's
single-rank image (golden fixtures).

The ranks are processes that share the one GPU; their exchanges go through
the library's host transport over a gloo process group, so no kernel of one
rank ever waits on another rank.
"""
import ctypes as C
import datetime
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SENDRECV = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_size_t, C.c_int, C.c_void_p, C.c_size_t, C.c_int)
PROC_NULL = -2
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = ("blobs_small", "modes_warp", "nonuniform_multi")


class Transport(C.Structure):
    _fields_ = [("size", C.c_int), ("rank", C.c_int), ("sendrecv", SENDRECV), ("user", C.c_void_p)]


def _worker(rank, world, port, pencil, outdir):
    import torch
    import torch.distributed as dist
    torch.cuda.set_device(0)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=120))
    from contour3d_gb300 import _abi, lib
    from tests import cases
    L = lib.load()

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
    sd = lib.sdecomp_table(L)
    info = C.c_void_p()
    try:
        comm = C.CFUNCTYPE(C.c_void_p)(C.cast(L.lib.c3d_comm_world, C.c_void_p).value)()
        construct = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(C.c_bool),
                                C.POINTER(C.c_void_p))(sd.construct)
        assert construct(comm, 3, (C.c_size_t * 3)(0, 0, 0), (C.c_bool * 3)(False, False, False),
                         C.byref(info)) == 0
        mysize = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_size_t, C.POINTER(C.c_size_t))(
            sd.get_pencil_mysize)
        offset = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_size_t, C.POINTER(C.c_size_t))(
            sd.get_pencil_offset)
        for name in CASES:
            scene = cases.SMALL_CASES[name]()
            # every rank names its own file: only rank 0 may write one (output.c:102-104)
            path = os.path.join(outdir, f"{name}.rank{rank}.ppm")
            args = _abi.ExecuteArgs(scene, L.converters, path, info.value)
            keep = []
            for idx, c in enumerate(scene.contours):
                nz, ny, nx = c.field.shape
                lo, sz = [], []
                for d, g in enumerate((nx, ny, nz)):
                    m, o = C.c_size_t(), C.c_size_t()
                    assert mysize(info, pencil, d, g, C.byref(m)) == 0
                    assert offset(info, pencil, d, g, C.byref(o)) == 0
                    lo.append(o.value)
                    sz.append(m.value)
                # the caller's pencil-local block (x fastest), global sizes and grids
                local = np.ascontiguousarray(c.field[lo[2]:lo[2] + sz[2], lo[1]:lo[1] + sz[1],
                                                     lo[0]:lo[0] + sz[0]], dtype=np.float64)
                keep.append(local)
                o = args.contours[idx]
                o.pencil = pencil
                o.array = local.ctypes.data_as(C.POINTER(C.c_double))
            rc = L.lib.contour3d_execute(*args.execute_tuple())
            assert rc == 0, f"rank {rank}: contour3d_execute failed on {name}"
            dist.barrier()
            if rank == 0:
                got = _abi.read_ppm(path)[2]
                want = np.load(os.path.join(GOLDEN, f"{name}.npz"))["rgb"]
                diff = (got != want).any(axis=2)
                assert diff.sum() == 0, f"{name}: {int(diff.sum())} pixels differ at {world} ranks, pencil {pencil}"
            else:
                assert not os.path.exists(path), f"rank {rank} wrote an image"
    finally:
        if info.value:
            C.CFUNCTYPE(C.c_int, C.c_void_p)(sd.destruct)(info)
        L.lib.contour3d_gb300_install_transport(None)
        dist.barrier()
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


# (ranks, pencil): X1 splits z at two ranks; Z1 splits y; at four ranks the
# Y2 pencil splits x and z in a 2 x 2 process grid
@pytest.mark.parametrize("world,pencil", [(2, 0), (2, 2), (4, 4)], ids=["2-X1", "2-Z1", "4-Y2"])
def test_rank_zero_image_equals_single_rank_reference(gpu, world, pencil, tmp_path):
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(world, _free_port(), pencil, str(tmp_path)), nprocs=world, join=True)
