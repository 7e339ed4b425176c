"""The allocation-free offsets entry point, called through the C ABI.

contour3d_gb300_cell_offsets_noalloc serves callers that cannot let the
library allocate device memory (a solver whose pool owns the GPU's memory,
or a loop that must not stall on cudaFree's device synchronisation).  Its
result must equal what the existing entry point contour3d_gb300_debug_cell_counts
gives (integers: exactly), on two calls in a row, since every call reuses
the same static scratch array.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from contour3d_gb300 import fields

pytestmark = pytest.mark.gpu


def _fn(gpu):
    # argument and result types are declared by contour3d_gb300/lib.py
    return gpu.lib.contour3d_gb300_cell_offsets_noalloc


# (nz, ny, nx) nodes: 44,352 cells (11 scan tiles of 4,096 cells); 4,095 cells,
# so that the n + 1 offsets fill exactly one tile; 128^3 cells (512 tiles), so
# that a tile's look-back walks past more than one window of 32 predecessors
SHAPES = [(37, 29, 45), (22, 14, 16), (129, 129, 129)]


@pytest.mark.parametrize("shape", SHAPES, ids=["x".join(map(str, s)) for s in SHAPES])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_noalloc_offsets_match_existing_entry_point(gpu, oracle, dtype, shape):
    import torch
    host, std = fields.modes(shape, nmodes=24, kmin=1, kmax=7, power=5.0 / 6.0, seed=31,
                             dtype=np.float64 if dtype == "f64" else np.float32)
    fn = _fn(gpu)
    dev = torch.from_numpy(host).cuda()
    nz, ny, nx = shape
    sizes = (C.c_size_t * 3)(nx, ny, nz)
    n = (nx - 1) * (ny - 1) * (nz - 1)
    for thr in (0.3 * std, -0.6 * std):
        # the existing entry point, and the oracle on the same (widened) values
        counts, total = gpu.cell_counts(host.astype(np.float64), thr)
        ocounts, ototal = oracle.cell_counts(host.astype(np.float64), thr)
        assert ototal == total and np.array_equal(ocounts, counts)
        expect = np.zeros(n + 1, dtype=np.int64)
        expect[1:] = np.cumsum(counts.ravel().astype(np.int64))
        assert expect[-1] == total
        for call in range(2):
            out = torch.full((n + 1,), -1, dtype=torch.int32, device="cuda")
            tot = torch.zeros(1, dtype=torch.int64, device="cuda")
            rc = fn(C.c_void_p(dev.data_ptr()), 0 if dtype == "f64" else 1, sizes, thr,
                    C.c_void_p(out.data_ptr()), C.c_void_p(tot.data_ptr()), None)
            assert rc == 0, f"call {call} failed"
            got = out.cpu().numpy().astype(np.int64) & 0xFFFFFFFF
            assert np.array_equal(got, expect), f"call {call}: offsets differ"
            assert int(tot.item()) == total


def test_noalloc_rejects_fields_beyond_its_limit(gpu):
    """Sizes above the static scratch limit are refused on the host, before any launch."""
    import torch
    fn = _fn(gpu)
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = torch.zeros(8, dtype=torch.int32, device="cuda")
    tot = torch.zeros(1, dtype=torch.int64, device="cuda")
    sizes = (C.c_size_t * 3)(1024, 1024, 1024)
    assert fn(C.c_void_p(dummy.data_ptr()), 0, sizes, 0.0, C.c_void_p(out.data_ptr()),
              C.c_void_p(tot.data_ptr()), None) == 1
