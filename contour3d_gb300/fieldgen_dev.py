"""Device field generation into torch tensors (same bytes as fields.py)."""
from __future__ import annotations


def modes_device(lib, shape, nmodes=64, kmin=1, kmax=16, power=5.0 / 6.0, seed=0, dtype=None, out=None,
                 time=0.0):
    """Fourier field on the device (into `out` when given, in place); returns (tensor, std)."""
    import torch
    dtype = dtype or torch.float64
    t = out if out is not None else torch.empty(shape, dtype=dtype, device="cuda")
    std = lib.fieldgen_modes_device(t.data_ptr(), 0 if t.dtype == torch.float64 else 1, tuple(t.shape), nmodes,
                                    kmin, kmax, power, seed, time=time)
    return t, std


def blobs_device(lib, shape, nblobs=8, seed=0):
    import torch
    t = torch.empty(shape, dtype=torch.float64, device="cuda")
    lib.fieldgen_blobs_device(t.data_ptr(), shape, nblobs, seed)
    return t
