"""Seeded workloads of the batched and served forms, generated on the device.

batch_set()   many fields of uneven, non-cubic shape (each dimension drawn in
              64..384 nodes by default), half float64 and half float32,
              Gaussian-blob or Fourier fields, 1-4 levels at sampled value
              quantiles in [0.3, 0.7], a random camera on a sphere of radius
              2.5 looking at the cube centre, 1024 x 1024 each.
served_set()  resident fields of the served stream: shapes drawn from
              {96^3, 192^3, 256x256x512, 384^3, 768^3}, float32 or float64,
              Fourier fields whose phases advance by omega dt (omega = |k|)
              every `advance_every` requests; 1-3 levels and a camera per
              request, 1280 x 720.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Tuple

import numpy as np

from . import _abi
from .fieldgen_dev import modes_device, blobs_device  # noqa: F401  (re-exported)


@dataclass
class FieldSpec:
    shape: Tuple[int, int, int]  # (nz, ny, nx)
    dtype: str                   # "f64" or "f32"
    kind: str                    # "blobs" or "modes"
    seed: int
    nblobs: int = 8
    nmodes: int = 32
    kmax: int = 8


@dataclass
class FrameSpec:
    field: int                   # index into the field list
    levels: List[float]
    colors: List[Tuple[int, int, int]]
    camera: Tuple[float, float, float]
    width: int
    height: int


def random_camera(rng, radius=2.5, centre=(0.5, 0.5, 0.5)):
    while True:
        v = rng.standard_normal(3)
        n = np.linalg.norm(v)
        if n > 1e-3 and abs(v[2] / n) < 0.95:
            break
    v = v / n * radius
    return tuple((np.asarray(centre) + v).tolist())


PALETTE = [(0, 255, 255), (255, 255, 0), (255, 64, 64), (64, 255, 64)]


def quantile_levels(dev_field, rng, count, lo=0.3, hi=0.7, samples=200_000):
    """Levels at uniformly drawn quantiles of a random sample of the values
    (a torch tensor, or a numpy array: the same draws give the same levels)."""
    if isinstance(dev_field, np.ndarray):
        flat = dev_field.reshape(-1)
        vals = flat[rng.integers(0, flat.size, size=min(samples, flat.size))].astype(np.float64)
    else:
        import torch
        flat = dev_field.reshape(-1)
        idx = torch.from_numpy(rng.integers(0, flat.numel(), size=min(samples, flat.numel()))).to(flat.device)
        vals = flat[idx].double().cpu().numpy()
    qs = np.sort(rng.uniform(lo, hi, size=count))
    return [float(np.quantile(vals, q)) for q in qs]


def batch_set(lib, nfields=64, nmin=64, nmax=384, width=1024, height=1024, seed=2024, host=False, twins=False):
    """Fields and frame specs of the batched workload: device tensors, or with
    host=True the same values as numpy arrays generated on the host cores
    (no GPU needed; `lib` is then unused).  With twins=True (device only) a
    third result maps the index of every float32 field to the float64 field
    it was made from (the same seed in double precision)."""
    from . import fields as hostgen
    rng = np.random.default_rng(seed)
    fields, frames, twin = [], [], {}
    for n in range(nfields):
        shape = tuple(int(x) for x in rng.integers(nmin, nmax + 1, size=3))
        dtype = "f64" if n % 2 == 0 else "f32"
        kind = "blobs" if rng.random() < 0.5 else "modes"
        if kind == "blobs":
            nb = int(rng.integers(4, 33))
            if host:
                f = hostgen.blobs_threaded(shape, nb, seed=1000 + n)
                f = f.astype(np.float32) if dtype == "f32" else f
            else:
                f = blobs_device(lib, shape, nb, seed=1000 + n)
                if dtype == "f32":
                    if twins:
                        twin[n] = f
                    f = f.float()
        else:
            if host:
                f, _ = hostgen.modes_threaded(shape, nmodes=64, kmin=1, kmax=16, power=5.0 / 6.0, seed=2000 + n,
                                              dtype=np.float64 if dtype == "f64" else np.float32)
            else:
                import torch
                f, _ = modes_device(lib, shape, nmodes=64, kmin=1, kmax=16, power=5.0 / 6.0, seed=2000 + n,
                                    dtype=torch.float64 if dtype == "f64" else torch.float32)
                if twins and dtype == "f32":
                    twin[n], _ = modes_device(lib, shape, nmodes=64, kmin=1, kmax=16, power=5.0 / 6.0,
                                              seed=2000 + n, dtype=torch.float64)
        fields.append(f)
        nlev = int(rng.integers(1, 5))
        levels = quantile_levels(f, rng, nlev)
        frames.append(FrameSpec(n, levels, PALETTE[:nlev], random_camera(rng), width, height))
    return (fields, frames, twin) if twins else (fields, frames)


SERVED_SHAPES = [(96, 96, 96), (192, 192, 192), (512, 256, 256), (384, 384, 384), (768, 768, 768)]


def frame_pack(lib, dev_field, spec: FrameSpec, rgb_dev):
    import torch
    nz, ny, nx = dev_field.shape
    grids = [_abi.unit_grid(n) for n in (nx, ny, nz)]
    dt = 0 if dev_field.dtype == torch.float64 else 1
    fl = [(dev_field.data_ptr(), dt, (nx, ny, nz), grids, lv, col) for lv, col in zip(spec.levels, spec.colors)]
    scene = _abi.make_scene(spec.camera, (0.5, 0.5, 0.5), spec.width, spec.height)
    return lib.frame(scene, fl, rgb_dev.data_ptr())
