"""Parity on the benchmark workloads themselves, not only on small scenes.

The FP32 filter's bounds depend on the scene (coordinate range, camera,
screen size, triangle density), so the configurations the bench times are
checked against the oracle at full size:

- the 512^3 float64 Fourier field at +-0.5 std, 1920 x 1080 (the bench's
  headline workload), with the filter self-check on: zero bound violations,
  the oracle's image byte for byte, per-cell triangle counts equal;
- three frames of the 64-field batched workload (a float32 field, a frame
  with four levels, the most elongated field near 384 nodes), rendered alone
  and inside the batched form, against the oracle on the widened field;
- the 1536^3 float32 workload's levels, camera and 3840 x 2160 image on the
  field's 256^3 centre crop, in one slab and in many.

The oracle runs with one emulated z-split rank per host core (the image does
not depend on the split: the nearest-depth reduction is exact).
"""
import os

import numpy as np
import pytest

from contour3d_gb300 import _abi, workloads
from tests import cases

pytestmark = pytest.mark.gpu

CORES = os.cpu_count() or 1


def _config1_field(gpu):
    import torch
    p = cases.config1_params()
    dev = torch.empty(p["shape"], dtype=torch.float64, device="cuda")
    std = gpu.fieldgen_modes_device(dev.data_ptr(), 0, p["shape"], p["nmodes"], p["kmin"], p["kmax"], p["power"],
                                    p["seed"])
    return dev, std


def test_bench_workload_matches_oracle(gpu, oracle):
    """512^3 f64, two levels, 1920 x 1080: device-resident and host paths,
    filter self-check, image and per-cell counts against the oracle."""
    import torch
    dev, std = _config1_field(gpu)
    nz, ny, nx = dev.shape
    host = dev.cpu().numpy()
    grids = [_abi.unit_grid(n) for n in (nx, ny, nz)]
    scene, levels = cases.config1_scene(std)
    W, H = scene.width, scene.height
    out = torch.zeros(W * H * 3, dtype=torch.uint8, device="cuda")
    gpu.set_filter_check(True)
    try:
        rc = gpu.render_device(scene, [(dev.data_ptr(), 0, (nx, ny, nz), grids, t, c) for t, c in levels],
                               out.data_ptr())
        torch.cuda.synchronize()
        st = gpu.stats()
    finally:
        gpu.set_filter_check(False)
    assert rc == 0
    assert list(st.filter_violations) == [0, 0, 0, 0, 0], "an FP32 raster decision left its bound"
    assert st.shade_violations == 0, "an FP32 colour differs from the FP64 one"
    assert st.candidate_overflows == 0
    img_dev = out.cpu().numpy().reshape(H, W, 3)
    scene.contours = [_abi.Contour(host, t, c, grids=tuple(grids)) for t, c in levels]
    ref = oracle.render(scene, nranks=CORES)
    diff = (img_dev != ref).any(axis=2)
    assert diff.sum() == 0, f"{int(diff.sum())} pixels differ from the oracle"
    # the drop-in's host path (chunked upload overlapped with the slabs) draws the same image
    assert np.array_equal(gpu.render(scene), ref)
    # triangulated set: per-cell counts and the device's own total
    total = 0
    for t, _ in levels:
        cg, tg = gpu.cell_counts(host, t)
        co, to = oracle.cell_counts(host, t)
        assert tg == to
        assert np.array_equal(cg, co)
        total += to
        del cg, co
    assert st.triangles == total
    assert st.slabs == 2, "the whole field is one slab per level"


def _pick_frames(fields, frames):
    """A float32 frame, a frame with four levels, and the frame whose field is
    the most elongated among those with a dimension of at least 320 nodes."""
    import torch
    f32 = next(q for q, s in enumerate(frames) if fields[s.field].dtype == torch.float32)
    four = next(q for q, s in enumerate(frames) if len(s.levels) == 4 and q != f32)

    def elongation(q):
        sh = fields[frames[q].field].shape
        return max(sh) / min(sh) if max(sh) >= 320 else 0.0

    rest = [q for q in range(len(frames)) if q not in (f32, four)]
    long_ = max(rest, key=elongation)
    return [f32, four, long_]


def test_batched_workload_frames_match_oracle(gpu, oracle):
    """Three frames of the batched workload, alone (filter self-check on) and
    inside one batch of all 64 frames, against the oracle on the widened field."""
    import torch
    fields, frames = workloads.batch_set(gpu)
    picks = _pick_frames(fields, frames)
    outs = [torch.zeros(s.width * s.height * 3, dtype=torch.uint8, device="cuda") for s in frames]
    packs = [workloads.frame_pack(gpu, fields[s.field], s, o) for s, o in zip(frames, outs)]
    alone = {}
    gpu.set_filter_check(True)
    try:
        for q in picks:
            assert gpu.render_pack(packs[q]) == 0
            torch.cuda.synchronize()
            st = gpu.stats()
            assert list(st.filter_violations) == [0, 0, 0, 0, 0], f"frame {q}"
            assert st.shade_violations == 0, f"frame {q}"
            alone[q] = outs[q].cpu().numpy().copy()
    finally:
        gpu.set_filter_check(False)
    for o in outs:
        o.zero_()
    gpu.render_batch(packs, workers=8)
    torch.cuda.synchronize()
    for q in picks:
        s = frames[q]
        f = fields[s.field]
        nz, ny, nx = f.shape
        grids = tuple(_abi.unit_grid(n) for n in (nx, ny, nz))
        host = f.double().cpu().numpy()  # a float32 field widened exactly
        scene = _abi.make_scene(s.camera, (0.5, 0.5, 0.5), s.width, s.height)
        scene.contours = [_abi.Contour(host, lv, c, grids=grids) for lv, c in zip(s.levels, s.colors)]
        ref = oracle.render(scene, nranks=CORES).reshape(-1)
        assert np.array_equal(alone[q], ref), f"frame {q} ({tuple(f.shape)}, {f.dtype}) differs alone"
        assert np.array_equal(outs[q].cpu().numpy(), ref), f"frame {q} differs inside the batch"


def test_large_workload_crop_matches_oracle(gpu, oracle):
    """The 1536^3 float32 field's workload (256 Fourier modes, |k| 1..48,
    |k|^-11/6, four levels at +-0.5 and +-1 std, 3840 x 2160) on the 256^3
    centre crop of the field: filter self-check on, the oracle's image on
    the widened values byte for byte, and the crop split into slabs of a few
    slices each (the 1536^3 frame takes 21 slabs per level) drawing the same
    image."""
    import torch
    n, crop = 1536, 256
    off = (n - crop) // 2
    dev = torch.empty((crop,) * 3, dtype=torch.float32, device="cuda")
    std = gpu.fieldgen_modes_device(dev.data_ptr(), 1, (crop,) * 3, 256, 1, 48, 11.0 / 6.0, 4, offset=(off,) * 3,
                                    glshape=(n, n, n))
    grids = [_abi.unit_grid(n)[off:off + crop]] * 3
    levels = list(zip([-std, -0.5 * std, 0.5 * std, std], workloads.PALETTE))
    scene = _abi.make_scene(cases.CAM0, cases.CENTRE, 3840, 2160)
    W, H = scene.width, scene.height
    fl = [(dev.data_ptr(), 1, (crop,) * 3, grids, t, c) for t, c in levels]
    out = torch.zeros(W * H * 3, dtype=torch.uint8, device="cuda")
    gpu.set_filter_check(True)
    try:
        rc = gpu.render_device(scene, fl, out.data_ptr())
        torch.cuda.synchronize()
        st = gpu.stats()
    finally:
        gpu.set_filter_check(False)
    assert rc == 0
    assert list(st.filter_violations) == [0, 0, 0, 0, 0], "an FP32 raster decision left its bound"
    assert st.shade_violations == 0, "an FP32 colour differs from the FP64 one"
    img = out.cpu().numpy().reshape(H, W, 3)
    host = dev.double().cpu().numpy()  # the float32 values widened exactly
    scene.contours = [_abi.Contour(host, t, c, grids=tuple(grids)) for t, c in levels]
    ref = oracle.render(scene, nranks=CORES)
    scene.contours = []
    diff = (img != ref).any(axis=2)
    assert diff.sum() == 0, f"{int(diff.sum())} pixels differ from the oracle"
    # many slabs per level: the image does not change
    gpu.set_slab_cells(12 * (crop - 1) ** 2)
    try:
        out.zero_()
        assert gpu.render_device(scene, fl, out.data_ptr()) == 0
        torch.cuda.synchronize()
        assert gpu.stats().slabs > 4 * 4
    finally:
        gpu.set_slab_cells(178956970)  # the default
    assert np.array_equal(out.cpu().numpy().reshape(H, W, 3), ref)
