"""Frames rendered with one host synchronisation (at the end) against frames
that synchronise after every slab pass.

Without synchronisation the buffers are sized before the counts are known,
from the largest counts the context has seen; every kernel that would find
more work than its buffer holds records an overflow instead, and the frame
is rendered again with synchronisation.  Either way the image and the
statistics must be the same as the synchronised frame's."""
import os

import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
# counts that depend only on the geometry; not the FP64-shaded pixels and
# their neighbour entries: the FP32 shading uses a winner's stored weights
# only when all three of its 16-byte words carry the winner's tag, and a
# fragment that lost the z-test after winning a CAS may overwrite a word
# late, so how many pixels fall back to the (exact) FP64 colour depends on
# timing -- the colours do not
KEYS = ("triangles", "vertices", "candidates", "tiny", "cover_triangles", "exact_fragments", "slivers", "winners",
        "slabs")


def _stats(gpu):
    st = gpu.stats()
    return {k: int(getattr(st, k)) for k in KEYS}, st


@pytest.mark.parametrize("name", sorted(cases.SMALL_CASES) + ["config0"])
def test_unsynchronised_frame_equals_synchronised(gpu, name):
    scene = cases.config0() if name == "config0" else cases.SMALL_CASES[name]()
    try:
        gpu.set_async(False)
        ref = gpu.render(scene)
        ref_stats, st = _stats(gpu)
        assert st.unsynchronised == 0
        gpu.set_async(True)
        gpu.render(scene)  # sizes learnt from this scene at the latest here
        img = gpu.render(scene)
        got_stats, st = _stats(gpu)
    finally:
        gpu.set_async(True)
    assert st.unsynchronised == 1 and st.redone == 0
    assert np.array_equal(img, ref)
    assert got_stats == ref_stats


def test_overflow_renders_the_frame_again(gpu):
    """Sizes learnt on a small scene are too small for a larger one: the
    unsynchronised pass records the overflow and the frame is rendered again
    with synchronisation, to the same image."""
    gpu.release()  # forget the sizes learnt so far
    small = cases.tiny()
    gpu.render(small)
    gpu.render(small)
    assert gpu.stats().unsynchronised == 1
    big = cases.config0()
    img = gpu.render(big)
    st = gpu.stats()
    assert st.redone == 1 and st.unsynchronised == 0
    import hashlib
    import json
    man = json.load(open(os.path.join(GOLDEN, "manifest.json")))["config0"]
    assert hashlib.sha256(img.tobytes()).hexdigest() == man["ppm_sha256"]
    # the next frame of the same scene runs unsynchronised with the learnt sizes
    img2 = gpu.render(big)
    assert gpu.stats().unsynchronised == 1 and np.array_equal(img, img2)


def test_shading_list_overflow_renders_the_frame_again(gpu, oracle):
    """The FP64 shading pass's neighbour lists, sized from another scene, are
    too small for a scene whose every won pixel takes that pass (a
    non-identity converter) at a larger image: the unsynchronised frame
    records the overflow and is rendered again, to the oracle's image.  The
    pass that overflowed still computes every list entry below the lists'
    capacity, so none of them is a stale word from an earlier frame."""
    gpu.release()  # forget the sizes learnt so far
    # more triangles and candidates than the converter scene, few FP64 pixels
    learn = cases.config0()
    gpu.render(learn)
    gpu.render(learn)
    st = gpu.stats()
    assert st.unsynchronised == 1
    learnt = st.normals
    big = cases.modes_warp(768, 576)
    img = gpu.render(big)
    st = gpu.stats()
    # the unsynchronised pass had room for about max(1.25 x learnt, 2^16) entries
    assert st.normals > 2 * max(learnt, 1 << 16), (st.normals, learnt)
    assert st.redone == 1 and st.unsynchronised == 0
    assert np.array_equal(img, oracle.render(big))
    img2 = gpu.render(big)
    assert gpu.stats().unsynchronised == 1 and np.array_equal(img, img2)


def test_repeated_device_frame_runs_as_a_graph(gpu, oracle):
    """An in-situ loop: the same device field, levels and camera every step,
    new field values.  The second frame with one description is recorded as
    a CUDA graph and later ones launch it; every image equals the oracle's
    on that step's values, and the graph runs on the caller's stream."""
    import torch
    from contour3d_gb300 import _abi
    shape = (48, 40, 44)
    dev = torch.empty(shape, dtype=torch.float64, device="cuda")
    std = gpu.fieldgen_modes_device(dev.data_ptr(), 0, shape, 16, 1, 5, 5.0 / 6.0, 17)
    nz, ny, nx = shape
    grids = [_abi.unit_grid(n) for n in (nx, ny, nz)]
    levels = [(-0.4 * std, (250, 60, 60)), (0.3 * std, (60, 90, 250))]
    scene = _abi.make_scene(cases.CAM0, cases.CENTRE, 200, 150)
    out = torch.zeros(200 * 150 * 3, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    fl = [(dev.data_ptr(), 0, (nx, ny, nz), grids, t, c) for t, c in levels]
    gpu.set_graphs(True)
    seen = []
    for step in range(5):
        # the solver advances the field in place on its stream (phases by omega dt)
        gpu.fieldgen_modes_device_async(dev.data_ptr(), 0, shape, 16, 1, 5, 5.0 / 6.0, 17, 0.01 * step,
                                        stream.cuda_stream)
        assert gpu.render_device(scene, fl, out.data_ptr(), stream.cuda_stream) == 0
        stream.synchronize()
        st = gpu.stats()
        seen.append(int(st.graph))
        host = dev.cpu().numpy()
        scene.contours = [_abi.Contour(host, t, c, grids=tuple(grids)) for t, c in levels]
        ref = oracle.render(scene)
        scene.contours = []
        assert np.array_equal(out.cpu().numpy().reshape(150, 200, 3), ref), f"step {step}"
        assert st.triangles > 0 and st.slabs == 2
    # first frame: learns the counts or runs unsynchronised; then recorded; then launched
    assert 1 in seen and seen[-1] == 2 and seen[-2] == 2
