"""Parity of the CUDA path with the reference (golden fixtures) and with the
CPU oracle on the same seeded inputs.  Everything integer (counts, cells,
edge ids, pixels) must be bit-exact; the FP64 arithmetic is bit-exact too,
because the device repeats the reference's unfused operations in the same
order -- the tolerance stated for floating point (1e-12 relative) is checked
as well so a failure says which bar was missed."""
import hashlib
import json
import os

import numpy as np
import pytest

from contour3d_gb300 import _abi, fields
from tests import cases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
MANIFEST = json.load(open(os.path.join(GOLDEN, "manifest.json")))
REL_TOL = 1e-12


def sha(b):
    return hashlib.sha256(b).hexdigest()


def assert_close_records(a, b):
    assert len(a) == len(b)
    for name in ("cell", "edge_ids"):
        assert np.array_equal(a[name], b[name]), name
    for name in ("vertices", "vertex_normals", "face_normal", "area"):
        x, y = a[name], b[name]
        finite = np.isfinite(y)
        assert np.array_equal(np.isfinite(x), finite), name
        scale = np.maximum(np.abs(y[finite]), 1e-300)
        assert np.all(np.abs(x[finite] - y[finite]) <= REL_TOL * np.maximum(scale, 1.0)), name
    assert a.tobytes() == b.tobytes(), "records differ in their last bits"


@pytest.mark.parametrize("name", sorted(cases.SMALL_CASES))
def test_image_matches_reference(gpu, name):
    scene = cases.SMALL_CASES[name]()
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    img = gpu.render(scene)
    diff = (img != g["rgb"]).any(axis=2)
    assert diff.sum() == 0, f"{diff.sum()} pixels differ"


@pytest.mark.parametrize("name", sorted(cases.SMALL_CASES))
def test_triangles_match_reference(gpu, name):
    scene = cases.SMALL_CASES[name]()
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    got = [gpu.triangles(c) for c in scene.contours]
    assert [len(t) for t, _ in got] == list(g["per_object"])
    assert [n for _, n in got] == list(g["triangulated"])
    tris = np.concatenate([t for t, _ in got]) if got else np.zeros(0, dtype=g["triangles"].dtype)
    if len(tris):
        assert_close_records(tris, g["triangles"])


def test_cell_counts_match_oracle(gpu, oracle):
    f, std = fields.modes((30, 26, 34), nmodes=24, kmin=1, kmax=6, power=5.0 / 6.0, seed=4)
    for thr in (-0.5 * std, 0.0, 0.5 * std, 10.0, float(f.flat[77])):
        a, ta = gpu.cell_counts(f, thr)
        b, tb = oracle.cell_counts(f, thr)
        assert ta == tb
        assert np.array_equal(a, b)


def test_config0_matches_reference(gpu):
    """128^3 blobs, 1024^2: the reference's own ppm hash and triangle hashes."""
    scene = cases.config0()
    man = MANIFEST["config0"]
    img = gpu.render(scene)
    assert sha(img.tobytes()) == man["ppm_sha256"]
    t, n = gpu.triangles(scene.contours[0])
    assert len(t) == man["rendered"] and n == man["triangulated"]
    assert sha(np.ascontiguousarray(t["vertices"]).tobytes()) == man["vertex_sha256"]
    assert sha(np.ascontiguousarray(t["vertex_normals"]).tobytes()) == man["normal_sha256"]


def test_execute_writes_reference_ppm(gpu, oracle, tmp_path):
    """The drop-in entry point writes the same file the reference would."""
    scene = cases.blobs_small()
    a, b = str(tmp_path / "gpu.ppm"), str(tmp_path / "oracle.ppm")
    assert gpu.execute(scene, a) == 0
    assert oracle.execute(scene, b) == 0
    assert open(a, "rb").read() == open(b, "rb").read()


@pytest.mark.parametrize("slab_cells", [64, 700, 5000])
def test_slab_size_does_not_change_the_image(gpu, slab_cells):
    scene = cases.nonuniform_multi()
    g = np.load(os.path.join(GOLDEN, "nonuniform_multi.npz"))
    try:
        assert gpu.set_slab_cells(slab_cells) == 0
        img = gpu.render(scene)
        tris = [gpu.triangles(c)[0] for c in scene.contours]
    finally:
        gpu.set_slab_cells(178956970)  # the default
    assert np.array_equal(img, g["rgb"])
    assert np.concatenate(tris).tobytes() == g["triangles"].tobytes()


def test_depth_buffer_matches_oracle(gpu, oracle):
    scene = cases.camera_inside()
    img_g, dep_g = gpu.render(scene, with_depth=True)
    img_o, dep_o = oracle.render(scene, with_depth=True)
    assert np.array_equal(img_g, img_o)
    assert dep_g.tobytes() == dep_o.tobytes()


def test_short_line_is_an_error(gpu, tmp_path):
    scene = cases.blobs_small()
    scene.lines[2].nitems = 1
    out = tmp_path / "x.ppm"
    assert gpu.execute(scene, str(out)) == 1
    assert not out.exists()


def test_device_resident_f32_field(gpu, oracle):
    """A float32 field resident on the device renders as its exact widening to double."""
    import torch
    shape = (33, 29, 31)
    f32, std = fields.modes(shape, nmodes=16, kmin=1, kmax=5, power=5.0 / 6.0, seed=12, dtype=np.float32)
    dev = torch.from_numpy(f32).cuda()
    scene = _abi.make_scene(cases.CAM0, cases.CENTRE, 120, 90)
    out = torch.zeros(90 * 120 * 3, dtype=torch.uint8, device="cuda")
    grids = [_abi.unit_grid(n) for n in (31, 29, 33)]
    rc = gpu.render_device(scene, [(dev.data_ptr(), 1, (31, 29, 33), grids, 0.25 * std, (255, 0, 0))],
                           out.data_ptr())
    assert rc == 0
    torch.cuda.synchronize()
    scene.contours = [_abi.Contour(f32.astype(np.float64), 0.25 * std, (255, 0, 0))]
    ref = oracle.render(scene)
    assert np.array_equal(out.cpu().numpy().reshape(90, 120, 3), ref)


def test_device_field_generator_matches_host(gpu):
    import torch
    shape = (20, 18, 22)
    host, std = fields.modes(shape, nmodes=32, kmin=1, kmax=8, power=5.0 / 6.0, seed=3)
    dev = torch.empty(shape, dtype=torch.float64, device="cuda")
    std2 = gpu.fieldgen_modes_device(dev.data_ptr(), 0, shape, 32, 1, 8, 5.0 / 6.0, 3)
    assert std2 == std
    assert dev.cpu().numpy().tobytes() == host.tobytes()
    h32, _ = fields.modes(shape, nmodes=32, kmin=1, kmax=8, power=5.0 / 6.0, seed=3, dtype=np.float32)
    d32 = torch.empty(shape, dtype=torch.float32, device="cuda")
    gpu.fieldgen_modes_device(d32.data_ptr(), 1, shape, 32, 1, 8, 5.0 / 6.0, 3)
    assert d32.cpu().numpy().tobytes() == h32.tobytes()
    b = fields.blobs(shape, nblobs=7, seed=8)
    db = torch.empty(shape, dtype=torch.float64, device="cuda")
    gpu.fieldgen_blobs_device(db.data_ptr(), shape, 7, 8)
    assert db.cpu().numpy().tobytes() == b.tobytes()


@pytest.mark.parametrize("name", sorted(cases.SMALL_CASES) + ["config0"])
def test_single_precision_filter_bounds_hold(gpu, name):
    """With the self-check on, every pixel the FP32 filter classifies is also
    classified with the reference's FP64 arithmetic: no certain decision may
    disagree, no depth may leave its interval, and the image is unchanged."""
    scene = cases.config0() if name == "config0" else cases.SMALL_CASES[name]()
    gpu.set_filter_check(True)
    try:
        img = gpu.render(scene)
        st = gpu.stats()
    finally:
        gpu.set_filter_check(False)
    assert list(st.filter_violations) == [0, 0, 0, 0, 0]
    assert st.shade_violations == 0, "an FP32 colour differs from the FP64 one"
    if name == "config0":
        assert sha(img.tobytes()) == MANIFEST["config0"]["ppm_sha256"]
    else:
        assert np.array_equal(img, np.load(os.path.join(GOLDEN, f"{name}.npz"))["rgb"])


def test_filter_settles_most_fragments(gpu):
    """The FP32 filter must leave only a small share of fragments to the exact path."""
    scene = cases.config0()
    gpu.render(scene)
    st = gpu.stats()
    assert st.candidate_overflows == 0
    assert 0 < st.candidates < 4 * st.triangles
    # the FP32 shading settles all but a small share of the won pixels
    assert st.winners > 0 and st.shade_exact < 0.05 * st.winners


def test_float32_field_threshold_edges(gpu, oracle):
    """float32 fields classify with a float threshold key; edge thresholds
    (between floats, at a float, +-0, huge) must count exactly like the
    double comparison of the widened values."""
    import torch  # noqa: F401
    rng = np.random.default_rng(5)
    f32 = (rng.standard_normal((18, 17, 19)) * 0.5).astype(np.float32)
    f32.flat[::97] = 0.0
    f32.flat[5::101] = -0.0
    as64 = f32.astype(np.float64)
    for thr in (0.0, -0.0, float(f32.flat[3]), float(np.nextafter(f32.flat[3], 1)) * 0.5 + float(f32.flat[3]) * 0.5,
                1e-50, -1e-50, 3.5e38, -3.5e38, 0.1):
        a, ta = gpu.cell_counts(as64, thr)
        b, tb = oracle.cell_counts(as64, thr)
        assert ta == tb and np.array_equal(a, b)
    # the device classify of a float32 field (render path) against the oracle on the widened field
    scene = _abi.make_scene(cases.CAM0, cases.CENTRE, 64, 48)
    out = torch.zeros(64 * 48 * 3, dtype=torch.uint8, device="cuda")
    dev = torch.from_numpy(f32).cuda()
    grids = [_abi.unit_grid(n) for n in (19, 17, 18)]
    for thr in (0.0, float(f32.flat[7]), 0.3):
        assert gpu.render_device(scene, [(dev.data_ptr(), 1, (19, 17, 18), grids, thr, (9, 200, 90))],
                                 out.data_ptr()) == 0
        torch.cuda.synchronize()
        scene.contours = [_abi.Contour(as64, thr, (9, 200, 90))]
        ref = oracle.render(scene)
        scene.contours = []
        assert np.array_equal(out.cpu().numpy().reshape(48, 64, 3), ref)


DBL_MAX = 1.7976931348623157e308
DBL_TRUE_MIN = 5e-324


def test_tma_classify_special_values(gpu, oracle):
    """The TMA classification (x = 20 nodes: 160-byte rows) on a field holding
    NaNs of both signs and several payloads, +-inf, +-0, denormals, +-DBL_MAX
    and values equal to the thresholds, against thresholds at the ends of
    the key ranges.  Only the codes are compared (no vertex is built), so
    non-finite values are fine here; triangulate.c's test is thr < value."""
    rng = np.random.default_rng(8)
    f = rng.standard_normal((14, 13, 20))
    nans = np.array([0x7FF8000000000000, 0xFFF8000000000000, 0x7FF0000000000001, 0xFFFFFFFFFFFFFFFF],
                    dtype=np.uint64).view(np.float64)
    special = np.concatenate([nans, [np.inf, -np.inf, 0.0, -0.0, DBL_TRUE_MIN, -DBL_TRUE_MIN, DBL_MAX, -DBL_MAX,
                                     0.5, -0.5]])
    flat = f.reshape(-1)
    idx = rng.choice(flat.size, 700, replace=False)
    flat[idx] = special[rng.integers(0, special.size, idx.size)]
    for thr in (0.0, -0.0, DBL_TRUE_MIN, -DBL_TRUE_MIN, np.inf, -np.inf, np.nan, DBL_MAX, -DBL_MAX, 0.5, -0.5,
                float(flat[3]), 1e-300, -1e-300):
        a, ta = gpu.cell_counts(f, thr)
        b, tb = oracle.cell_counts(f, thr)
        assert ta == tb and np.array_equal(a, b), thr


def test_tma_classify_float32_threshold_edges(gpu, oracle):
    """The TMA classification of a float32 field (x = 20 nodes: 80-byte rows),
    one and two levels per pass, at thresholds between floats, at a float,
    +-0, beyond FLT_MAX, infinite and NaN, against the oracle on the widened
    field."""
    import torch
    rng = np.random.default_rng(6)
    f32 = (rng.standard_normal((18, 17, 20)) * 0.5).astype(np.float32)
    f32.flat[::97] = 0.0
    f32.flat[5::101] = -0.0
    as64 = f32.astype(np.float64)
    v = float(f32.flat[3])
    between = float(np.nextafter(f32.flat[3], np.float32(1))) * 0.5 + v * 0.5
    scene = _abi.make_scene(cases.CAM0, cases.CENTRE, 64, 48)
    out = torch.zeros(64 * 48 * 3, dtype=torch.uint8, device="cuda")
    dev = torch.from_numpy(f32).cuda()
    sizes = (20, 17, 18)
    grids = [_abi.unit_grid(n) for n in sizes]
    levels = [(0.0,), (-0.0,), (v,), (between,), (1e-50,), (-1e-50,), (3.5e38,), (-3.5e38,), (np.inf,), (-np.inf,),
              (np.nan,), (0.1, -0.2), (v, between), (-0.0, 0.3)]
    cols = ((9, 200, 90), (200, 30, 120))
    for lv in levels:
        objs = [(dev.data_ptr(), 1, sizes, grids, t, c) for t, c in zip(lv, cols)]
        assert gpu.render_device(scene, objs, out.data_ptr()) == 0
        torch.cuda.synchronize()
        scene.contours = [_abi.Contour(as64, t, c) for t, c in zip(lv, cols)]
        ref = oracle.render(scene)
        scene.contours = []
        assert np.array_equal(out.cpu().numpy().reshape(48, 64, 3), ref), lv


@pytest.mark.parametrize("camera", [(2.5, 2.0, 1.5), (0.6, 0.4, 3.0)], ids=["ascending-z", "descending-z"])
def test_pipelined_host_upload_matches_device_field(gpu, camera):
    """A host field large enough to be uploaded in chunks, with the slabs of
    both objects starting as their node slices arrive (both slab orders),
    draws the image the device-resident field draws."""
    import torch
    shape = (200, 200, 210)  # 67 MB of float64
    dev = torch.empty(shape, dtype=torch.float64, device="cuda")
    std = gpu.fieldgen_modes_device(dev.data_ptr(), 0, shape, 24, 1, 6, 5.0 / 6.0, 21)
    host = dev.cpu().numpy()
    sizes = (shape[2], shape[1], shape[0])
    grids = [_abi.unit_grid(n) for n in sizes]
    levels = [(0.3 * std, (250, 40, 40)), (-0.4 * std, (40, 80, 250))]
    scene = _abi.make_scene(camera, cases.CENTRE, 320, 240)
    out = torch.zeros(240 * 320 * 3, dtype=torch.uint8, device="cuda")
    assert gpu.render_device(scene, [(dev.data_ptr(), 0, sizes, grids, thr, col) for thr, col in levels],
                             out.data_ptr()) == 0
    torch.cuda.synchronize()
    scene.contours = [_abi.Contour(host, thr, col, grids=tuple(grids)) for thr, col in levels]
    img = gpu.render(scene)
    assert np.array_equal(img, out.cpu().numpy().reshape(240, 320, 3))
    # both objects take the field in more than one slab as it arrives
    assert gpu.stats().slabs > 2


def test_five_levels_of_one_field(gpu, oracle):
    """Five objects on one host field: the objects are classified together
    (four thresholds in one pass over the field, then the fifth), each keeps
    its own cell codes, and the image is the reference's."""
    f, std = fields.modes((30, 26, 34), nmodes=16, kmin=1, kmax=5, power=5.0 / 6.0, seed=31)
    levels = [(-1.0, (250, 40, 40)), (-0.5, (40, 250, 40)), (0.0, (40, 40, 250)), (0.5, (250, 250, 40)),
              (1.0, (40, 250, 250))]
    s = _abi.make_scene(cases.CAM0, cases.CENTRE, 160, 120)
    s.contours = [_abi.Contour(f, q * std, c) for q, c in levels]
    assert np.array_equal(gpu.render(s), oracle.render(s))


def test_five_levels_of_one_device_f32_field(gpu, oracle):
    """The same on a float32 field resident on the device (thresholds compared
    through float keys in the shared pass)."""
    import torch
    shape = (26, 30, 22)
    f32, std = fields.modes(shape, nmodes=16, kmin=1, kmax=5, power=5.0 / 6.0, seed=33, dtype=np.float32)
    dev = torch.from_numpy(f32).cuda()
    sizes = (shape[2], shape[1], shape[0])
    grids = [_abi.unit_grid(n) for n in sizes]
    levels = [(-0.8 * std, (250, 40, 40)), (-0.3 * std, (40, 250, 40)), (0.1 * std, (40, 40, 250)),
              (0.4 * std, (250, 250, 40)), (0.9 * std, (40, 250, 250))]
    scene = _abi.make_scene(cases.CAM0, cases.CENTRE, 160, 120)
    out = torch.zeros(120 * 160 * 3, dtype=torch.uint8, device="cuda")
    assert gpu.render_device(scene, [(dev.data_ptr(), 1, sizes, grids, t, c) for t, c in levels], out.data_ptr()) == 0
    torch.cuda.synchronize()
    scene.contours = [_abi.Contour(f32.astype(np.float64), t, c) for t, c in levels]
    assert np.array_equal(out.cpu().numpy().reshape(120, 160, 3), oracle.render(scene))


def test_dense_field_scans_again_with_a_larger_map(gpu, oracle):
    """White noise crosses about 7.5 triangles per cell, far more than the
    triangle -> cell map a fresh context sizes for a slab (one entry per two
    cells): the scan finds that its map does not fit, the map grows and the
    slab is scanned again.  Image and per-cell counts stay the oracle's."""
    rng = np.random.default_rng(41)
    f = rng.random((34, 38, 36))
    s = _abi.make_scene(cases.CAM0, cases.CENTRE, 160, 120)
    s.contours = [_abi.Contour(f, 0.5, (200, 120, 40))]
    gpu.release()  # a fresh context: buffers sized from this frame alone
    gpu.set_async(False)
    try:
        img = gpu.render(s)
        st = gpu.stats()
    finally:
        gpu.set_async(True)
    ncell = 35 * 37 * 33
    assert st.triangles > ncell // 2 + 1024, "the map was large enough: the test no longer covers the rescan"
    assert np.array_equal(img, oracle.render(s))
    cg, tg = gpu.cell_counts(f, 0.5)
    co, to = oracle.cell_counts(f, 0.5)
    assert tg == to and np.array_equal(cg, co)
