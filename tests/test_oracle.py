"""The CPU oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the reference compiled from its sources),
and against the reference itself where its tree is present."""
import hashlib
import json
import os

import numpy as np
import pytest

from contour3d_gb300 import fields
from tests import cases

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
MANIFEST = json.load(open(os.path.join(GOLDEN, "manifest.json")))


def sha(b):
    return hashlib.sha256(b).hexdigest()


def test_field_generator_is_pinned(built):
    """The seeded generator gives the bytes recorded when the fixtures were made."""
    man = MANIFEST["fields"]
    assert sha(fields.blobs((128, 128, 128), nblobs=8, seed=0).tobytes()) == man["blobs_128_seed0"]
    f, std = fields.modes((40, 36, 48), nmodes=64, kmin=1, kmax=16, power=5.0 / 6.0, seed=1)
    assert sha(f.tobytes()) == man["modes_48x36x40_seed1_f64"]
    assert repr(std) == man["modes_seed1_std"]
    g, _ = fields.modes((40, 36, 48), nmodes=64, kmin=1, kmax=16, power=5.0 / 6.0, seed=1,
                        dtype=np.float32)
    assert sha(g.tobytes()) == man["modes_48x36x40_seed1_f32"]


@pytest.mark.parametrize("name", sorted(cases.SMALL_CASES))
def test_oracle_image_matches_reference(oracle, name):
    scene = cases.SMALL_CASES[name]()
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    img = oracle.render(scene)
    assert img.shape == g["rgb"].shape
    assert np.array_equal(img, g["rgb"])
    assert sha(img.tobytes()) == MANIFEST["cases"][name]["ppm_sha256"]


@pytest.mark.parametrize("name", sorted(cases.SMALL_CASES))
def test_oracle_triangles_match_reference(oracle, name):
    scene = cases.SMALL_CASES[name]()
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    got = [oracle.triangles(c) for c in scene.contours]
    tris = np.concatenate([t for t, _ in got]) if got else np.zeros(0)
    assert [len(t) for t, _ in got] == list(g["per_object"])
    assert [n for _, n in got] == list(g["triangulated"])
    # bit-exact: vertices, vertex normals, face normals, areas, cells, edge ids
    assert tris.tobytes() == g["triangles"].tobytes()


def test_oracle_config0_matches_reference(oracle):
    """128^3 blobs at 1024^2: the reference's ppm hash and triangle hashes."""
    scene = cases.config0()
    img = oracle.render(scene)
    man = MANIFEST["config0"]
    assert sha(img.tobytes()) == man["ppm_sha256"]
    t, n = oracle.triangles(scene.contours[0])
    assert len(t) == man["rendered"] and n == man["triangulated"]
    assert sha(np.ascontiguousarray(t["vertices"]).tobytes()) == man["vertex_sha256"]
    assert sha(np.ascontiguousarray(t["vertex_normals"]).tobytes()) == man["normal_sha256"]


@pytest.mark.parametrize("nranks", [2, 3, 4])
def test_oracle_emulated_ranks(oracle, nranks):
    """The z-split emulation of extend.c + the nearest-depth reduce gives the
    single-rank image (duplicated seam triangles are identical)."""
    scene = cases.blobs_small()
    a = oracle.render(scene)
    b = oracle.render(scene, nranks=nranks)
    assert (a != b).any(axis=2).sum() <= 0.001 * a.shape[0] * a.shape[1]


def test_oracle_cell_counts_total(oracle):
    scene = cases.blobs_small()
    counts, total = oracle.cell_counts(scene.contours[0].field, 0.5)
    _, triangulated = oracle.triangles(scene.contours[0])
    assert counts.sum() == total == triangulated


def test_oracle_rejects_short_line(oracle, tmp_path):
    scene = cases.blobs_small()
    scene.lines[0].nitems = 1
    assert oracle.execute(scene, str(tmp_path / "x.ppm")) == 1


def test_against_reference_build(tmp_path):
    """Direct comparison with the compiled reference (only where its tree exists)."""
    from oracle import lib as olib
    if not os.path.isdir(olib.REF_TREE):
        pytest.skip("reference tree not present on this host")
    olib.build(with_reference=True)
    ref, orc = olib.Reference(), olib.Oracle()
    for seed in range(3):
        f = fields.blobs((15 + seed, 17, 19 - seed), nblobs=5, seed=100 + seed)
        from contour3d_gb300 import _abi
        s = _abi.make_scene((2.0 + seed, -1.5, 1.0), (0.5, 0.5, 0.5), 90, 70)
        s.contours = [_abi.Contour(f, 0.3 + 0.1 * seed, (255, 255, 255))]
        s.lines = _abi.cube_edges(nitems=2 + seed, width=1.0 + seed)
        assert np.array_equal(ref.render(s, str(tmp_path)), orc.render(s))
        assert ref.triangles(s.contours[0])[0].tobytes() == orc.triangles(s.contours[0])[0].tobytes()


def test_against_reference_build_special_values(tmp_path):
    """NaNs (both signs, several payloads), +-inf, +-0, denormals and
    +-DBL_MAX in the field, at thresholds on the edges of the comparison
    (triangulate.c: threshold < value): the oracle's triangle counts and
    images equal the compiled reference's, and its triangle records equal
    them value for value, NaN where the reference has NaN.  The NaN bit
    patterns themselves are not compared: which operand's payload and sign an
    x86 operation propagates depends on the compiler's operand order, which
    differs between the two builds."""
    from oracle import lib as olib
    from contour3d_gb300 import _abi
    if not os.path.isdir(olib.REF_TREE):
        pytest.skip("reference tree not present on this host")
    olib.build(with_reference=True)
    ref, orc = olib.Reference(), olib.Oracle()
    dbl_max, tmin = 1.7976931348623157e308, 5e-324
    rng = np.random.default_rng(8)
    f = rng.standard_normal((14, 13, 20))
    nans = np.array([0x7FF8000000000000, 0xFFF8000000000000, 0x7FF0000000000001, 0xFFFFFFFFFFFFFFFF],
                    dtype=np.uint64).view(np.float64)
    special = np.concatenate([nans, [np.inf, -np.inf, 0.0, -0.0, tmin, -tmin, dbl_max, -dbl_max, 0.5, -0.5]])
    flat = f.reshape(-1)
    idx = rng.choice(flat.size, 700, replace=False)
    flat[idx] = special[rng.integers(0, special.size, idx.size)]
    for thr in (0.0, -0.0, tmin, -tmin, np.inf, -np.inf, np.nan, dbl_max, -dbl_max, 0.5, -0.5):
        c = _abi.Contour(f, thr, (200, 100, 50))
        rt, rn = ref.triangles(c)
        ot, on = orc.triangles(c)
        assert rn == on and rt.shape == ot.shape, thr
        for name in rt.dtype.names:
            if rt[name].dtype.kind == "f":
                assert np.array_equal(rt[name], ot[name], equal_nan=True), (thr, name)
            else:
                assert np.array_equal(rt[name], ot[name]), (thr, name)
        s = _abi.make_scene((2.5, 2.0, 1.5), (0.5, 0.5, 0.5), 90, 70)
        s.contours = [c]
        assert np.array_equal(ref.render(s, str(tmp_path)), orc.render(s)), thr
