"""Host-side checks that need no GPU: the native library loads and exports
every symbol the public headers declare; the built-in decomposition answers
the queries the reference makes of SimpleDecomp."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in ("contour3d.h", "contour3d_gb300.h", "sdecomp.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:extern\s+)?[A-Za-z_][\w\s\*]*?\b(\w+)\s*\(", src, flags=re.M):
            name = m.group(1)
            if name.startswith(("contour3d_", "c3d_")) and not name.endswith("_t"):
                names.add(name)
        for m in re.finditer(r"extern\s+const\s+\w+\s+(\w+)\s*;", src):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(built):
    from contour3d_gb300 import lib
    so = lib.LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    want = declared_symbols()
    assert {"contour3d_execute", "contour3d_gb300_render_device", "sdecomp", "c3d_comm_world"} <= want
    missing = want - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    L = lib.Library()
    for name in want:
        if name != "sdecomp":
            assert getattr(L.lib, name) is not None


def test_library_loads_without_gpu(built):
    from contour3d_gb300 import lib
    L = lib.Library()
    s = lib.Stats()
    assert L.lib.contour3d_gb300_last_stats(C.byref(s)) == 0
    assert L.lib.contour3d_gb300_set_slab_cells(C.c_uint64(10)) == 1  # below the minimum
    assert L.lib.contour3d_gb300_set_slab_cells(C.c_uint64(1 << 27)) == 0


def test_missing_library_fails_loudly(tmp_path):
    from contour3d_gb300 import lib
    with pytest.raises(lib.NativeLibraryMissing):
        lib.Library(str(tmp_path / "nope.so"))


def _sdecomp(L):
    from contour3d_gb300 import lib
    return lib.sdecomp_table(L)


def test_single_process_decomposition(built):
    from contour3d_gb300 import lib
    L = lib.Library()
    sd = _sdecomp(L)
    world = C.CFUNCTYPE(C.c_void_p)(C.cast(L.lib.c3d_comm_world, C.c_void_p).value)()
    construct = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(C.c_bool),
                            C.POINTER(C.c_void_p))(sd.construct)
    info = C.c_void_p()
    assert construct(world, 3, (C.c_size_t * 3)(0, 0, 0), (C.c_bool * 3)(True, True, True), C.byref(info)) == 0
    mysize = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_size_t, C.POINTER(C.c_size_t))(
        sd.get_pencil_mysize)
    offset = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_size_t, C.POINTER(C.c_size_t))(
        sd.get_pencil_offset)
    nb = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int))(sd.get_neighbours)
    for d, g in enumerate((13, 17, 19)):
        m, o = C.c_size_t(), C.c_size_t()
        assert mysize(info, 0, d, g, C.byref(m)) == 0 and m.value == g
        assert offset(info, 0, d, g, C.byref(o)) == 0 and o.value == 0
        n2 = (C.c_int * 2)()
        nb(info, 0, d, n2)
        assert list(n2) == [0, 0]  # periodic with one process: myself
    destruct = C.CFUNCTYPE(C.c_int, C.c_void_p)(sd.destruct)
    assert destruct(info) == 0


def test_execute_without_gpu_fails_loudly(built, tmp_path):
    """No usable GPU: contour3d_execute returns 1, logs a [CONTOUR3D ERROR]
    line and writes no file -- nothing falls back to the CPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible here")
    import sys
    out = tmp_path / "frame.ppm"
    script = (
        "import sys; sys.path.insert(0, %r)\n"
        "from contour3d_gb300 import lib\n"
        "from tests import cases\n"
        "L = lib.Library()\n"
        "rc = L.execute(cases.blobs_small(), %r)\n"
        "print('rc', rc)\n"
        "try:\n"
        "    L.render(cases.blobs_small())\n"
        "    print('render ok')\n"
        "except RuntimeError:\n"
        "    print('render raised')\n" % (ROOT, str(out)))
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "rc 1" in r.stdout and "render raised" in r.stdout
    assert "[CONTOUR3D ERROR]" in r.stderr
    assert not out.exists()


def _write_ppm(L, path, rgb, w, h):
    f = L.lib.c3d_write_ppm
    f.restype = C.c_int
    f.argtypes = [C.c_char_p, C.c_size_t, C.c_size_t, C.c_void_p]
    return f(str(path).encode(), w, h, rgb.ctypes.data)


def test_ppm_writer(built, tmp_path):
    """The ppm file of contour3d_execute (output.c:113-148): header and body
    as the reference writes them, whether the file is new, longer or shorter
    than the image (overwritten in place, then cut to size), or a device."""
    import numpy as np
    from contour3d_gb300 import lib
    L = lib.Library()
    w, h = 37, 23
    rgb = np.random.default_rng(3).integers(0, 256, (h, w, 3), dtype=np.uint8)
    want = b"P6\n37 23\n255\n" + rgb.tobytes()
    p = tmp_path / "a.ppm"
    assert _write_ppm(L, p, rgb, w, h) == 0 and p.read_bytes() == want
    p.write_bytes(b"x" * 100000)  # a longer file: cut to the image's size
    assert _write_ppm(L, p, rgb, w, h) == 0 and p.read_bytes() == want
    p.write_bytes(b"y" * 10)  # a shorter one
    assert _write_ppm(L, p, rgb, w, h) == 0 and p.read_bytes() == want
    assert _write_ppm(L, "/dev/null", rgb, w, h) == 0
    assert _write_ppm(L, tmp_path / "missing" / "b.ppm", rgb, w, h) == 1


def test_ppm_writer_matches_the_oracle_file(built, oracle, tmp_path):
    """The writer's file equals, byte for byte, the one the oracle's
    contour3d_execute writes (header layout and row order as output.c)."""
    from contour3d_gb300 import lib
    from tests import cases
    L = lib.Library()
    scene = cases.blobs_small()
    ref = tmp_path / "oracle.ppm"
    assert oracle.execute(scene, str(ref)) == 0
    img = oracle.render(scene)  # rows in ppm order
    h, w, _ = img.shape
    mine = tmp_path / "mine.ppm"
    assert _write_ppm(L, mine, img, w, h) == 0
    assert mine.read_bytes() == ref.read_bytes()
