"""The library built for MPI callers, on CPU.

A flow solver that runs under MPI links the library built with
-DCONTOUR3D_USE_MPI: the halo exchange (src/contour3d/contour/extend.c:10-147)
and the nearest-depth reduction (src/contour3d/output.c:77-82) then go through
MPI_Sendrecv on the decomposition's communicator.  A solver that also links
the real SimpleDecomp adds -DCONTOUR3D_EXTERNAL_SDECOMP, and the library calls
the caller's `sdecomp` table instead of its own.

MPI is not installed here, so both builds are compiled against a two-process
MPI stand-in (tests/mpi_stub: a forked process pair over a socket), and a C
driver checks two ranks' extended blocks and the reduced pixels.  No GPU is
used: both functions are host code.
"""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STUB = os.path.join(ROOT, "tests", "mpi_stub")
INC = os.path.join(ROOT, "include")
CSRC = os.path.join(ROOT, "contour3d_gb300", "csrc")
WORK = os.path.join(ROOT, "contour3d_gb300", "_build", "mpi_stub")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, " ".join(cmd) + "\n" + r.stdout + r.stderr
    return r.stdout


def _stub_object():
    os.makedirs(WORK, exist_ok=True)
    obj = os.path.join(WORK, "mpi_stub.o")
    _run(["gcc", "-std=c99", "-O1", "-fPIC", "-Wall", "-I" + STUB, "-c", os.path.join(STUB, "mpi_stub.c"),
          "-o", obj])
    return obj


def _driver(extra, objs, out):
    src = os.path.join(STUB, "driver.c")
    obj = out + ".o"
    _run(["gcc", "-std=c99", "-D_DEFAULT_SOURCE", "-Wall", "-DCONTOUR3D_USE_MPI"] + extra +
         ["-I" + STUB, "-I" + INC, "-c", src, "-o", obj])
    _run(["g++", "-o", out, obj] + objs + ["-lpthread"])
    return out


def test_mpi_build_links_and_exchanges(built):
    """The whole library (CUDA units included) built with -DCONTOUR3D_USE_MPI
    links, and two ranks exchange halos and reduce pixels through it."""
    from contour3d_gb300 import build
    stub = _stub_object()
    lib = build.build_mpi(out_dir=os.path.join(WORK, "lib"), cflags=["-I" + STUB], libs=[stub])
    exe = _driver([], [lib, "-Wl,-rpath," + os.path.dirname(lib)], os.path.join(WORK, "driver_mpi"))
    out = _run([exe])
    assert "rank0 0 rank1 0" in out
    # built with MPI, the library has no transport to install
    nm = _run(["nm", "-D", "--defined-only", lib])
    assert " contour3d_execute" in nm and " sdecomp" in nm and "c3d_comm_world" not in nm


def test_external_simpledecomp_build(built, tmp_path):
    """-DCONTOUR3D_EXTERNAL_SDECOMP: the library compiles against the caller's
    SimpleDecomp header (a stand-in directory that comes first on the include
    path), defines no `sdecomp` table of its own, and drives the caller's."""
    stub = _stub_object()
    ext = tmp_path / "simpledecomp"
    ext.mkdir()
    # the stand-in for SimpleDecomp's header declares the interface the library binds
    (ext / "sdecomp.h").write_text(f'#include "{os.path.join(INC, "sdecomp.h")}"\n')
    flags = ["-DCONTOUR3D_EXTERNAL_SDECOMP", "-I" + str(ext), "-DCONTOUR3D_USE_MPI", "-I" + STUB, "-I" + INC,
             "-I" + CSRC]
    dobj = str(tmp_path / "decomp.o")
    _run(["g++", "-std=c++17", "-O1", "-fPIC", "-Wall", "-Wextra"] + flags +
         ["-c", os.path.join(CSRC, "decomp.cpp"), "-o", dobj])
    syms = _run(["nm", dobj])
    assert any(line.split()[-2:] == ["U", "sdecomp"] for line in syms.splitlines()), "sdecomp must be the caller's"
    # the runtime compiles in this configuration too
    _run([os.environ.get("NVCC", "nvcc"), "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17"] + flags +
         ["-c", os.path.join(CSRC, "runtime.cu"), "-o", str(tmp_path / "runtime.o")])
    exe = _driver(["-DEXTERNAL_TABLE", "-I" + str(ext)], [dobj, stub], str(tmp_path / "driver_ext"))
    assert "rank0 0 rank1 0" in _run([exe])


def test_external_sdecomp_needs_mpi(built, tmp_path):
    r = subprocess.run(["g++", "-std=c++17", "-DCONTOUR3D_EXTERNAL_SDECOMP", "-I" + INC, "-I" + CSRC, "-c",
                        os.path.join(CSRC, "decomp.cpp"), "-o", str(tmp_path / "x.o")],
                       capture_output=True, text=True)
    assert r.returncode != 0 and "needs -DCONTOUR3D_USE_MPI" in r.stderr

