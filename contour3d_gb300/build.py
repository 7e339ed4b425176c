"""In-tree build of the native library (no cmake, no torch).

    python -m contour3d_gb300.build

compiles the CUDA and C++ sources for sm_103a into
contour3d_gb300/_build/libcontour3d_gb300.so, and the host-only field
generator into contour3d_gb300/_build/libc3d_fieldgen.so.  Translation units
compile in parallel; a unit is rebuilt when it or a header is newer than its
object file.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcontour3d_gb300.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false and -ffp-contract=off: no fused multiply-adds anywhere, the
# reference's arithmetic is unfused IEEE double.
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false",
                     "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
                     "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
             "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
CUDA_SOURCES = ["kernels.cu", "runtime.cu", "fieldgen.cu", "noalloc.cu"]
CXX_SOURCES = ["decomp.cpp"]


def _headers_mtime() -> float:
    hs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    return max(os.path.getmtime(h) for h in hs)


def _stale(src: str, obj: str, hdr: float) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or hdr > t


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _compile_and_link(out_dir: str, lib: str, extra_flags, link_extra, verbose: bool) -> None:
    os.makedirs(out_dir, exist_ok=True)
    hdr = _headers_mtime()
    jobs = []
    objs = []
    for s in CUDA_SOURCES:
        src, obj = os.path.join(CSRC, s), os.path.join(out_dir, s + ".o")
        objs.append(obj)
        if _stale(src, obj, hdr):
            jobs.append([NVCC] + list(extra_flags) + NVCC_FLAGS + ["-c", src, "-o", obj])
    for s in CXX_SOURCES:
        src, obj = os.path.join(CSRC, s), os.path.join(out_dir, s + ".o")
        objs.append(obj)
        if _stale(src, obj, hdr):
            jobs.append(["g++"] + list(extra_flags) + CXX_FLAGS + ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out:
                print(out)
    if jobs or not os.path.exists(lib):
        _run([NVCC] + ARCH + ["-shared", "-o", lib] + objs + list(link_extra) +
             ["-lcudart_static", "-lrt", "-lpthread", "-ldl"])


def _mpi_flags():
    """Compile and link flags of the MPI installation: $C3D_MPI_CFLAGS and
    $C3D_MPI_LIBS when set, else what `mpicxx --showme` reports."""
    cflags, libs = os.environ.get("C3D_MPI_CFLAGS"), os.environ.get("C3D_MPI_LIBS")
    if cflags is None or libs is None:
        try:
            c = subprocess.run(["mpicxx", "--showme:compile"], capture_output=True, text=True, check=True).stdout
            ln = subprocess.run(["mpicxx", "--showme:link"], capture_output=True, text=True, check=True).stdout
        except (OSError, subprocess.CalledProcessError):
            raise RuntimeError("MPI build: set C3D_MPI_CFLAGS and C3D_MPI_LIBS (no mpicxx found)")
        cflags = c if cflags is None else cflags
        libs = ln if libs is None else libs
    return cflags.split(), libs.split()


def build_mpi(out_dir: str = os.path.join(HERE, "_build_mpi"), external_sdecomp_include: str = None,
              cflags=None, libs=None, verbose: bool = False) -> str:
    """The library for callers that run under MPI: -DCONTOUR3D_USE_MPI, so the
    halo exchange and the depth reduction use the decomposition's MPI
    communicator instead of an installed transport.  With
    `external_sdecomp_include` (the directory of the real SimpleDecomp's
    sdecomp.h) the library also leaves out its own `sdecomp` table and binds
    the caller's (-DCONTOUR3D_EXTERNAL_SDECOMP).  The result is
    out_dir/libcontour3d_gb300_mpi.so; the default build is unchanged."""
    if cflags is None or libs is None:
        mc, ml = _mpi_flags()
        cflags = mc if cflags is None else cflags
        libs = ml if libs is None else libs
    flags = ["-DCONTOUR3D_USE_MPI"] + list(cflags)
    if external_sdecomp_include:
        # the caller's SimpleDecomp header is found before include/sdecomp.h
        flags = ["-DCONTOUR3D_EXTERNAL_SDECOMP", "-I" + external_sdecomp_include] + flags
    lib = os.path.join(out_dir, "libcontour3d_gb300_mpi.so")
    _compile_and_link(out_dir, lib, flags, list(libs), verbose)
    return lib


def build(verbose: bool = False) -> str:
    _compile_and_link(OUT, LIB, [], [], verbose)
    fg = os.path.join(OUT, "libc3d_fieldgen.so")
    src = os.path.join(CSRC, "fieldgen_cpu.c")
    if _stale(src, fg, _headers_mtime()):
        _run(["gcc", "-std=c99", "-O2", "-ffp-contract=off", "-fPIC", "-Wall", "-shared", "-o", fg, src, "-lm"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
