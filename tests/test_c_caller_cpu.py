"""A C caller of the drop-in boundary: a program that includes only the
reference's headers (contour3d.h, sdecomp.h), builds a decomposition and one
contour object the way src/main.c:310-326 does, calls contour3d_execute, and
is linked against libcontour3d_gb300 with the command line of the
integration notes.  Without a GPU the call must return 1 and log a
[CONTOUR3D ERROR] line (no CPU fallback)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CALLER = r"""
#include <stdio.h>
#include <stdlib.h>
#include "contour3d.h"
#include "sdecomp.h"

int main(void) {
  const size_t n[3] = {9, 8, 7};
  double *grid[3];
  for (int d = 0; d < 3; d++) {
    grid[d] = malloc(n[d] * sizeof(double));
    for (size_t i = 0; i < n[d]; i++) grid[d][i] = (double)i / (double)(n[d] - 1);
  }
  double *field = malloc(n[0] * n[1] * n[2] * sizeof(double));
  for (size_t q = 0; q < n[0] * n[1] * n[2]; q++) field[q] = (double)(q % 7) / 7.0;
  sdecomp_info_t *info = NULL;
  if (sdecomp.construct(MPI_COMM_WORLD, 3, (size_t[3]){0, 0, 0}, (bool[3]){false, false, false}, &info)) return 10;
  contour3d_contour_obj_t obj = {0};
  obj.pencil = SDECOMP_X1PENCIL;
  for (int d = 0; d < 3; d++) {
    obj.glsizes[d] = n[d];
    obj.grids[d] = grid[d];
  }
  obj.converter = NULL;
  obj.threshold = 0.5;
  obj.color = (contour3d_color_t){255, 0, 0};
  obj.array = field;
  const contour3d_vector_t camera = {2.5, 2.0, 1.5}, look_at = {0.5, 0.5, 0.5}, light = {0.0, 2.0, -1.0};
  const contour3d_vector_t center = {1.5, 1.25, 1.0};
  const contour3d_vector_t local[2] = {{0.4, -0.5, 0.0}, {-0.1, -0.1, 0.3}};
  const size_t sizes[2] = {32, 24};
  const contour3d_color_t bg = {0, 0, 0};
  const int rc = contour3d_execute(info, &camera, &look_at, &light, sizes, &center, local, &bg, 1, &obj, 0, NULL,
                                   OUT_PATH);
  sdecomp.destruct(info);
  printf("rc %d\n", rc);
  return 0;
}
"""


def test_c_caller_links_and_fails_loudly_without_gpu(built, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible here")
    src = tmp_path / "caller.c"
    src.write_text(CALLER)
    exe = tmp_path / "caller"
    out = tmp_path / "frame.ppm"
    libdir = os.path.join(ROOT, "contour3d_gb300", "_build")
    cmd = ["cc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"),
           f'-DOUT_PATH="{out}"', str(src), "-o", str(exe), "-L" + libdir, "-lcontour3d_gb300",
           "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "rc 1" in r.stdout
    assert "[CONTOUR3D ERROR]" in r.stderr
    assert not out.exists()
