"""Generate the golden fixtures from the reference library itself.

Runs the reference's own sources, compiled into oracle/_ref/ with single-rank
MPI/SimpleDecomp shims (oracle/Makefile target `ref`), on the seeded cases of
tests/cases.py, and stores what the reference produced:
  <case>.npz      ppm body and every rendered triangle record
  manifest.json   sha256 of the generated input fields, of each case's ppm
                  and, for the 128^3 / 1024^2 configuration, of its ppm
Needs the reference tree (only present where the fixtures are made):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from contour3d_gb300 import fields  # noqa: E402
from oracle import lib as olib  # noqa: E402
from tests import cases  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def field_hashes():
    out = {}
    out["blobs_128_seed0"] = sha(fields.blobs((128, 128, 128), nblobs=8, seed=0).tobytes())
    f, std = fields.modes((40, 36, 48), nmodes=64, kmin=1, kmax=16, power=5.0 / 6.0, seed=1)
    out["modes_48x36x40_seed1_f64"] = sha(f.tobytes())
    out["modes_seed1_std"] = repr(std)
    g, _ = fields.modes((40, 36, 48), nmodes=64, kmin=1, kmax=16, power=5.0 / 6.0, seed=1,
                        dtype=np.float32)
    out["modes_48x36x40_seed1_f32"] = sha(g.tobytes())
    return out


def main():
    olib.build(with_reference=True)
    ref = olib.Reference()
    manifest = {"fields": field_hashes(), "cases": {}}
    with tempfile.TemporaryDirectory() as tmp:
        for name, fn in cases.SMALL_CASES.items():
            scene = fn()
            img = ref.render(scene, tmp)
            tris = []
            ntri = []
            for c in scene.contours:
                t, n = ref.triangles(c)
                tris.append(t)
                ntri.append(n)
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), rgb=img,
                                triangles=np.concatenate(tris) if tris else np.zeros(0),
                                per_object=np.array([len(t) for t in tris], dtype=np.int64),
                                triangulated=np.array(ntri, dtype=np.int64))
            manifest["cases"][name] = {"ppm_sha256": sha(img.tobytes()),
                                       "rendered": [len(t) for t in tris], "triangulated": ntri}
            print(name, [len(t) for t in tris], ntri)
        s0 = cases.config0()
        img0 = ref.render(s0, tmp)
        t0, n0 = ref.triangles(s0.contours[0])
        manifest["config0"] = {"ppm_sha256": sha(img0.tobytes()), "rendered": len(t0),
                               "triangulated": n0,
                               "vertex_sha256": sha(np.ascontiguousarray(t0["vertices"]).tobytes()),
                               "normal_sha256": sha(np.ascontiguousarray(t0["vertex_normals"]).tobytes())}
        print("config0", len(t0), n0)
    with open(os.path.join(HERE, "manifest.json"), "w") as fp:
        json.dump(manifest, fp, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
