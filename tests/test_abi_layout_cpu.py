"""The ctypes structures of the Python bindings against the C headers: a C
program compiled with include/contour3d.h and include/contour3d_gb300.h
prints sizeof and offsetof of every field, and each must equal the ctypes
layout.  A field added to one side and not the other fails here, on the CPU,
instead of as garbled arguments or statistics on the GPU."""
import ctypes as C
import json
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _structs():
    from contour3d_gb300 import _abi, lib
    from tests.test_multirank_cpu import Transport
    return {
        "contour3d_vector_t": _abi.Vector,
        "contour3d_color_t": _abi.Color,
        "contour3d_contour_obj_t": _abi.ContourObj,
        "contour3d_line_obj_t": _abi.LineObj,
        "contour3d_gb300_stats_t": lib.Stats,
        "contour3d_gb300_field_t": lib.Field,
        "contour3d_gb300_frame_t": lib.Frame,
        "contour3d_gb300_request_stats_t": lib.RequestStats,
        "contour3d_gb300_server_memory_t": lib.ServerMemory,
        "contour3d_gb300_transport_t": Transport,
    }


def test_ctypes_layouts_match_headers(built, tmp_path):
    structs = _structs()
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "contour3d.h"', '#include "contour3d_gb300.h"',
             "int main(void) {", '  printf("{");']
    first = True
    for cname, ct in structs.items():
        sep = "" if first else ","
        first = False
        lines.append(f'  printf("{sep}\\"{cname}\\": {{\\"@sizeof\\": %zu", sizeof({cname}));')
        for fname, *_ in ct._fields_:
            lines.append(f'  printf(", \\"{fname}\\": %zu", offsetof({cname}, {fname}));')
        lines.append('  printf("}");')
    lines += ['  printf("}\\n");', "  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    r = subprocess.run(["cc", "-std=c11", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = json.loads(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout)
    for cname, ct in structs.items():
        c = got[cname]
        assert c["@sizeof"] == C.sizeof(ct), (cname, c["@sizeof"], C.sizeof(ct))
        for fname, *_ in ct._fields_:
            assert c[fname] == getattr(ct, fname).offset, (cname, fname, c[fname], getattr(ct, fname).offset)
