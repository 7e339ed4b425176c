"""The error of FP32 field storage against FP64, stated per workload.

The library renders a float32 field as its exact widening to double, so its
result is the reference's FP64 arithmetic on the rounded values; what float32
storage changes is the input.  vertex_error() measures that change where it
first shows: the iso-surface vertices.  For every edge of the six-tetrahedra
split (the three axes, the three face diagonals and the body diagonal, each
from the cell's lower corner) and every level, an edge is crossed when
exactly one end satisfies threshold < value (src/contour3d/contour/triangulate.c:
95-131), and its vertex is interpolated as triangulate.c:40-73 does (the first
end when |v1 - v0| < 1e-8).  Edges crossed in both fields give the vertex
displacement; edges crossed in one field only change the topology locally and
are counted.  The computation runs in torch on the device (a measurement, not
part of the rendering path).
"""
from __future__ import annotations

import numpy as np

# edge directions of the six-tetrahedra split, from the cell's lower corner
DIRECTIONS = ((1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1), (1, 1, 1))


def vertex_error(f64, f32, levels, grids):
    """f64, f32: device tensors (nz, ny, nx) of the same field; levels: the
    thresholds; grids: (gx, gy, gz) node coordinates.  Returns the largest
    and RMS vertex displacement (absolute, and in units of the smallest node
    spacing), the edges compared and the edges crossed in one field only."""
    import torch
    dev = f64.device
    a64 = f64.double()
    a32 = f32.double()  # the exact widening the library reads
    nz, ny, nx = a64.shape
    g = [torch.as_tensor(np.asarray(x, dtype=np.float64), device=dev) for x in grids]
    h = min(float(np.min(np.diff(np.asarray(x, dtype=np.float64)))) for x in grids)
    worst = 0.0
    sq = 0.0
    n = 0
    differ = 0
    for thr in levels:
        for dx, dy, dz in DIRECTIONS:
            sl0 = (slice(0, nz - dz), slice(0, ny - dy), slice(0, nx - dx))
            sl1 = (slice(dz, nz), slice(dy, ny), slice(dx, nx))
            c64 = (thr < a64[sl0]) != (thr < a64[sl1])
            c32 = (thr < a32[sl0]) != (thr < a32[sl1])
            differ += int((c64 != c32).sum())
            both = c64 & c32
            m = int(both.sum())
            if m == 0:
                continue
            idx = both.nonzero(as_tuple=True)
            k, j, i = idx
            for arr, tag in ((a64, 64), (a32, 32)):
                v0 = arr[sl0][idx]
                v1 = arr[sl1][idx]
                dv = v1 - v0
                f = torch.where(dv.abs() < 1e-8, torch.zeros_like(dv), (thr - v0) / dv)
                pos = torch.stack([g[0][i] + f * (g[0][i + dx] - g[0][i]),
                                   g[1][j] + f * (g[1][j + dy] - g[1][j]),
                                   g[2][k] + f * (g[2][k + dz] - g[2][k])], dim=1)
                if tag == 64:
                    p64 = pos
                else:
                    p32 = pos
            d = (p64 - p32).abs().max(dim=1).values
            worst = max(worst, float(d.max()))
            sq += float((d * d).sum())
            n += m
            del p64, p32, d, idx
    rms = (sq / n) ** 0.5 if n else 0.0
    return {"edges_compared": n, "edges_crossed_in_one_field_only": differ, "max_abs": worst, "rms_abs": rms,
            "max_in_node_spacings": worst / h, "rms_in_node_spacings": rms / h, "node_spacing": h}


def image_difference(img_a, img_b):
    """Pixels whose colour differs between two (H*W*3) uint8 images, and the
    largest channel difference."""
    a = img_a.reshape(-1, 3).astype(np.int16)
    b = img_b.reshape(-1, 3).astype(np.int16)
    d = np.abs(a - b).max(axis=1)
    return {"pixels_differing": int((d > 0).sum()), "pixels": int(d.size), "max_channel_diff": int(d.max())}
