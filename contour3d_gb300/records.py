"""Record layout of contour3d_gb300_debug_triangles (224 bytes per triangle)."""
import numpy as np

TRI_DTYPE = np.dtype([
    ("vertices", "<f8", (9,)),
    ("vertex_normals", "<f8", (9,)),
    ("face_normal", "<f8", (3,)),
    ("area", "<f8"),
    ("cell", "<i8", (3,)),
    ("edge_ids", "<i8", (3,)),
])
