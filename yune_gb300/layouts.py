"""numpy views of the buffer layouts in include/yune_types.h.

Each dtype is byte-for-byte the C struct (and Yune's include/CL_headers.h:57-107), so an
array of them is handed to the C-ABI as a plain pointer.
"""
import numpy as np

F4 = ("<f4", (4,))

TRIANGLE = np.dtype([("v1", *F4), ("v2", *F4), ("v3", *F4), ("vn1", *F4), ("vn2", *F4), ("vn3", *F4),
                     ("matID", "<i4"), ("pad", "<f4", (3,))], align=False)
AABB = np.dtype([("p_min", *F4), ("p_max", *F4)])
BVH_NODE = np.dtype([("p_min", *F4), ("p_max", *F4), ("vert_list", "<i4", (10,)), ("child_idx", "<i4"),
                     ("vert_len", "<i4")])
MATERIAL = np.dtype([("ke", *F4), ("kd", *F4), ("ks", *F4), ("n", "<f4"), ("k", "<f4"), ("px", "<f4"),
                     ("py", "<f4"), ("alpha_x", "<f4"), ("alpha_y", "<f4"), ("is_specular", "<i4"),
                     ("is_transmissive", "<i4")])
QUAD_LIGHT = np.dtype([("pos", *F4), ("normal", *F4), ("ke", *F4), ("kd", *F4), ("ks", *F4), ("edge_l", *F4),
                       ("edge_w", *F4), ("phong_exponent", "<f4"), ("pad", "<f4", (3,))])
CAM = np.dtype([("r1", *F4), ("r2", *F4), ("r3", *F4), ("r4", *F4), ("view_plane_dist", "<f4"),
                ("pad", "<f4", (3,))])

assert TRIANGLE.itemsize == 112 and BVH_NODE.itemsize == 80 and MATERIAL.itemsize == 80
assert QUAD_LIGHT.itemsize == 128 and CAM.itemsize == 80 and AABB.itemsize == 32


def ptr(a):
    """Address of a C-contiguous numpy array (or None) for a void* argument."""
    if a is None:
        return None
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data
