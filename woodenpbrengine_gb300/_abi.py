"""ctypes mirrors of the plain-C structures in include/wpbr_scene.h and
include/wpbr_record.h (the library's ABI; layouts must match byte for byte)."""
import ctypes as C

import numpy as np


class Mat4(C.Structure):
    _fields_ = [("m", C.c_float * 16)]


class Material(C.Structure):
    _fields_ = [
        ("type", C.c_uint32),
        ("alpha_x", C.c_float),
        ("alpha_y", C.c_float),
        ("R", C.c_float * 3),
        ("eta_i", C.c_float * 3),
        ("eta_t", C.c_float * 3),
        ("k", C.c_float * 3),
        ("tex", C.c_uint16 * 2),
    ]


class Sphere(C.Structure):
    _fields_ = [
        ("object_to_world", Mat4),
        ("world_to_object", Mat4),
        ("radius", C.c_float),
        ("material", C.c_uint32),
        ("pad", C.c_uint32 * 2),
    ]


class Mesh(C.Structure):
    _fields_ = [("tri_begin", C.c_uint32), ("tri_count", C.c_uint32), ("material", C.c_uint32), ("flags", C.c_uint32)]


class Light(C.Structure):
    _fields_ = [("type", C.c_uint32), ("sphere_index", C.c_uint32), ("Le", C.c_float * 3)]


class EnvMap(C.Structure):
    _fields_ = [
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("rgb", C.POINTER(C.c_float)),
        ("light_to_world", Mat4),
        ("world_to_light", Mat4),
    ]


class Camera(C.Structure):
    _fields_ = [
        ("camera_to_world", Mat4),
        ("world_to_camera", Mat4),
        ("fov_deg", C.c_float),
        ("near_z", C.c_float),
        ("far_z", C.c_float),
        ("screen", C.c_float * 4),
        ("res_x", C.c_uint32),
        ("res_y", C.c_uint32),
    ]


class Texture(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("rgb", C.POINTER(C.c_float))]


class SceneDesc(C.Structure):
    _fields_ = [
        ("spheres", C.POINTER(Sphere)),
        ("n_spheres", C.c_uint32),
        ("n_vertices", C.c_uint32),
        ("positions", C.POINTER(C.c_float)),
        ("normals", C.POINTER(C.c_float)),
        ("tangents", C.POINTER(C.c_float)),
        ("uvs", C.POINTER(C.c_float)),
        ("n_triangles", C.c_uint32),
        ("indices", C.POINTER(C.c_uint32)),
        ("meshes", C.POINTER(Mesh)),
        ("n_meshes", C.c_uint32),
        ("materials", C.POINTER(Material)),
        ("n_materials", C.c_uint32),
        ("lights", C.POINTER(Light)),
        ("n_lights", C.c_uint32),
        ("envmap", C.POINTER(EnvMap)),
        ("camera", Camera),
        ("textures", C.POINTER(Texture)),
        ("n_textures", C.c_uint32),
    ]


RECORD_FIELDS = [
    ("pfilm", "f", 2), ("ray_o", "f", 3), ("ray_d", "f", 3), ("ray_dx_d", "f", 3), ("ray_dy_d", "f", 3),
    ("hit_prim", "u", 1), ("hit_t", "f", 1),
    ("si_p", "f", 3), ("si_n", "f", 3), ("si_wo", "f", 3), ("si_sn", "f", 3), ("si_sdpdu", "f", 3),
    ("si_dpdu", "f", 3), ("si_dpdv", "f", 3), ("si_dndu", "f", 3), ("si_dndv", "f", 3),
    ("frame", "f", 9), ("le", "f", 3), ("light_idx", "u", 1),
    ("l_wi", "f", 3), ("l_li", "f", 3), ("l_pdf", "f", 1), ("l_flags", "u", 1), ("l_f", "f", 3), ("l_fpdf", "f", 1),
    ("b_wi", "f", 3), ("b_f", "f", 3), ("b_pdf", "f", 1), ("b_flags", "u", 1), ("b_li", "f", 3), ("b_lpdf", "f", 1),
    ("L", "f", 3),
]


class PassRecord(C.Structure):
    _fields_ = [(name, C.POINTER(C.c_float) if kind == "f" else C.POINTER(C.c_uint32)) for name, kind, _ in RECORD_FIELDS]


def make_record(n, fields=None, fill=np.nan):
    """Allocate numpy arrays for a pass record of n pixels; returns (struct, dict).

    Float fields start as NaN and integer fields as 0xFFFFFFFF, so a stage a
    pixel never reaches is visible as untouched on both sides."""
    rec = PassRecord()
    arrays = {}
    for name, kind, width in RECORD_FIELDS:
        if fields is not None and name not in fields:
            continue
        if kind == "f":
            a = np.full(n * width, fill, dtype=np.float32)
            setattr(rec, name, a.ctypes.data_as(C.POINTER(C.c_float)))
        else:
            a = np.full(n * width, 0xFFFFFFFF, dtype=np.uint32)
            setattr(rec, name, a.ctypes.data_as(C.POINTER(C.c_uint32)))
        arrays[name] = a.reshape(n, width) if width > 1 else a
    return rec, arrays


def fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None


def uptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32)) if a is not None else None


class BatchInfo(C.Structure):
    _fields_ = [
        ("n_scenes", C.c_uint32), ("spp", C.c_uint32), ("total_pixels", C.c_uint64), ("total_prims", C.c_uint64),
        ("arena_bytes", C.c_uint64), ("rays_per_block", C.c_uint32), ("autotune_source", C.c_uint32),
    ]
