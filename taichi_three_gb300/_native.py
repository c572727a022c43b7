"""ctypes binding of libtina3.so (the C ABI in include/tina3.h).

The Structure classes mirror the C structs field for field; `check_layout()`
compares their sizes with the library's own sizeof() values.  Loading fails
loudly when the library is missing: there is no CPU fallback for the render
path.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libtina3.so")

# ---- constants (tina3.h) ----------------------------------------------------
T3_OK = 0
T3_EINVAL = -1
T3_ECUDA = -2
T3_EOVERFLOW = -3
T3_ETIMEOUT = -4
T3_ETOOBIG = -5
T3_EUNSUPPORTED = -6
ERRORS = {T3_EINVAL: "invalid argument", T3_ECUDA: "CUDA error", T3_EOVERFLOW: "capacity overflow",
          T3_ETIMEOUT: "device wait timed out", T3_ETOOBIG: "size exceeds a fixed maximum",
          T3_EUNSUPPORTED: "unsupported feature combination"}

T3_MAX_LIGHTS = 16
T3_MAX_NODES = 24
T3_MAX_OBJECTS = 8
T3_MAXDEPTH = 1 << 30
T3_NOALLOC_MAX_PIXELS = 1 << 21
T3_NOALLOC_MAX_BIG_FACES = 1 << 16

T3_CULLING, T3_CLIPPING, T3_SMOOTHING, T3_TEXTURING, T3_TONEMAP = 1, 2, 4, 8, 16
T3_WIRE_CLIPPING = 32
T3_SHADE_OWNED, T3_SHADE_EMPTY = 128, 256
T3_STARVE_BIN_COPY = 512
T3_STARVE_NETWORK = 1024
T3_MESH_SOUP, T3_MESH_GRID, T3_MESH_INDEXED, T3_MESH_PARTICLES, T3_MESH_LINES = 0, 1, 2, 3, 4
T3_MESH_TRANSFORM, T3_MESH_NOCULL, T3_MESH_FLIP_ORDER, T3_MESH_FLIP_NORMAL, T3_MESH_FLAT_NORMAL = \
    1, 2, 4, 8, 16
T3_MESH_WIREFRAME = 32
T3_MESH_QUADS = 64

T3_OP_CONST, T3_OP_ATTR, T3_OP_INPUT, T3_OP_FRESNEL, T3_OP_TEXTURE, T3_OP_CHECKER = 0, 1, 2, 3, 4, 5
T3_OP_LAMBERT, T3_OP_PHONG, T3_OP_COOK, T3_OP_EMISSION = 16, 17, 18, 19
T3_OP_MIX, T3_OP_SCALE, T3_OP_ADD = 32, 33, 34

T3_LIGHT_LAMPS, T3_LIGHT_IBL_MC, T3_LIGHT_IBL_MLP, T3_LIGHT_IBL_PREFILTERED = 0, 1, 2, 3
T3_MLP_IN, T3_MLP_HID, T3_MLP_OUT = 400, 64, 16
T3_STATUS_BIG_OVERFLOW, T3_STATUS_BIN_OVERFLOW, T3_STATUS_TIMEOUT = 1, 2, 4
T3_RASTER_DIRECT, T3_RASTER_BINNED = 0, 1


class t3_frame(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("flags", C.c_int32),
                ("maxdepth", C.c_int32), ("W2V", C.c_float * 16), ("V2W", C.c_float * 16),
                ("bias", C.c_float * 2), ("bgcolor", C.c_float * 3), ("linecolor", C.c_float * 3),
                ("wait_limit", C.c_int32), ("_pad", C.c_int32)]


class t3_mesh(C.Structure):
    _fields_ = [("kind", C.c_int32), ("flags", C.c_int32), ("nfaces", C.c_int64),
                ("verts", C.c_void_p), ("norms", C.c_void_p), ("coors", C.c_void_p),
                ("faces", C.c_void_p), ("face_stride", C.c_int32), ("corner_stride", C.c_int32),
                ("slot_vert", C.c_int32), ("slot_coor", C.c_int32), ("slot_norm", C.c_int32),
                ("grid_nx", C.c_int32), ("grid_ny", C.c_int32), ("attr_stride", C.c_int32),
                ("face_attr", C.c_void_p), ("trans", C.c_float * 16),
                ("trans_normal", C.c_float * 9), ("nverts", C.c_int32)]


class t3_node(C.Structure):
    _fields_ = [("op", C.c_int32), ("a", C.c_int32), ("b", C.c_int32), ("c", C.c_int32),
                ("v", C.c_float * 4)]


T3_MAX_TEXTURES = 4


class t3_texture(C.Structure):
    _fields_ = [("data", C.c_void_p), ("w", C.c_int32), ("h", C.c_int32), ("channels", C.c_int32),
                ("_pad", C.c_int32)]


class t3_material(C.Structure):
    _fields_ = [("nnodes", C.c_int32), ("root", C.c_int32), ("nodes", t3_node * T3_MAX_NODES),
                ("textures", t3_texture * T3_MAX_TEXTURES)]


class t3_object(C.Structure):
    _fields_ = [("mesh", t3_mesh), ("material", t3_material), ("face_base", C.c_int64),
                ("nfaces", C.c_int64)]


class t3_light(C.Structure):
    _fields_ = [("dir", C.c_float * 4), ("color", C.c_float * 4)]


T3_IBL_LEVELS = 7


class t3_ibl_map(C.Structure):
    _fields_ = [("data", C.c_void_p), ("w", C.c_int32), ("h", C.c_int32), ("half", C.c_int32),
                ("_pad", C.c_int32)]


class t3_ibl_tables(C.Structure):
    _fields_ = [("spec", t3_ibl_map * T3_IBL_LEVELS), ("diffuse", t3_ibl_map), ("lut", C.c_void_p),
                ("lut_w", C.c_int32), ("lut_h", C.c_int32)]


class t3_lighting(C.Structure):
    _fields_ = [("mode", C.c_int32), ("nlights", C.c_int32), ("ambient", C.c_float * 4),
                ("lights", t3_light * T3_MAX_LIGHTS), ("env", C.c_void_p), ("env_w", C.c_int32),
                ("env_h", C.c_int32), ("env_half", C.c_int32), ("spp", C.c_int32),
                ("seed", C.c_uint32), ("_pad", C.c_int32), ("mlp", C.c_void_p),
                ("tables", C.POINTER(t3_ibl_tables))]


class t3_scene(C.Structure):
    _fields_ = [("frame", t3_frame), ("lighting", t3_lighting), ("nobjects", C.c_int32),
                ("_pad", C.c_int32), ("objects", t3_object * T3_MAX_OBJECTS)]


class t3_outputs(C.Structure):
    _fields_ = [("rgb", C.c_void_p), ("face_id", C.c_void_p), ("depth", C.c_void_p),
                ("depth_f", C.c_void_p)]


class t3_batch_config(C.Structure):
    _fields_ = [("faces_per_item", C.c_int32), ("pixels_per_item", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("raster", C.c_int32), ("tile", C.c_int32), ("tile_threads", C.c_int32),
                ("bin_capacity", C.c_int64)]


T3_BATCH_MAX_SCENES = 64

STRUCTS = [t3_frame, t3_mesh, t3_node, t3_material, t3_object, t3_light, t3_lighting, t3_scene,
           t3_outputs]

# entry points: name -> (restype, argtypes)
_VP, _I32, _I64, _SZ = C.c_void_p, C.c_int32, C.c_int64, C.c_size_t
SIGNATURES = {
    "t3_version": (C.c_int, []),
    "t3_struct_sizes": (C.c_int, [C.POINTER(C.c_int64), C.c_int]),
    "t3_workspace_size": (C.c_int, [C.POINTER(t3_scene), C.c_int, C.c_int, _I64,
                                    C.POINTER(C.c_size_t)]),
    "t3_clear": (C.c_int, [_VP, _I64, _VP]),
    "t3_bin_capacity": (C.c_int, [C.POINTER(t3_scene), C.c_int, _I64, C.POINTER(C.c_int64)]),
    "t3_bin_counts_max": (C.c_int, [C.POINTER(t3_scene), C.c_int, _I64, _VP, _SZ,
                                    C.POINTER(C.c_int64), _VP]),
    "t3_raster": (C.c_int, [C.POINTER(t3_frame), C.POINTER(t3_object), _VP, _VP, _SZ, _VP, _VP]),
    "t3_shade": (C.c_int, [C.POINTER(t3_scene), _VP, _VP, _SZ, C.POINTER(t3_outputs), _VP]),
    "t3_render": (C.c_int, [C.POINTER(t3_scene), C.c_int, C.c_int, _I64, _VP, _SZ, _VP,
                            C.POINTER(t3_outputs), _VP]),
    "t3_read_status": (C.c_int, [_VP, C.POINTER(C.c_int32), _VP]),
    "t3_grid_normals": (C.c_int, [_VP, _VP, C.c_int, C.c_int, _VP]),
    "t3_smooth_normals_workspace_size": (C.c_int, [_I64, _I64, C.POINTER(_SZ)]),
    "t3_smooth_normals": (C.c_int, [C.POINTER(t3_mesh), _I64, _VP, _VP, _SZ, _VP]),
    "t3_tonemap": (C.c_int, [_VP, _I64, _VP]),
    "t3_grid_wave": (C.c_int, [_VP, C.c_int, C.c_int] + [C.c_float] * 6 + [_VP]),
    "t3_bloom_workspace_floats": (C.c_int64, [C.c_int, C.c_int]),
    "t3_bloom": (C.c_int, [_VP, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                           _VP, _I64, _VP]),
    "t3_fxaa_workspace_floats": (C.c_int64, [C.c_int, C.c_int]),
    "t3_fxaa": (C.c_int, [_VP, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, _VP, _I64, _VP]),
    "t3_accumulate": (C.c_int, [_VP, _VP, _I64, C.c_int, _VP]),
    "t3_render_staged": (C.c_int, [C.POINTER(t3_scene), C.c_int, C.c_int, _I64, _VP, _SZ, _VP,
                                   C.POINTER(t3_outputs), _VP, C.POINTER(C.c_void_p)]),
    "t3_render_staged_n": (C.c_int, [C.POINTER(t3_scene), C.c_int, C.c_int, _I64, _VP, _SZ, _VP,
                                     C.POINTER(t3_outputs), _VP, C.POINTER(C.c_void_p), C.c_int]),
    "t3_render_noalloc": (C.c_int, [C.POINTER(t3_scene), _VP, C.POINTER(t3_outputs), _VP]),
    "t3_raster_fragments": (C.c_int, [C.POINTER(t3_scene), _VP, _SZ, C.POINTER(C.c_int64), _VP]),
    "t3_red_min_rate": (C.c_int, [_VP, _I64, C.c_int, _VP]),
    "t3_batch_workspace_size": (C.c_int, [C.POINTER(t3_scene), C.c_int, C.POINTER(t3_batch_config),
                                          C.POINTER(C.c_size_t)]),
    "t3_render_batch": (C.c_int, [C.POINTER(t3_scene), C.POINTER(t3_outputs), C.c_int,
                                  C.POINTER(t3_batch_config), _VP, _SZ, _VP, _VP]),
    "t3_mlp_param_count": (C.c_int64, []),
    "t3_mlp_packed_bytes": (C.c_int64, []),
    "t3_mlp_irradiance_map": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.c_uint32, _VP, _VP]),
    "t3_mlp_targets": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, _VP, C.c_int, C.c_int, _VP, _VP,
                                 _I64, C.c_int, C.c_uint32, _VP, _VP]),
    "t3_mlp_encode": (C.c_int, [_VP, _VP, _VP, _I64, _VP, _VP]),
    "t3_mlp_forward": (C.c_int, [_VP, _VP, _I64, _VP, _VP, _VP]),
    "t3_mlp_backward": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _I64, _VP, _VP, _VP, _VP]),
    "t3_mlp_adam": (C.c_int, [_VP, _VP, _VP, _VP, _I64, C.c_float, C.c_float, C.c_float, C.c_float,
                              C.c_int, _VP]),
    "t3_mlp_pack": (C.c_int, [_VP, _VP, _VP]),
    "t3_mlp_infer": (C.c_int, [_VP, _VP, _I64, _VP, _VP, _VP]),
    "t3_mlp_infer_f32": (C.c_int, [_VP, _VP, _I64, _VP, _VP]),
    "t3_ibl_bake": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int, C.c_uint32, _VP,
                              C.c_int, C.c_int, _VP]),
    "t3_event_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "t3_event_destroy": (C.c_int, [_VP]),
    "t3_event_elapsed_ms": (C.c_int, [_VP, _VP, C.POINTER(C.c_float)]),
}

_lib = None


def load(path=LIB_PATH):
    """Loads libtina3.so (building it first when the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    from . import build as _build
    if _build.stale():
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"libtina3.so not found at {path}: run taichi_three_gb300/build.py")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    check_layout(lib)
    return lib


def check_layout(lib):
    n = lib.t3_struct_sizes(None, 0)
    buf = (C.c_int64 * n)()
    lib.t3_struct_sizes(buf, n)
    for cls, size in zip(STRUCTS, buf):
        if C.sizeof(cls) != size:
            raise RuntimeError(f"ABI layout mismatch for {cls.__name__}: "
                               f"python {C.sizeof(cls)} vs C {size}")


def check(rc, what):
    if rc != T3_OK:
        raise RuntimeError(f"{what} failed: {ERRORS.get(rc, rc)} ({rc})")


def new_workspace(nbytes, device):
    """A t3_render workspace: uninitialised except its first 16 bytes, the
    frame state t3_render keeps between frames, which start at zero."""
    import torch
    ws = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
    ws[:16].zero_()
    return ws
