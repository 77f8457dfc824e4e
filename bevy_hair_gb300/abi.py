"""ctypes bindings of ``include/hairgb.h`` and ``include/hairgb_bake.h``.

Struct layouts are numpy structured dtypes with the exact byte layout of the
reference's uniform and storage buffers (``src/render/pass.rs:42-78``,
``src/render/shaders/common.wgsl:10-54``).  Loading fails loudly when the
native library is missing: there is no Python or CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_DIR = Path(__file__).resolve().parent / "_lib"

LAYER_COUNT = 16
STYLE_TEXELS = 1024
DOM_LAYERS = 16
MAX_LIGHTS = 256
SCAN_NOALLOC_MAX_BUNDLES = 65536
MLP_PARAMS = 14608
MLP_COMPACT_PARAMS = 2128
MLP_COMPACT_OUTPUTS = 3
MLP_INPUTS = 10
MLP_OUTPUTS = 12
MLP_ARCH_DEEP, MLP_ARCH_COMPACT = 0, 1
SHADE_KARIS, SHADE_SURROGATE, SHADE_SURROGATE_MMA, SHADE_SURROGATE_COMPACT = 0, 1, 2, 3

# --------------------------------------------------------------------- dtypes

HAIR_PARAMS = np.dtype([
    ("clip_from_world", "<f4", 16),
    ("world_from_clip", "<f4", 16),
    ("world_from_model", "<f4", 16),
    ("light_clip_from_world", "<f4", 16),
    ("camera_pos", "<f4", 4),
    ("camera_forward", "<f4", 4),
    ("screen", "<f4", 4),
    ("appearance", "<f4", 4),
    ("filter_params", "<f4", 4),
    ("albedo", "<f4", 4),
    ("flags", "<u4", 4),
    ("pass_mode", "<u4", 4),
    ("light_eye", "<f4", 4),
    ("light_forward", "<f4", 4),
    ("dom_info", "<f4", 4),
])
assert HAIR_PARAMS.itemsize == 432

GPU_BUNDLE = np.dtype([("layer_offset", "<u4"), ("style_offset", "<u4"), ("strand_count", "<u4"), ("pad", "<u4")])
GPU_LAYER = np.dtype([("pos_ao", "<f4", 4), ("tangent", "<f4", 4)])
LOD_RECORD = np.dtype([("n_lod", "<u4"), ("control_points", "<u4"), ("strand_count", "<u4"), ("pad", "<u4")])
STRAND_REF = np.dtype([("bundle", "<u4"), ("strand", "<u4"), ("n_lod", "<u4"), ("control_points", "<u4")])
LIGHT = np.dtype([
    ("kind", "<u4"), ("flags", "<u4"), ("range", "<f4"), ("pad0", "<f4"),
    ("position", "<f4", 4), ("color", "<f4", 4), ("direction", "<f4", 4),
    ("spot", "<f4", 4), ("right", "<f4", 4), ("up", "<f4", 4),
])
assert LIGHT.itemsize == 112

SHADOW_LIGHT = np.dtype([("light_clip_from_world", "<f4", 16), ("light_eye", "<f4", 4), ("light_forward", "<f4", 4),
                         ("depth", "<f4", 4)])
assert SHADOW_LIGHT.itemsize == 112

LIGHT_POINT, LIGHT_SPOT, LIGHT_DIRECTIONAL, LIGHT_RECT = 0, 1, 2, 3
LIGHT_CASTS_SHADOWS = 1

SLOT_CAMERA, SLOT_DOM = 0, 1
CAMERA_RASTER_DIRECT, CAMERA_RASTER_BINNED = 0, 1
BUF_CENTER, BUF_CONSERVATIVE, BUF_BETA, BUF_DOM = 0, 1, 2, 3
BUF_SHADED, BUF_SHADED_DEPTH, BUF_FILTERED, BUF_FILTERED_DEPTH = 4, 5, 6, 7
BUF_COLOR, BUF_DEPTH = 8, 9
GBUF_LOD, GBUF_REFS, GBUF_INDIRECT, GBUF_STRAND_CACHE = 0, 1, 2, 3

STATUS = {
    0: "ok", 1: "invalid argument", 2: "out of device memory", 3: "CUDA error",
    4: "capacity exceeded", 5: "device timeout", 6: "not ready", 7: "device reported an error",
}
HG_OK, HG_INVALID_ARG, HG_OUT_OF_MEMORY, HG_CUDA_ERROR = 0, 1, 2, 3
HG_CAPACITY_EXCEEDED, HG_DEVICE_TIMEOUT, HG_NOT_READY, HG_DEVICE_ERROR = 4, 5, 6, 7


class HairGbError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class ShadeDesc(C.Structure):
    _fields_ = [
        ("lights", C.c_void_p),
        ("light_count", C.c_uint32),
        ("ortho", C.c_uint32),
        ("exposure", C.c_float),
        ("shade_model", C.c_uint32),
    ]


class FrameDesc(C.Structure):
    _fields_ = [
        ("camera", C.c_void_p),
        ("dom", C.c_void_p),
        ("scene_depth", C.c_void_p),
        ("shade", ShadeDesc),
        ("composite", C.c_uint32),
        ("clear_color", C.c_uint32),
    ]


class EnvDesc(C.Structure):
    _fields_ = [
        ("specular", C.c_void_p),
        ("specular_size", C.c_uint32),
        ("specular_levels", C.c_uint32),
        ("diffuse", C.c_void_p),
        ("diffuse_size", C.c_uint32),
        ("diffuse_levels", C.c_uint32),
        ("rotation", C.c_float * 4),
        ("intensity", C.c_float),
    ]


class ViewDesc(C.Structure):
    _fields_ = [
        ("world_from_view", C.c_float * 16),
        ("clip_from_view", C.c_float * 16),
        ("clip_from_world", C.c_float * 16),
        ("has_clip_from_world", C.c_uint32),
        ("width", C.c_uint32),
        ("height", C.c_uint32),
    ]


class GroomDesc(C.Structure):
    _fields_ = [
        ("world_from_model", C.c_float * 16),
        ("bounds_min", C.c_float * 3),
        ("bounds_max", C.c_float * 3),
        ("bundle_count", C.c_uint32),
        ("roughness", C.c_float),
        ("tilt", C.c_float),
        ("lambda_", C.c_float),
        ("center_diameter", C.c_float),
        ("albedo", C.c_float * 4),
        ("lod", C.c_uint32),
        ("filter", C.c_uint32),
        ("ambient_occlusion", C.c_uint32),
        ("deep_opacity", C.c_uint32),
    ]


DIRECTIONAL = np.dtype([("direction_to_light", "<f4", 3), ("casts_shadows", "<u4")])


class BatchItem(C.Structure):
    _fields_ = [
        ("groom", C.c_void_p),
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("dom_w", C.c_uint32),
        ("dom_h", C.c_uint32),
    ]


class BatchTuning(C.Structure):
    _fields_ = [
        ("raster_chunk", C.c_uint32),
        ("raster_blocks_per_sm", C.c_uint32),
        ("tile_w", C.c_uint32),
        ("tile_h", C.c_uint32),
        ("filter_tile", C.c_uint32),
        ("ms", C.c_float),
    ]

    def as_dict(self) -> dict:
        # ms unrounded: the tuner keeps the strictly fastest shape, and rounding
        # here would turn near ties into ties
        return {n: (float(getattr(self, n)) if n == "ms" else int(getattr(self, n))) for n, _ in self._fields_}


BATCH_GRAPH, BATCH_LAUNCHES, BATCH_SEPARATE = 0, 1, 2
BATCH_MAX_ITEMS = 128

# --------------------------------------------------------------------- loading

_LIB = None
_BAKE = None

_VP, _U32, _I32, _SZ, _F32 = C.c_void_p, C.c_uint32, C.c_int, C.c_size_t, C.c_float

_SIGNATURES = {
    "hg_abi_version": (_U32, []),
    "hg_status_string": (C.c_char_p, [_I32]),
    "hg_last_error": (C.c_char_p, [_VP]),
    "hg_create": (_I32, [_I32, _VP, C.POINTER(_VP)]),
    "hg_destroy": (_I32, [_VP]),
    "hg_synchronize": (_I32, [_VP, C.POINTER(_U32)]),
    "hg_ensure_targets": (_I32, [_VP, _U32, _U32, _U32, _U32]),
    "hg_buffer": (_I32, [_VP, _I32, C.POINTER(_VP), C.POINTER(_SZ)]),
    "hg_copy_out": (_I32, [_VP, _I32, _VP, _SZ]),
    "hg_copy_in": (_I32, [_VP, _I32, _VP, _SZ]),
    "hg_groom_upload": (_I32, [_VP, _VP, _U32, _VP, _U32, _VP, _U32, C.POINTER(_VP)]),
    "hg_groom_destroy": (_I32, [_VP, _VP]),
    "hg_groom_buffer": (_I32, [_VP, _VP, _I32, _I32, C.POINTER(_VP), C.POINTER(_SZ)]),
    "hg_groom_copy_out": (_I32, [_VP, _VP, _I32, _I32, _VP, _SZ]),
    "hg_clear": (_I32, [_VP]),
    "hg_clear_dom": (_I32, [_VP]),
    "hg_lod": (_I32, [_VP, _VP, _VP, _I32]),
    "hg_scan": (_I32, [_VP, _VP, _VP, _I32]),
    "hg_raster": (_I32, [_VP, _VP, _VP, _I32, _VP]),
    "hg_set_camera_raster": (_I32, [_VP, _U32]),
    "hg_generate": (_I32, [_VP, _VP, _VP]),
    "hg_shade": (_I32, [_VP, _VP, C.POINTER(ShadeDesc)]),
    "hg_filter": (_I32, [_VP, _VP]),
    "hg_composite": (_I32, [_VP, _VP, _U32]),
    "hg_clear_color": (_I32, [_VP, _F32]),
    "hg_groom_frame": (_I32, [_VP, _VP, C.POINTER(FrameDesc)]),
    "hg_scan_noalloc": (_I32, [_VP, _U32, _U32, _VP, _VP, _VP]),
    "hg_shadow_light_from": (_I32, [_VP, _VP]),
    "hg_groom_params": (_I32, [_VP, _VP, _VP, _U32, _U32, _U32, _VP, _VP]),
    "hg_copy_out_async": (_I32, [_VP, _I32, _VP, _SZ]),
    "hg_copy_wait": (_I32, [_VP]),
    "hg_batch_copy_out_async": (_I32, [_VP, _U32, _I32, _VP, _SZ]),
    "hg_hair_visibility": (_I32, [_VP, _VP, _VP, _U32, _VP]),
    "hg_mlp_create": (_I32, [_VP, C.POINTER(_VP)]),
    "hg_mlp_create_arch": (_I32, [_VP, _U32, C.POINTER(_VP)]),
    "hg_mlp_param_count": (_U32, [_VP]),
    "hg_mlp_output_count": (_U32, [_VP]),
    "hg_mlp_destroy": (None, [_VP]),
    "hg_mlp_set_params": (_I32, [_VP, _VP, _U32]),
    "hg_mlp_get_params": (_I32, [_VP, _VP, _U32]),
    "hg_mlp_samples": (_I32, [_VP, C.c_uint64, C.c_uint64, _U32, _F32, _VP, _VP, _VP]),
    "hg_mlp_infer": (_I32, [_VP, _VP, _U32, _VP, _VP]),
    "hg_mlp_infer_tc": (_I32, [_VP, _VP, _U32, _VP, _VP]),
    "hg_mlp_gradients": (_I32, [_VP, _VP, _VP, _U32, _VP, C.POINTER(_F32)]),
    "hg_mlp_train_step": (_I32, [_VP, _VP, _VP, _U32, _F32, _VP]),
    "hg_mlp_bind": (_I32, [_VP, _VP]),
    "hg_karis_lobes": (_I32, [_VP, _VP, _U32, _F32, _VP]),
    "hg_env_set": (_I32, [_VP, C.POINTER(EnvDesc)]),
    "hg_batch_create": (_I32, [_VP, _VP, _U32, C.POINTER(_VP)]),
    "hg_batch_destroy": (None, [_VP]),
    "hg_batch_set_params": (_I32, [_VP, _U32, _VP, _VP]),
    "hg_batch_frame": (_I32, [_VP, C.POINTER(ShadeDesc), _I32]),
    "hg_batch_launches": (_I32, [_VP, _I32, C.POINTER(_U32)]),
    "hg_batch_profile": (_I32, [_VP, C.POINTER(ShadeDesc), _VP]),
    "hg_batch_tune": (_I32, [_VP, C.POINTER(ShadeDesc), _VP, _U32, C.POINTER(_U32)]),
    "hg_batch_set_tuning": (_I32, [_VP, C.POINTER(BatchTuning)]),
    "hg_batch_get_tuning": (_I32, [_VP, C.POINTER(BatchTuning)]),
    "hg_batch_buffer": (_I32, [_VP, _U32, _I32, C.POINTER(_VP), C.POINTER(_SZ)]),
    "hg_batch_copy_out": (_I32, [_VP, _U32, _I32, _VP, _SZ]),
}

_BAKE_SIGNATURES = {
    "hg_bake": (_VP, [_VP, _U32, _VP, _VP, _U32, _U32]),
    "hg_bake_scalp": (_VP, [_VP, _U32, _VP, _VP, _U32, _VP, _U32, _VP, _U32, _U32]),
    "hg_bake_bundle_count": (_U32, [_VP]),
    "hg_bake_layer_count": (_U32, [_VP]),
    "hg_bake_style_count": (_U32, [_VP]),
    "hg_bake_copy": (None, [_VP, _VP, _VP, _VP, _VP]),
    "hg_bake_free": (None, [_VP]),
}


def _bind(lib: C.CDLL, sigs: dict) -> C.CDLL:
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def lib_path() -> Path:
    return LIB_DIR / "libhairgb.so"


def load() -> C.CDLL:
    """The CUDA pipeline library.  Raises when it has not been built."""
    global _LIB
    if _LIB is None:
        path = lib_path()
        if not path.exists():
            raise RuntimeError(
                f"{path} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
                "(there is no CPU fallback)")
        _LIB = _bind(C.CDLL(str(path)), _SIGNATURES)
    return _LIB


def load_bake() -> C.CDLL:
    global _BAKE
    if _BAKE is None:
        path = LIB_DIR / "libhairbake.so"
        if not path.exists():
            raise RuntimeError(f"{path} is missing: build it first (bevy_hair_gb300.build.build_bake)")
        _BAKE = _bind(C.CDLL(str(path)), _BAKE_SIGNATURES)
    return _BAKE


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def ptr(a: np.ndarray | None) -> int | None:
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays passed to the C ABI must be contiguous"
    return a.ctypes.data
