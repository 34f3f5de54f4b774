"""ctypes binding of the C ABI declared in include/splotch_gb300.h.

Loads the in-tree ``libsplgpu.so``.  There is no fallback: if the library is
missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

SPL_MAX_TYPES = 8
SPL_OK, SPL_ERR_INVALID, SPL_ERR_CUDA, SPL_ERR_ALLOC, SPL_ERR_CAPACITY, SPL_ERR_TIMEOUT, \
    SPL_ERR_UNSUPPORTED, SPL_ERR_INTERNAL = range(8)
SPL_MEM_HOST, SPL_MEM_DEVICE = 0, 1
SPL_LAYOUT_AOS, SPL_LAYOUT_SOA = 0, 1
SPL_WRITEBACK_NONE, SPL_WRITEBACK_FULL = 0, 1
SPL_ORDER_BACK_TO_FRONT, SPL_ORDER_FRONT_TO_BACK = 0, 1
SPL_SPLIT_OFF, SPL_SPLIT_ON, SPL_SPLIT_ADDITIVE = 0, 1, 2

LIB_PATH = Path(__file__).resolve().parent / "libsplgpu.so"

# Every symbol include/splotch_gb300.h declares (checked by the CPU tests).
EXPORTED = [
    "spl_context_create", "spl_context_destroy", "spl_context_set_stream",
    "spl_last_error_string", "spl_version", "spl_frame_desc_defaults", "spl_camera_setup",
    "spl_render", "spl_get_stats", "spl_debug_get_projected", "spl_debug_get_order",
    "spl_debug_get_bins", "spl_debug_count_fragments", "spl_debug_set_options",
    "spl_splat_config_count", "spl_splat_config_valid", "spl_sort_pairs_noalloc",
    "spl_prefetch", "spl_context_set_split_tiles",
    "spl_render_backward", "spl_context_set_differentiable", "spl_batch_options_defaults",
    "spl_batch_create", "spl_batch_render", "spl_batch_get_info", "spl_batch_destroy",
    "spl_post_desc_defaults", "spl_postprocess", "spl_image_encode", "spl_write_image",
    "spl_particle_normalize", "spl_rays_desc_defaults", "spl_render_rays",
    "spl_debug_fail_alloc",
]
SPL_NOALLOC_MAX_PAIRS = 1 << 21
SPL_DEBUG_EXACT_FP64 = 1
SPL_DEBUG_RADIX_REDUCE_SCAN = 2
SPL_DEBUG_LOOKBACK_STALL = 4
SPL_DEBUG_SHORT_COUNT = 16


class Camera(C.Structure):
    _fields_ = [("mat", C.c_float * 12), ("res2", C.c_float), ("ycorr", C.c_float),
                ("fovfct", C.c_float), ("xfac", C.c_float), ("xshift", C.c_double),
                ("yshift", C.c_double)]


class FrameDesc(C.Structure):
    _fields_ = [
        ("xres", C.c_int), ("yres", C.c_int), ("fov", C.c_float), ("zmin", C.c_float),
        ("zmax", C.c_float), ("minrad_pix", C.c_float), ("projection", C.c_int),
        ("ptypes", C.c_int), ("smooth_factor", C.c_float * SPL_MAX_TYPES),
        ("brightness", C.c_float * SPL_MAX_TYPES),
        ("color_is_vector", C.c_int * SPL_MAX_TYPES), ("b_brightness", C.c_float),
        ("pal_n", C.c_int * SPL_MAX_TYPES), ("pal_x", C.c_void_p * SPL_MAX_TYPES),
        ("pal_rgb", C.c_void_p * SPL_MAX_TYPES), ("a_eq_e", C.c_int),
        ("gray_absorption", C.c_float), ("sort_type", C.c_int), ("tile_size", C.c_int),
        ("campos", C.c_double * 3), ("lookat", C.c_double * 3), ("sky", C.c_double * 3),
        ("centerpos", C.c_double * 3), ("order_mode", C.c_int), ("ftb_epsilon", C.c_float),
        ("splat_config", C.c_int), ("ftb_relative", C.c_float),
    ]


class Particles(C.Structure):
    _fields_ = [("n", C.c_int64), ("layout", C.c_int), ("memspace", C.c_int),
                ("aos", C.c_void_p), ("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p),
                ("r", C.c_void_p), ("I", C.c_void_p), ("cr", C.c_void_p), ("cg", C.c_void_p),
                ("cb", C.c_void_p), ("type", C.c_void_p)]


class Image(C.Structure):
    _fields_ = [("pic", C.c_void_p), ("memspace", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("h2d_ms", C.c_float), ("project_ms", C.c_float), ("sort_ms", C.c_float),
                ("bin_ms", C.c_float), ("splat_ms", C.c_float), ("d2h_ms", C.c_float),
                ("total_ms", C.c_float), ("n_active", C.c_int64), ("n_entries", C.c_int64),
                ("n_tiles", C.c_int64), ("kernel_launches", C.c_int),
                ("n_fallback", C.c_int64), ("n_wide", C.c_int64),
                ("bwd_splat_ms", C.c_float), ("bwd_project_ms", C.c_float),
                ("bwd_total_ms", C.c_float)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


GRAD_FIELDS = ("I", "cr", "cg", "cb", "x", "y", "z", "r")


class Grads(C.Structure):
    _fields_ = [("memspace", C.c_int)] + [(f, C.c_void_p) for f in GRAD_FIELDS] + [
        ("campos", C.c_double * 3)]


class NormalizeDesc(C.Structure):
    _fields_ = [("ptypes", C.c_int)] + [
        (k, C.c_int * SPL_MAX_TYPES) for k in (
            "intensity_log", "color_log", "color_asinh", "color_is_vector",
            "has_intensity_min", "has_intensity_max", "has_color_min", "has_color_max")] + [
        (k, C.c_float * SPL_MAX_TYPES) for k in (
            "intensity_min", "intensity_max", "color_min", "color_max")]


class NormalizeResult(C.Structure):
    _fields_ = [(k, C.c_float * SPL_MAX_TYPES) for k in (
        "range_min", "range_max", "clamp_min", "clamp_max", "intensity_min", "intensity_max",
        "size_min", "size_max")]


class PostDesc(C.Structure):
    _fields_ = [("a_eq_e", C.c_int), ("gamma", C.c_double), ("brightness", C.c_double),
                ("contrast", C.c_double), ("colorbar", C.c_int)]


class BatchFrame(C.Structure):
    _fields_ = [("set", C.c_int), ("desc", FrameDesc), ("pic", C.c_void_p)]


class BatchOptions(C.Structure):
    _fields_ = [("tile_size", C.c_int), ("splat_config_additive", C.c_int),
                ("splat_config_absorption", C.c_int), ("capacity_margin", C.c_float),
                ("use_graph", C.c_int), ("tune_cache", C.c_int)]


class BatchInfo(C.Structure):
    _fields_ = [("tile_size", C.c_int), ("splat_config_additive", C.c_int),
                ("splat_config_absorption", C.c_int), ("graph", C.c_int),
                ("cap_active", C.c_int64), ("cap_entries", C.c_int64),
                ("total_tiles", C.c_int64), ("n_active", C.c_int64), ("n_entries", C.c_int64),
                ("render_ms", C.c_float), ("tune_ms", C.c_float), ("kernel_launches", C.c_int),
                ("replans", C.c_int), ("tune_cached", C.c_int), ("plan_ms", C.c_float)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class RaysDesc(C.Structure):
    """spl_rays_desc: the ray-sphere renderer's own keys."""
    _fields_ = [("dome", C.c_int), ("fov", C.c_double), ("minrad_pix", C.c_double)]


class SplotchError(RuntimeError):
    """A non-zero spl_status; the message is spl_last_error_string()."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"spl_status {code}: {msg}")
        self.code = code


_lib = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Load libsplgpu.so (once).  Raises if it is absent: no CPU fallback."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is not built; run splotch_gb300.build.build() first")
    lib = C.CDLL(str(p))
    vp, i64 = C.c_void_p, C.c_int64
    sig = {
        "spl_context_create": (C.c_int, [C.POINTER(vp), C.c_int]),
        "spl_context_destroy": (C.c_int, [vp]),
        "spl_context_set_stream": (C.c_int, [vp, vp]),
        "spl_last_error_string": (C.c_char_p, []),
        "spl_version": (C.c_char_p, []),
        "spl_frame_desc_defaults": (None, [C.POINTER(FrameDesc)]),
        "spl_camera_setup": (C.c_int, [C.POINTER(FrameDesc), C.POINTER(Camera)]),
        "spl_render": (C.c_int, [vp, C.POINTER(FrameDesc), C.POINTER(Particles),
                                 C.POINTER(Image), C.c_int]),
        "spl_get_stats": (C.c_int, [vp, C.POINTER(Stats)]),
        "spl_debug_get_projected": (C.c_int, [vp, vp, i64]),
        "spl_debug_get_order": (C.c_int, [vp, vp, i64, vp]),
        "spl_debug_get_bins": (C.c_int, [vp, vp, i64, vp, i64]),
        "spl_debug_count_fragments": (C.c_int, [vp, vp]),
        "spl_debug_set_options": (C.c_int, [vp, C.c_int]),
        "spl_debug_fail_alloc": (C.c_int, [i64]),
        "spl_splat_config_count": (C.c_int, []),
        "spl_splat_config_valid": (C.c_int, [C.c_int, C.c_int]),
        "spl_sort_pairs_noalloc": (C.c_int, [vp, vp, vp, vp, i64, C.c_int, vp]),
        "spl_prefetch": (C.c_int, [vp, C.POINTER(Particles)]),
        "spl_context_set_split_tiles": (C.c_int, [vp, C.c_int]),
        "spl_render_backward": (C.c_int, [vp, C.POINTER(Image), C.POINTER(Grads)]),
        "spl_context_set_differentiable": (C.c_int, [vp, C.c_int]),
        "spl_batch_options_defaults": (None, [C.POINTER(BatchOptions)]),
        "spl_batch_create": (C.c_int, [vp, vp, C.c_int, vp, C.c_int,
                                       C.POINTER(BatchOptions), C.POINTER(vp)]),
        "spl_batch_render": (C.c_int, [vp]),
        "spl_batch_get_info": (C.c_int, [vp, C.POINTER(BatchInfo)]),
        "spl_batch_destroy": (C.c_int, [vp]),
        "spl_particle_normalize": (C.c_int, [vp, C.POINTER(NormalizeDesc), C.POINTER(Particles),
                                             C.POINTER(NormalizeResult)]),
        "spl_rays_desc_defaults": (None, [C.POINTER(RaysDesc)]),
        "spl_render_rays": (C.c_int, [vp, C.POINTER(FrameDesc), C.POINTER(RaysDesc),
                                      C.POINTER(Particles), C.POINTER(Image)]),
        "spl_post_desc_defaults": (None, [C.POINTER(PostDesc)]),
        "spl_postprocess": (C.c_int, [vp, C.POINTER(FrameDesc), C.POINTER(PostDesc),
                                      C.POINTER(Image)]),
        "spl_image_encode": (C.c_int, [vp, C.POINTER(Image), C.c_int, C.c_int, C.c_int, vp,
                                       i64, C.POINTER(i64)]),
        "spl_write_image": (C.c_int, [vp, C.POINTER(Image), C.c_int, C.c_int, C.c_int,
                                      C.c_char_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(code: int) -> None:
    if code != SPL_OK:
        msg = load().spl_last_error_string()
        raise SplotchError(code, msg.decode() if msg else "")


def ptr(a) -> int | None:
    """Address of a numpy array or torch tensor (None for None)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return int(a.data_ptr())
