"""splotch_gb300 -- GB300-native particle renderer behind Splotch's host_rendering().

Host-side mirror of the reference interface, on top of the C ABI
(include/splotch_gb300.h, libsplgpu.so):

* ``PARTICLE_DTYPE``  -- the 36-byte ``particle_sim`` record
  (splotch/splotchutils.h:52-72).
* ``ParamFile``       -- ``paramfile`` semantics: ``find(key, default)`` converts
  like ``stringToData`` and inserts the default (cxxsupport/paramfile.cc:96-103).
* ``Palette``, ``load_palette``, ``get_colourmaps`` -- ``linearMap<COLOUR>`` knots
  as built by ``get_colourmaps`` (splotch/splotchutils.cc:63-125).
* ``RenderContext``   -- ``render_context`` (splotch/splotchutils.h:98-122).
* ``host_rendering(params, particles, rc)`` -- the drop-in for
  ``host_rendering`` (splotch/splotch_host.cc:711-834): same keys, same
  defaults, same in-place side effects on ``particles`` and ``rc.pic``.

Everything runs through the CUDA path; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import math
import re
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _abi
from ._abi import SplotchError  # noqa: F401

__all__ = [
    "PARTICLE_DTYPE", "ParamFile", "Palette", "load_palette", "get_colourmaps",
    "RenderContext", "update_res", "frame_desc", "Renderer", "host_rendering",
    "SplotchError", "make_particles",
]

PARTICLE_DTYPE = np.dtype({
    "names": ["er", "eg", "eb", "x", "y", "z", "r", "I", "type", "active", "pad"],
    "formats": ["<f4"] * 8 + ["<u2", "u1", "u1"],
    "offsets": [0, 4, 8, 12, 16, 20, 24, 28, 32, 34, 35],
    "itemsize": 36,
})


def make_particles(n: int) -> np.ndarray:
    """Zero-initialised particle_sim array."""
    return np.zeros(n, dtype=PARTICLE_DTYPE)


# ---------------------------------------------------------------------------
# paramfile


class ParamFile:
    """``paramfile`` (cxxsupport/paramfile.{h,cc}).

    ``find(key, default)`` converts the stored string like ``stringToData``
    (cxxsupport/string_utils.cc:109-140) and, when the key is absent, stores the
    default -- the reference's side effect that later readers rely on.
    ``find(key)`` without a default raises ``KeyError`` for a missing key.
    """

    _NODEF = object()

    def __init__(self, source: dict | str | Path | None = None):
        self.params: dict[str, str] = {}
        self.read: set[str] = set()
        if isinstance(source, dict):
            self.params = {str(k): self._to_str(v) for k, v in source.items()}
        elif source is not None:
            self.params = _parse_file(Path(source))

    @staticmethod
    def _to_str(v) -> str:
        if isinstance(v, bool):
            return "T" if v else "F"
        if isinstance(v, float):
            return repr(v)
        return str(v).strip()

    @staticmethod
    def _convert(s: str, typ):
        s = s.strip()
        if typ is bool:
            low = s.lower()
            if low in ("f", "n", "false", ".false."):
                return False
            if low in ("t", "y", "true", ".true."):
                return True
            raise ValueError(f'conversion error in stringToData<bool>("{s}")')
        if typ is int:
            if not re.fullmatch(r"[+-]?\d+", s):
                raise ValueError(f'conversion error in stringToData<int>("{s}")')
            return int(s)
        if typ is float:
            return float(s)
        return s

    def find(self, key: str, default=_NODEF, typ=None):
        if typ is None:
            typ = type(default) if default is not self._NODEF else str
        if key in self.params:
            self.read.add(key)
            return self._convert(self.params[key], typ)
        if default is self._NODEF:
            raise KeyError(f"Cannot find the key '{key}'.")
        self.params[key] = self._to_str(default)
        self.read.add(key)
        return default

    def param_present(self, key: str) -> bool:
        return key in self.params

    def set_param(self, key: str, value) -> None:
        self.params[key] = self._to_str(value)


def _parse_file(path: Path) -> dict[str, str]:
    """key=value lines, '#' comments (cxxsupport/string_utils.cc parse_file)."""
    out = {}
    for line in path.read_text().splitlines():
        line = line.split("#", 1)[0].strip()
        if not line or "=" not in line:
            continue
        k, v = line.split("=", 1)
        out[k.strip()] = v.strip()
    return out


# ---------------------------------------------------------------------------
# palettes


@dataclass
class Palette:
    """``linearMap<COLOUR>`` knots: ascending positions ``x`` (float64) and
    colours ``rgb`` (float32, shape (n,3))."""

    x: np.ndarray
    rgb: np.ndarray

    def __post_init__(self):
        self.x = np.ascontiguousarray(self.x, dtype=np.float64)
        self.rgb = np.ascontiguousarray(self.rgb, dtype=np.float32).reshape(-1, 3)
        if len(self.x) != len(self.rgb) or len(self.x) == 0:
            raise ValueError("palette needs n>0 knots with one colour each")

    @classmethod
    def from_rgb255(cls, rgb255) -> "Palette":
        """Knots at i/(n-1) with colours c/255 in float, like the .pal loader
        (splotch/splotchutils.cc:105-119)."""
        a = np.asarray(rgb255, dtype=np.float32).reshape(-1, 3)
        n = len(a)
        step = 1.0 / (n - 1) if n > 1 else 0.0
        x = np.arange(n, dtype=np.float64) * step
        return cls(x, (a / np.float32(255)).astype(np.float32))


def load_palette(path: str | Path) -> Palette:
    """Read a Splotch .pal file: ``name`` / ``0100`` / ``n`` then n lines r g b."""
    tok = Path(path).read_text().split()
    n = int(tok[2])
    vals = np.array([float(t) for t in tok[3:3 + 3 * n]], dtype=np.float32)
    return Palette.from_rgb255(vals.reshape(n, 3))


def get_colourmaps(params: ParamFile) -> list[Palette | None]:
    """``get_colourmaps`` (splotch/splotchutils.cc:63-125)."""
    ptypes = params.find("ptypes", 1)
    amap: list[Palette | None] = []
    for t in range(ptypes):
        if params.find(f"color_is_vector{t}", False):
            amap.append(None)
        else:
            amap.append(load_palette(params.find(f"palette{t}", typ=str)))
    return amap


# ---------------------------------------------------------------------------
# render_context


@dataclass
class RenderContext:
    """``render_context`` (splotch/splotchutils.h:98-122).  ``pic`` is the
    x-major image, shape (xres, yres, 3) float32 (``arr2<COLOUR>``)."""

    campos: np.ndarray = field(default_factory=lambda: np.zeros(3))
    centerpos: np.ndarray = field(default_factory=lambda: np.zeros(3))
    lookat: np.ndarray = field(default_factory=lambda: np.zeros(3))
    sky: np.ndarray = field(default_factory=lambda: np.array([0.0, 1.0, 0.0]))
    amap: list = field(default_factory=list)
    pic: np.ndarray | None = None
    npart: int = 0
    npart_all: int = 0
    b_brightness: float = 1.0
    xres: int = 0
    yres: int = 0


def update_res(params: ParamFile, rc: RenderContext) -> None:
    """``update_res`` (splotch/splotchutils.cc:292-302)."""
    xres = params.find("xres", 800)
    yres = params.find("yres", xres)
    if xres != rc.xres or yres != rc.yres or rc.pic is None:
        rc.xres, rc.yres = xres, yres
        rc.pic = np.zeros((xres, yres, 3), dtype=np.float32)


def frame_desc(params: ParamFile, rc: RenderContext, keep: list | None = None) -> _abi.FrameDesc:
    """Read every key host_rendering() reads, with the reference's defaults
    (splotch_host.cc:62-109, 256-265, 806, 812, 823-825), into a FrameDesc.
    ``keep`` collects arrays that must outlive the call (palette buffers)."""
    lib = _abi.load()
    d = _abi.FrameDesc()
    lib.spl_frame_desc_defaults(C.byref(d))
    d.xres = params.find("xres", 800)
    d.yres = params.find("yres", d.xres)
    d.zmax = params.find("zmax", 1.0e23)
    d.zmin = params.find("zmin", 0.0)
    d.fov = params.find("fov", 45.0)
    d.ptypes = params.find("ptypes", 1)
    if not 1 <= d.ptypes <= _abi.SPL_MAX_TYPES:
        raise ValueError("ptypes must be in [1,8]")
    for t in range(d.ptypes):
        d.smooth_factor[t] = params.find(f"smooth_factor{t}", 1.0)
    d.projection = 1 if params.find("projection", True) else 0
    d.minrad_pix = params.find("minrad_pix", 1.0)
    for t in range(d.ptypes):
        d.brightness[t] = params.find(f"brightness{t}", 1.0)
        d.color_is_vector[t] = 1 if params.find(f"color_is_vector{t}", False) else 0
    d.a_eq_e = 1 if params.find("a_eq_e", True) else 0
    d.sort_type = params.find("sort_type", 1)
    d.gray_absorption = params.find("gray_absorption", 0.2)
    d.tile_size = int(params.find("tile_size_cpu", 50.0))  # read as float32, then int
    if params.param_present("gpu_order"):
        d.order_mode = (_abi.SPL_ORDER_FRONT_TO_BACK
                        if params.find("gpu_order", "ftb", typ=str) == "ftb"
                        else _abi.SPL_ORDER_BACK_TO_FRONT)
    if params.param_present("gpu_ftb_epsilon"):
        d.ftb_epsilon = params.find("gpu_ftb_epsilon", 1e-9)
    if params.param_present("gpu_ftb_relative"):
        d.ftb_relative = params.find("gpu_ftb_relative", 1e-5)
    if params.param_present("gpu_splat_config"):
        d.splat_config = params.find("gpu_splat_config", -1)
    d.b_brightness = float(rc.b_brightness)
    for i in range(3):
        d.campos[i] = float(rc.campos[i])
        d.lookat[i] = float(rc.lookat[i])
        d.sky[i] = float(rc.sky[i])
        d.centerpos[i] = float(rc.centerpos[i])
    keep = keep if keep is not None else []
    for t in range(d.ptypes):
        if d.color_is_vector[t]:
            continue
        if t >= len(rc.amap) or rc.amap[t] is None:
            raise ValueError(f"trying to access an empty map (palette of type {t})")
        pal = rc.amap[t]
        keep.extend([pal.x, pal.rgb])
        d.pal_n[t] = len(pal.x)
        d.pal_x[t] = pal.x.ctypes.data
        d.pal_rgb[t] = pal.rgb.ctypes.data
    return d


def rays_desc(params: ParamFile) -> _abi.RaysDesc:
    """The keys host_rendering_new reads beyond frame_desc's, at its precision
    (splotch/new_renderer.cc:588-613: dome, fov and minrad_pix as double)."""
    r = _abi.RaysDesc()
    _abi.load().spl_rays_desc_defaults(C.byref(r))
    r.dome = 1 if params.find("dome", False) else 0
    r.fov = float(params.find("fov", 45.0))
    r.minrad_pix = float(params.find("minrad_pix", 1.0))
    return r


class Renderer:
    """Owns one spl_context (device buffers pooled across frames)."""

    def __init__(self, device: int = 0):
        self.lib = _abi.load()
        self.ctx = C.c_void_p()
        _abi.check(self.lib.spl_context_create(C.byref(self.ctx), device))
        self.device = device
        self._last_n = 0

    def close(self) -> None:
        if self.ctx:
            self.lib.spl_context_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr: int | None) -> None:
        _abi.check(self.lib.spl_context_set_stream(self.ctx, stream_ptr))

    # -- plain frame --------------------------------------------------------
    def render_aos(self, desc: _abi.FrameDesc, particles, pic, *, device: bool = False,
                   writeback: bool = False) -> None:
        """Render a particle_sim array (numpy, or a torch uint8 tensor of
        n*36 bytes when device=True) into pic (x-major float32)."""
        n = len(particles) if isinstance(particles, np.ndarray) else particles.numel() // 36
        p = _abi.Particles(n=n, layout=_abi.SPL_LAYOUT_AOS,
                           memspace=_abi.SPL_MEM_DEVICE if device else _abi.SPL_MEM_HOST,
                           aos=_abi.ptr(particles))
        img = _abi.Image(pic=_abi.ptr(pic), memspace=_abi.SPL_MEM_DEVICE if device
                         else _abi.SPL_MEM_HOST)
        _abi.check(self.lib.spl_render(self.ctx, C.byref(desc), C.byref(p), C.byref(img),
                                       _abi.SPL_WRITEBACK_FULL if writeback
                                       else _abi.SPL_WRITEBACK_NONE))
        self._last_n = n

    def prefetch_aos(self, particles) -> None:
        """spl_prefetch of a host particle_sim array: its copy to the device
        starts now, on a stream of its own, for a later render_aos of the same
        array (which waits for it instead of copying)."""
        n = len(particles) if isinstance(particles, np.ndarray) else particles.numel() // 36
        p = _abi.Particles(n=n, layout=_abi.SPL_LAYOUT_AOS, memspace=_abi.SPL_MEM_HOST,
                           aos=_abi.ptr(particles))
        _abi.check(self.lib.spl_prefetch(self.ctx, C.byref(p)))

    def render_soa(self, desc: _abi.FrameDesc, soa: dict, pic, *, device: bool = True) -> None:
        """Render SoA fields x,y,z,r,I,cr[,cg,cb][,type] (float32 / uint16)."""
        n = int(soa["x"].shape[0])
        p = _abi.Particles(n=n, layout=_abi.SPL_LAYOUT_SOA,
                           memspace=_abi.SPL_MEM_DEVICE if device else _abi.SPL_MEM_HOST)
        for f in ("x", "y", "z", "r", "I", "cr", "cg", "cb", "type"):
            setattr(p, f, _abi.ptr(soa.get(f)))
        img = _abi.Image(pic=_abi.ptr(pic), memspace=_abi.SPL_MEM_DEVICE if device
                         else _abi.SPL_MEM_HOST)
        _abi.check(self.lib.spl_render(self.ctx, C.byref(desc), C.byref(p), C.byref(img),
                                       _abi.SPL_WRITEBACK_NONE))
        self._last_n = n

    # -- ray-sphere frame (new_renderer=true) ---------------------------------
    def render_rays(self, desc: _abi.FrameDesc, rays: _abi.RaysDesc, particles, pic, *,
                    device: bool = False) -> None:
        """spl_render_rays: host_rendering_new (splotch/new_renderer.cc:522-641)
        of a particle_sim array (numpy, or a torch uint8 tensor of n*36 bytes
        when device=True) or of a dict of SoA fields, into pic (x-major)."""
        mem = _abi.SPL_MEM_DEVICE if device else _abi.SPL_MEM_HOST
        if isinstance(particles, dict):
            p = _abi.Particles(n=int(particles["x"].shape[0]), layout=_abi.SPL_LAYOUT_SOA,
                               memspace=mem)
            for f in ("x", "y", "z", "r", "I", "cr", "cg", "cb", "type"):
                setattr(p, f, _abi.ptr(particles.get(f)))
        else:
            n = len(particles) if isinstance(particles, np.ndarray) else particles.numel() // 36
            p = _abi.Particles(n=n, layout=_abi.SPL_LAYOUT_AOS, memspace=mem,
                               aos=_abi.ptr(particles))
        img = _abi.Image(pic=_abi.ptr(pic), memspace=mem)
        _abi.check(self.lib.spl_render_rays(self.ctx, C.byref(desc), C.byref(rays), C.byref(p),
                                            C.byref(img)))
        self._last_n = 0

    def stats(self) -> dict:
        s = _abi.Stats()
        _abi.check(self.lib.spl_get_stats(self.ctx, C.byref(s)))
        return s.as_dict()

    def set_split_tiles(self, mode: bool | int = True) -> None:
        """Which frames have heavy tiles cut into list segments in later
        renders (one GPU block per segment, results folded per pixel): True or
        SPL_SPLIT_ON additive and front-to-back frames, False or SPL_SPLIT_OFF
        none, SPL_SPLIT_ADDITIVE (the default) additive frames only."""
        m = mode if not isinstance(mode, bool) else (_abi.SPL_SPLIT_ON if mode
                                                      else _abi.SPL_SPLIT_OFF)
        _abi.check(self.lib.spl_context_set_split_tiles(self.ctx, int(m)))

    # -- gradients ------------------------------------------------------------
    def set_differentiable(self, enable: bool = True) -> None:
        """Ordered frames keep what spl_render_backward needs (per-pixel optical
        depth and stop position) while this is on."""
        _abi.check(self.lib.spl_context_set_differentiable(self.ctx, 1 if enable else 0))

    def backward(self, grad_pic, out: dict | None = None, *, device: bool = False) -> dict:
        """spl_render_backward for the last frame: dL/d(I, cr, cg, cb, x, y, z, r)
        per particle and dL/dcampos, given grad_pic = dL/dpic.  out maps field
        names to preallocated float32 arrays (numpy, or device tensors when
        device=True); by default numpy arrays are allocated."""
        if out is None:
            out = {f: np.zeros(self._last_n, np.float32) for f in _abi.GRAD_FIELDS}
            device = False
        g = _abi.Grads(memspace=_abi.SPL_MEM_DEVICE if device else _abi.SPL_MEM_HOST)
        for f in _abi.GRAD_FIELDS:
            setattr(g, f, _abi.ptr(out.get(f)))
        dev_img = not isinstance(grad_pic, np.ndarray)
        img = _abi.Image(pic=_abi.ptr(grad_pic),
                         memspace=_abi.SPL_MEM_DEVICE if dev_img else _abi.SPL_MEM_HOST)
        _abi.check(self.lib.spl_render_backward(self.ctx, C.byref(img), C.byref(g)))
        res = dict(out)
        res["campos"] = np.array(g.campos[:], dtype=np.float64)
        return res

    # -- test hooks -----------------------------------------------------------
    def projected(self, n: int) -> np.ndarray:
        out = np.zeros(n, dtype=PARTICLE_DTYPE)
        _abi.check(self.lib.spl_debug_get_projected(self.ctx, out.ctypes.data, n))
        return out

    def order(self, n: int) -> np.ndarray:
        """Visiting order of the active particles of the last frame."""
        out = np.zeros(max(n, 1), dtype=np.uint32)
        na = C.c_int64()
        _abi.check(self.lib.spl_debug_get_order(self.ctx, out.ctypes.data, n, C.byref(na)))
        return out[: na.value]

    def set_debug(self, flags: int) -> None:
        """spl_debug_set_options: bit 0 forces the exact FP64 projection."""
        _abi.check(self.lib.spl_debug_set_options(self.ctx, flags))

    def fragments(self) -> int:
        """Exact reference fragment count of the last frame."""
        v = C.c_int64()
        _abi.check(self.lib.spl_debug_count_fragments(self.ctx, C.byref(v)))
        return int(v.value)

    def bins(self, ntiles: int) -> tuple[np.ndarray, np.ndarray]:
        ts = np.zeros(ntiles + 1, dtype=np.int64)
        s = self.stats()
        ent = np.zeros(max(1, s["n_entries"]), dtype=np.uint32)
        _abi.check(self.lib.spl_debug_get_bins(self.ctx, ts.ctypes.data, ntiles + 1,
                                               ent.ctypes.data, len(ent)))
        return ts, ent[: s["n_entries"]]


def _renderer() -> "Renderer":
    global _default_renderer
    if _default_renderer is None:
        _default_renderer = Renderer()
    return _default_renderer


def particle_normalize(params: ParamFile, particles, renderer: Renderer | None = None, *,
                       device: bool = False) -> dict:
    """sceneMaker::particle_normalize (splotch/scenemaker.cc:40-296), in place
    on a particle_sim array (numpy, or a device uint8 tensor of n*36 bytes when
    device=True).  Like the reference it records the colour range of the data
    and the range applied as the range_min/max{t} and clamp_min/max{t} keys."""
    r = renderer or _renderer()
    d = _abi.NormalizeDesc()
    d.ptypes = params.find("ptypes", 1)
    for t in range(d.ptypes):
        d.intensity_log[t] = 1 if params.find(f"intensity_log{t}", False) else 0
        d.color_log[t] = 1 if params.find(f"color_log{t}", False) else 0
        d.color_asinh[t] = 1 if params.find(f"color_asinh{t}", False) else 0
        d.color_is_vector[t] = 1 if params.find(f"color_is_vector{t}", False) else 0
        for key in ("intensity_min", "intensity_max", "color_min", "color_max"):
            if params.param_present(f"{key}{t}"):
                getattr(d, "has_" + key)[t] = 1
                getattr(d, key)[t] = params.find(f"{key}{t}", 0.0)
    n = len(particles) if isinstance(particles, np.ndarray) else particles.numel() // 36
    p = _abi.Particles(n=n, layout=_abi.SPL_LAYOUT_AOS,
                       memspace=_abi.SPL_MEM_DEVICE if device else _abi.SPL_MEM_HOST,
                       aos=_abi.ptr(particles))
    res = _abi.NormalizeResult()
    _abi.check(r.lib.spl_particle_normalize(r.ctx, C.byref(d), C.byref(p), C.byref(res)))
    out = {k: [float(v) for v in getattr(res, k)[:d.ptypes]] for k, _ in res._fields_}
    for t in range(d.ptypes):
        for key in ("range_min", "range_max", "clamp_min", "clamp_max"):
            params.set_param(f"{key}{t}", out[key][t])
    return out


def post_desc(params: ParamFile, a_eq_e: bool | None = None) -> _abi.PostDesc:
    """The keys of splotch.cc:272-291 (a_eq_e, pic_gamma, pic_brightness,
    pic_contrast, colorbar) with the reference's defaults."""
    p = _abi.PostDesc()
    _abi.load().spl_post_desc_defaults(C.byref(p))
    p.a_eq_e = 1 if (params.find("a_eq_e", True) if a_eq_e is None else a_eq_e) else 0
    p.gamma = params.find("pic_gamma", 1.0)
    p.brightness = params.find("pic_brightness", 0.0)
    p.contrast = params.find("pic_contrast", 1.0)
    p.colorbar = 1 if params.find("colorbar", False) else 0
    return p


def postprocess(params: ParamFile, rc: RenderContext, renderer: Renderer | None = None,
                pic=None) -> None:
    """The master's post-processing after host_rendering (splotch.cc:272-291),
    in place on rc.pic (or on pic: a numpy array or a device tensor)."""
    r = renderer or _renderer()
    keep: list = []
    desc = frame_desc(params, rc, keep)
    target = rc.pic if pic is None else pic
    dev = not isinstance(target, np.ndarray)
    img = _abi.Image(pic=_abi.ptr(target), memspace=_abi.SPL_MEM_DEVICE if dev
                     else _abi.SPL_MEM_HOST)
    _abi.check(r.lib.spl_postprocess(r.ctx, C.byref(desc), C.byref(post_desc(params)),
                                     C.byref(img)))


PICTYPES = {0: ".tga", 2: ".ppm", 3: ".tga"}


def encode_image(pic, pictype: int = 0, renderer: Renderer | None = None) -> bytes:
    """The bytes of LS_Image's file for pictype 0 (TGA), 2 (PPM), 3 (RLE TGA)."""
    r = renderer or _renderer()
    dev = not isinstance(pic, np.ndarray)
    xres, yres = int(pic.shape[0]), int(pic.shape[1])
    img = _abi.Image(pic=_abi.ptr(pic), memspace=_abi.SPL_MEM_DEVICE if dev
                     else _abi.SPL_MEM_HOST)
    n = C.c_int64()
    _abi.check(r.lib.spl_image_encode(r.ctx, C.byref(img), xres, yres, pictype, None, 0,
                                      C.byref(n)))
    buf = np.zeros(n.value, np.uint8)
    _abi.check(r.lib.spl_image_encode(r.ctx, C.byref(img), xres, yres, pictype,
                                      buf.ctypes.data, n.value, C.byref(n)))
    return buf.tobytes()


def write_image(params: ParamFile, rc: RenderContext, outfile: str,
                renderer: Renderer | None = None) -> str:
    """splotch.cc:295-323: write rc.pic as outfile + .tga/.ppm by pictype."""
    pictype = params.find("pictype", 0)
    if pictype == 1:
        raise _abi.SplotchError(_abi.SPL_ERR_UNSUPPORTED, "ASCII PPM no longer supported")
    if pictype not in PICTYPES:
        raise _abi.SplotchError(_abi.SPL_ERR_INVALID, "No valid image file type given ...")
    r = renderer or _renderer()
    path = outfile + PICTYPES[pictype]
    img = _abi.Image(pic=_abi.ptr(rc.pic), memspace=_abi.SPL_MEM_HOST)
    _abi.check(r.lib.spl_write_image(r.ctx, C.byref(img), rc.pic.shape[0], rc.pic.shape[1],
                                     pictype, path.encode()))
    return path


class Batch:
    """spl_batch_*: many frames rendered by one captured CUDA graph.

    sets: list of device SoA dicts (x, y, z, r, I, cr[, cg, cb][, type] as
    tensors); frames: list of (set index, FrameDesc, device image tensor).
    The descs' palette arrays are copied at create."""

    def __init__(self, renderer: Renderer, sets: list, frames: list, *, tile_size: int = 0,
                 splat_config_additive: int = -1, splat_config_absorption: int = -1,
                 capacity_margin: float = 1.1, use_graph: bool = True,
                 tune_cache: bool = True):
        self.lib = renderer.lib
        self._keep = [sets, frames]
        psets = (_abi.Particles * max(1, len(sets)))()
        for k, soa in enumerate(sets):
            p = psets[k]
            p.n = int(soa["x"].shape[0])
            p.layout = _abi.SPL_LAYOUT_SOA
            p.memspace = _abi.SPL_MEM_DEVICE
            for f in ("x", "y", "z", "r", "I", "cr", "cg", "cb", "type"):
                setattr(p, f, _abi.ptr(soa.get(f)))
        pframes = (_abi.BatchFrame * len(frames))()
        for k, (s, desc, pic) in enumerate(frames):
            pframes[k].set = int(s)
            pframes[k].desc = desc
            pframes[k].pic = _abi.ptr(pic)
        opt = _abi.BatchOptions()
        self.lib.spl_batch_options_defaults(C.byref(opt))
        opt.tile_size = tile_size
        opt.splat_config_additive = splat_config_additive
        opt.splat_config_absorption = splat_config_absorption
        opt.capacity_margin = capacity_margin
        opt.use_graph = 1 if use_graph else 0
        opt.tune_cache = 1 if tune_cache else 0
        self.handle = C.c_void_p()
        _abi.check(self.lib.spl_batch_create(renderer.ctx, psets, len(sets), pframes,
                                             len(frames), C.byref(opt), C.byref(self.handle)))

    def render(self) -> None:
        _abi.check(self.lib.spl_batch_render(self.handle))

    def info(self) -> dict:
        i = _abi.BatchInfo()
        _abi.check(self.lib.spl_batch_get_info(self.handle, C.byref(i)))
        return i.as_dict()

    def close(self) -> None:
        if self.handle:
            self.lib.spl_batch_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_renderer: Renderer | None = None


def host_rendering(params: ParamFile, particles: np.ndarray, rc: RenderContext,
                   renderer: Renderer | None = None) -> np.ndarray:
    """Drop-in for ``host_rendering`` (splotch/splotch_host.cc:711-834).

    Overwrites ``rc.pic`` and mutates ``particles`` in place exactly as the
    reference does: projected x,y,z,r,I, colourised e, active flags, and the
    stable z order when ``a_eq_e`` is false.  Returns the particles the
    caller's vector still holds: all of them, or none after the ray-sphere
    renderer (``new_renderer=true``, splotch_host.cc:714-723), which empties
    the reference's vector (new_renderer.cc:584) and leaves this array as it
    was.
    """
    global _default_renderer
    if particles.dtype != PARTICLE_DTYPE or not particles.flags.c_contiguous:
        raise TypeError("particles must be a C-contiguous PARTICLE_DTYPE array")
    if renderer is None:
        if _default_renderer is None:
            _default_renderer = Renderer()
        renderer = _default_renderer
    keep: list = []
    desc = frame_desc(params, rc, keep)
    if rc.pic is None or rc.pic.shape != (desc.xres, desc.yres, 3):
        rc.pic = np.zeros((desc.xres, desc.yres, 3), dtype=np.float32)
    n = int(rc.npart) if rc.npart else len(particles)
    if params.find("new_renderer", False):
        renderer.render_rays(desc, rays_desc(params), particles[:n], rc.pic)
        return particles[:0]
    renderer.render_aos(desc, particles[:n], rc.pic, writeback=True)
    return particles
