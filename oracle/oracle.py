"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Two checkers:

* ``Port``  -- liboracle.so, the plain-C restatement in spl_oracle.c (builds
  anywhere, including the AArch64 GPU host), with an FP64 splat and FP64 adjoint.
* ``Ref``   -- oracle/_ref/libsplotch_ref*.so, the reference's own
  host_rendering/particle_project/render_new compiled from its sources by
  build_ref.sh (only where those sources exist).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module.  The product path (splotch_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
PORT_LIB = BUILD / "liboracle.so"
REF_DIR = HERE / "_ref"
MAXT = 8

PARTICLE_DTYPE = np.dtype({
    "names": ["er", "eg", "eb", "x", "y", "z", "r", "I", "type", "active", "pad"],
    "formats": ["<f4"] * 8 + ["<u2", "u1", "u1"],
    "offsets": [0, 4, 8, 12, 16, 20, 24, 28, 32, 34, 35],
    "itemsize": 36,
})


def build_port(force: bool = False) -> Path:
    """Compile spl_oracle.c (plain C, OpenMP, no fused multiply-add)."""
    BUILD.mkdir(exist_ok=True)
    srcs = [HERE / "spl_oracle.c", HERE / "spl_oracle_rays.c"]
    hdr = HERE / "spl_oracle.h"
    newest = max(f.stat().st_mtime for f in srcs + [hdr])
    if not force and PORT_LIB.exists() and PORT_LIB.stat().st_mtime >= newest:
        return PORT_LIB
    cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           *[str(s) for s in srcs], "-o", str(PORT_LIB), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    return PORT_LIB


LEGACY_LIB = BUILD / "liblegacy_gpu.so"
LEGACY_PTX = REF_DIR / "legacy_cuda_kernel.ptx"


def build_legacy() -> bool:
    """Compile the host driver of the reference's legacy GPU kernels
    (legacy_gpu.cc; CUDA runtime only, so it builds on the GPU host too)."""
    BUILD.mkdir(exist_ok=True)
    src = HERE / "legacy_gpu.cc"
    if LEGACY_LIB.exists() and LEGACY_LIB.stat().st_mtime >= src.stat().st_mtime:
        return True
    nvcc = None
    for cand in ("nvcc", "/usr/local/cuda/bin/nvcc"):
        r = subprocess.run(["bash", "-c", f"command -v {cand}"], capture_output=True, text=True)
        if r.returncode == 0:
            nvcc = r.stdout.strip()
            break
    if nvcc is None:
        return False
    r = subprocess.run([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-x", "cu",
                        str(src), "-o", str(LEGACY_LIB), "-lcudart"], capture_output=True,
                       text=True)
    if r.returncode:
        raise RuntimeError(f"legacy driver build failed:\n{r.stderr}")
    return True


def ref_dir() -> Path:
    """Where the reference sources are read from (build_ref.sh decides)."""
    r = subprocess.run(["bash", str(HERE / "build_ref.sh"), "--where"], capture_output=True,
                       text=True)
    return Path(r.stdout.strip())


def build_ref() -> bool:
    """Compile the reference sources into oracle/_ref (no-op without them)."""
    r = subprocess.run(["bash", str(HERE / "build_ref.sh")], capture_output=True, text=True)
    return r.returncode == 0 and (REF_DIR / "libsplotch_ref.so").exists()


class SpoParams(C.Structure):
    _fields_ = [
        ("xres", C.c_int), ("yres", C.c_int), ("fov", C.c_float), ("zmin", C.c_float),
        ("zmax", C.c_float), ("minrad_pix", C.c_float), ("projection", C.c_int),
        ("ptypes", C.c_int), ("smooth_factor", C.c_float * MAXT),
        ("brightness", C.c_float * MAXT), ("color_is_vector", C.c_int * MAXT),
        ("b_brightness", C.c_float), ("pal_n", C.c_int * MAXT),
        ("pal_x", C.c_void_p * MAXT), ("pal_rgb", C.c_void_p * MAXT), ("a_eq_e", C.c_int),
        ("gray_absorption", C.c_float), ("sort_type", C.c_int), ("tile_size", C.c_int),
        ("campos", C.c_double * 3), ("lookat", C.c_double * 3), ("sky", C.c_double * 3),
        ("centerpos", C.c_double * 3),
    ]


class SpoCamera(C.Structure):
    _fields_ = [("mat", C.c_float * 12), ("res2", C.c_float), ("ycorr", C.c_float),
                ("fovfct", C.c_float), ("xfac", C.c_float), ("xshift", C.c_double),
                ("yshift", C.c_double)]


class SpoRaysParams(C.Structure):
    _fields_ = [("dome", C.c_int), ("fov", C.c_double), ("minrad_pix", C.c_double)]


class SpoNormParams(C.Structure):
    _fields_ = [("ptypes", C.c_int)] + [
        (k, C.c_int * MAXT) for k in ("intensity_log", "color_log", "color_asinh",
                                       "color_is_vector", "has_intensity_min",
                                       "has_intensity_max", "has_color_min", "has_color_max")] + [
        (k, C.c_float * MAXT) for k in ("intensity_min", "intensity_max", "color_min",
                                         "color_max")]


class SpoNormOut(C.Structure):
    _fields_ = [(k, C.c_double * MAXT) for k in ("range_min", "range_max", "clamp_min",
                                                  "clamp_max", "intensity_min", "intensity_max",
                                                  "size_min", "size_max")]


def norm_params(params: dict) -> SpoNormParams:
    """The keys particle_normalize reads (scenemaker.cc:44-55, 222-232)."""
    p = SpoNormParams()
    p.ptypes = _get(params, "ptypes", 1)
    for t in range(p.ptypes):
        p.intensity_log[t] = 1 if _get(params, f"intensity_log{t}", False) else 0
        p.color_log[t] = 1 if _get(params, f"color_log{t}", False) else 0
        p.color_asinh[t] = 1 if _get(params, f"color_asinh{t}", False) else 0
        p.color_is_vector[t] = 1 if _get(params, f"color_is_vector{t}", False) else 0
        for key, has, val in (("intensity_min", "has_intensity_min", "intensity_min"),
                              ("intensity_max", "has_intensity_max", "intensity_max"),
                              ("color_min", "has_color_min", "color_min"),
                              ("color_max", "has_color_max", "color_max")):
            if f"{key}{t}" in params:
                getattr(p, has)[t] = 1
                getattr(p, val)[t] = float(np.float32(_get(params, f"{key}{t}", 0.0)))
    return p


class SpoPost(C.Structure):
    _fields_ = [("a_eq_e", C.c_int), ("gamma", C.c_double), ("brightness", C.c_double),
                ("contrast", C.c_double), ("colorbar", C.c_int)]


def _get(params: dict, key: str, default):
    """paramfile::find semantics on a plain dict of strings (no insertion)."""
    if key not in params:
        return default
    s = str(params[key]).strip()
    if isinstance(default, bool):
        return s.lower() in ("t", "y", "true", ".true.")
    if isinstance(default, int):
        return int(s)
    if isinstance(default, float):
        return float(s)
    return s


def make_params(params: dict, rc, keep: list) -> SpoParams:
    """Everything host_rendering reads (splotch_host.cc:62-109, 256-265, 806-825)."""
    p = SpoParams()
    p.xres = _get(params, "xres", 800)
    p.yres = _get(params, "yres", p.xres)
    p.fov = _get(params, "fov", 45.0)
    p.zmin = _get(params, "zmin", 0.0)
    p.zmax = _get(params, "zmax", 1e23)
    p.minrad_pix = _get(params, "minrad_pix", 1.0)
    p.projection = 1 if _get(params, "projection", True) else 0
    p.ptypes = _get(params, "ptypes", 1)
    for t in range(p.ptypes):
        p.smooth_factor[t] = _get(params, f"smooth_factor{t}", 1.0)
        p.brightness[t] = _get(params, f"brightness{t}", 1.0)
        p.color_is_vector[t] = 1 if _get(params, f"color_is_vector{t}", False) else 0
        if not p.color_is_vector[t]:
            pal = rc.amap[t]
            x = np.ascontiguousarray(pal.x, np.float64)
            rgb = np.ascontiguousarray(pal.rgb, np.float32)
            keep += [x, rgb]
            p.pal_n[t] = len(x)
            p.pal_x[t] = x.ctypes.data
            p.pal_rgb[t] = rgb.ctypes.data
    p.b_brightness = float(rc.b_brightness)
    p.a_eq_e = 1 if _get(params, "a_eq_e", True) else 0
    p.gray_absorption = _get(params, "gray_absorption", 0.2)
    p.sort_type = _get(params, "sort_type", 1)
    p.tile_size = int(_get(params, "tile_size_cpu", 50.0))
    for i in range(3):
        p.campos[i] = float(rc.campos[i])
        p.lookat[i] = float(rc.lookat[i])
        p.sky[i] = float(rc.sky[i])
        p.centerpos[i] = float(rc.centerpos[i])
    return p


def _vp(a):
    return None if a is None else a.ctypes.data


class Port:
    """The C restatement (spl_oracle.c)."""

    def __init__(self, threads: int = 0):
        lib = C.CDLL(str(build_port()))
        vp, i64, i32 = C.c_void_p, C.c_int64, C.c_int
        for name, res, args in [
            ("spo_set_threads", None, [i32]),
            ("spo_get_threads", i32, []),
            ("spo_camera_setup", i32, [vp, vp]),
            ("spo_project", None, [vp, vp, vp, i64]),
            ("spo_colorize", None, [vp, vp, i64]),
            ("spo_sort_perm", i32, [vp, i64, i32, vp]),
            ("spo_apply_perm", None, [vp, vp, i64, vp]),
            ("spo_bin", i64, [vp, vp, i64, i32, i32, i32, vp, vp]),
            ("spo_render_fp32", i64, [vp, vp, i64, i32, i32, i32, i32, C.c_float, i32, vp]),
            ("spo_render_fp64", i64, [vp, vp, i64, i32, i32, i32, i32, C.c_double, vp]),
            ("spo_host_rendering", i32, [vp, vp, i64, i32, vp]),
            ("spo_splat_adjoint_fp64", i32,
             [vp, vp, i64, i32, i32, i32, i32, C.c_double, vp, vp, vp, vp, vp]),
            ("spo_model_project_all", i32, [vp, vp, vp, i64, vp]),
            ("spo_model_vjp_all", i32, [vp, vp, vp, i64, vp, vp, vp]),
            ("spo_render_frozen_fp64", i64,
             [vp, vp, vp, i64, i32, i32, i32, i32, C.c_double, vp]),
            ("spo_render_frozen_vjp_fp64", i32,
             [vp, vp, vp, i64, i32, i32, i32, i32, C.c_double, vp, vp]),
            ("spo_grad_fp64", i32, [vp, vp, vp, vp, i64, i32, vp, vp, vp]),
            ("spo_fd_particles", i32,
             [vp, vp, vp, vp, i64, i32, vp, vp, i32, C.c_double, vp, vp]),
            ("spo_fd_campos", i32, [vp, vp, vp, vp, i64, i32, vp, C.c_double, vp]),
            ("spo_postprocess", i32, [vp, vp, vp, i32, i32]),
            ("spo_image_bytes", i64, [vp, i32, i32, i32, vp, i64]),
            ("spo_particle_normalize", i32, [vp, vp, i64, vp]),
            ("spo_render_rays", i32, [vp, vp, vp, i64, i32, vp, vp, vp]),
        ]:
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        self.lib = lib
        if threads:
            lib.spo_set_threads(threads)

    @property
    def threads(self) -> int:
        return self.lib.spo_get_threads()

    def camera(self, params: dict, rc) -> SpoCamera:
        keep: list = []
        prm = make_params(params, rc, keep)
        cam = SpoCamera()
        if self.lib.spo_camera_setup(C.byref(prm), C.byref(cam)):
            raise ValueError("degenerate matrix")
        return cam

    def project_colorize(self, params: dict, rc, p: np.ndarray, colorize: bool = True) -> None:
        keep: list = []
        prm = make_params(params, rc, keep)
        cam = SpoCamera()
        if self.lib.spo_camera_setup(C.byref(prm), C.byref(cam)):
            raise ValueError("degenerate matrix")
        self.lib.spo_project(C.byref(prm), C.byref(cam), _vp(p), len(p))
        if colorize:
            self.lib.spo_colorize(C.byref(prm), _vp(p), len(p))

    def sort_perm(self, p: np.ndarray, sort_type: int) -> np.ndarray:
        perm = np.zeros(len(p), dtype=np.uint32)
        if self.lib.spo_sort_perm(_vp(p), len(p), sort_type, _vp(perm)):
            raise ValueError("unknown sorting chosen ...")
        return perm

    def bins(self, p: np.ndarray, order, xres: int, yres: int, T: int):
        ncx, ncy = (xres + T - 1) // T, (yres + T - 1) // T
        ts = np.zeros(ncx * ncy + 1, dtype=np.int64)
        tot = self.lib.spo_bin(_vp(p), _vp(order), len(p), xres, yres, T, _vp(ts), None)
        ent = np.zeros(max(1, tot), dtype=np.uint32)
        self.lib.spo_bin(_vp(p), _vp(order), len(p), xres, yres, T, _vp(ts), _vp(ent))
        return ts, ent[:tot]

    def render_fp32(self, p, order, xres, yres, T, a_eq_e, gray, simd=False):
        pic = np.zeros((xres, yres, 3), dtype=np.float32)
        fr = self.lib.spo_render_fp32(_vp(p), _vp(order), len(p), xres, yres, T, int(a_eq_e),
                                      float(gray), int(simd), _vp(pic))
        return pic, fr

    def render_fp64(self, p, order, xres, yres, T, a_eq_e, gray):
        pic = np.zeros((xres, yres, 3), dtype=np.float64)
        fr = self.lib.spo_render_fp64(_vp(p), _vp(order), len(p), xres, yres, T, int(a_eq_e),
                                      float(np.float32(gray)), _vp(pic))
        return pic, fr

    def host_rendering(self, params: dict, rc, p: np.ndarray, simd: bool = False) -> np.ndarray:
        keep: list = []
        prm = make_params(params, rc, keep)
        pic = np.zeros((prm.xres, prm.yres, 3), dtype=np.float32)
        if self.lib.spo_host_rendering(C.byref(prm), _vp(p), len(p), int(simd), _vp(pic)):
            raise RuntimeError("oracle host_rendering failed")
        return pic

    def splat_adjoint_fp64(self, p, order, xres, yres, T, a_eq_e, gray, gpic):
        n = len(p)
        gx, gy, gr = (np.zeros(n) for _ in range(3))
        ge = np.zeros((n, 3))
        g = np.ascontiguousarray(gpic, dtype=np.float64)
        self.lib.spo_splat_adjoint_fp64(_vp(p), _vp(order), n, xres, yres, T, int(a_eq_e),
                                        float(np.float32(gray)), _vp(g), _vp(gx), _vp(gy),
                                        _vp(gr), _vp(ge))
        return gx, gy, gr, ge

    # ---- after host_rendering: post-processing and image output -------------
    def postprocess(self, params: dict, rc, pic: np.ndarray, a_eq_e: bool) -> np.ndarray:
        keep: list = []
        prm = make_params(params, rc, keep)
        post = SpoPost(a_eq_e=int(a_eq_e), gamma=_get(params, "pic_gamma", 1.0),
                       brightness=_get(params, "pic_brightness", 0.0),
                       contrast=_get(params, "pic_contrast", 1.0),
                       colorbar=1 if _get(params, "colorbar", False) else 0)
        out = np.ascontiguousarray(pic, np.float32).copy()
        self.lib.spo_postprocess(C.byref(prm), C.byref(post), _vp(out), out.shape[0],
                                 out.shape[1])
        return out

    def render_rays(self, params: dict, rc, p: np.ndarray, exact: bool = True):
        """host_rendering with new_renderer=true (new_renderer.cc:522-641) on a
        copy of p.  Returns (image, stats): float64 with exact exp and double
        sums when exact, else float32 in the reference's arithmetic."""
        keep: list = []
        prm = make_params(params, rc, keep)
        rp = SpoRaysParams(dome=1 if _get(params, "dome", False) else 0,
                           fov=_get(params, "fov", 45.0),
                           minrad_pix=_get(params, "minrad_pix", 1.0))
        q = np.ascontiguousarray(p).copy()
        shape = (prm.xres, prm.yres, 3)
        pic = None if exact else np.zeros(shape, np.float32)
        pic64 = np.zeros(shape, np.float64) if exact else None
        stats = np.zeros(5, np.int64)
        rc_ = self.lib.spo_render_rays(C.byref(prm), C.byref(rp), _vp(q), len(q), int(exact),
                                       _vp(pic), _vp(pic64), _vp(stats))
        if rc_ == -1:
            raise ValueError("inconsistent: the ray-sphere renderer needs a_eq_e")
        if rc_ == -2:
            raise ValueError("inconsistency: a dome needs xres == yres")
        names = ("n_used", "n_grid", "n_overlap", "levels", "fragments")
        return (pic64 if exact else pic), dict(zip(names, (int(v) for v in stats)))

    def particle_normalize(self, params: dict, p: np.ndarray) -> dict:
        """In place on particle_sim records; returns the per-type ranges it
        leaves in the paramfile (range_min/max, clamp_min/max) and more."""
        np_ = norm_params(params)
        out = SpoNormOut()
        if self.lib.spo_particle_normalize(C.byref(np_), _vp(p), len(p), C.byref(out)):
            raise ValueError("particle type outside [0, ptypes)")
        return {k: list(getattr(out, k)[:np_.ptypes]) for k, _ in SpoNormOut._fields_}

    def image_bytes(self, pic: np.ndarray, pictype: int) -> bytes:
        p = np.ascontiguousarray(pic, np.float32)
        n = self.lib.spo_image_bytes(_vp(p), p.shape[0], p.shape[1], pictype, None, 0)
        if n < 0:
            raise ValueError("No valid image file type given ...")
        buf = np.zeros(n, np.uint8)
        self.lib.spo_image_bytes(_vp(p), p.shape[0], p.shape[1], pictype, _vp(buf), n)
        return buf.tobytes()

    # ---- differentiable FP64 model (checker of the adjoint path) ----------
    # raw: particle_sim records before projection (world inputs); cov: the same
    # records after project_colorize (their active flags, positions and radii
    # fix coverage, bins and order).  Gradient columns: I, e.r, e.g, e.b, x, y,
    # z, r (hsml).

    GRAD_FIELDS = ("I", "er", "eg", "eb", "x", "y", "z", "r")

    def model_project(self, params: dict, rc, raw, cov) -> np.ndarray:
        keep: list = []
        prm = make_params(params, rc, keep)
        w = np.zeros((len(raw), 6))
        if self.lib.spo_model_project_all(C.byref(prm), _vp(raw), _vp(cov), len(raw), _vp(w)):
            raise ValueError("degenerate matrix")
        return w

    def render_frozen_fp64(self, params: dict, cov, w, order) -> np.ndarray:
        xres = int(_get(params, "xres", 800))
        yres = int(_get(params, "yres", xres))
        T = int(_get(params, "tile_size_cpu", 50.0))
        a_eq_e = 1 if _get(params, "a_eq_e", True) else 0
        gray = float(np.float32(_get(params, "gray_absorption", 0.2)))
        pic = np.zeros((xres, yres, 3))
        w = np.ascontiguousarray(w, dtype=np.float64)
        if self.lib.spo_render_frozen_fp64(_vp(cov), _vp(w), _vp(order), len(cov), xres, yres,
                                           T, a_eq_e, gray, _vp(pic)) < 0:
            raise RuntimeError("frozen render failed")
        return pic

    def grad_fp64(self, params: dict, rc, raw, cov, order, gpic):
        """FP64 adjoint: dL/d(inputs) (n x 8) and dL/dcampos for L = sum(gpic*pic)."""
        keep: list = []
        prm = make_params(params, rc, keep)
        g = np.ascontiguousarray(gpic, dtype=np.float64)
        grad = np.zeros((len(raw), 8))
        gc = np.zeros(3)
        if self.lib.spo_grad_fp64(C.byref(prm), _vp(raw), _vp(cov), _vp(order), len(raw),
                                  prm.tile_size, _vp(g), _vp(grad), _vp(gc)):
            raise RuntimeError("oracle gradient failed")
        return grad, gc

    def model_vjp(self, params: dict, rc, raw, cov, gw):
        keep: list = []
        prm = make_params(params, rc, keep)
        gw = np.ascontiguousarray(gw, dtype=np.float64)
        grad = np.zeros((len(raw), 8))
        gc = np.zeros(3)
        if self.lib.spo_model_vjp_all(C.byref(prm), _vp(raw), _vp(cov), len(raw), _vp(gw),
                                      _vp(grad), _vp(gc)):
            raise ValueError("degenerate matrix")
        return grad, gc

    def fd_particles(self, params: dict, rc, raw, cov, order, target, sel, h: float = 1e-4):
        """Central differences of sum((pic - target)^2), coverage frozen."""
        keep: list = []
        prm = make_params(params, rc, keep)
        sel = np.ascontiguousarray(sel, dtype=np.int64)
        t = np.ascontiguousarray(target, dtype=np.float32)
        fd = np.zeros((len(sel), 8))
        ex = np.zeros((len(sel), 8), dtype=np.uint8)
        if self.lib.spo_fd_particles(C.byref(prm), _vp(raw), _vp(cov), _vp(order), len(raw),
                                     prm.tile_size, _vp(t), _vp(sel), len(sel), h, _vp(fd),
                                     _vp(ex)):
            raise RuntimeError("oracle finite differences failed")
        return fd, ex.astype(bool)

    def fd_campos(self, params: dict, rc, raw, cov, order, target, h: float = 1e-4):
        keep: list = []
        prm = make_params(params, rc, keep)
        t = np.ascontiguousarray(target, dtype=np.float32)
        fd = np.zeros(3)
        if self.lib.spo_fd_campos(C.byref(prm), _vp(raw), _vp(cov), _vp(order), len(raw),
                                  prm.tile_size, _vp(t), h, _vp(fd)):
            raise RuntimeError("oracle finite differences failed")
        return fd


class Ref:
    """The reference's own compiled host renderer (oracle/_ref)."""

    def __init__(self, scalar: bool = False):
        name = "libsplotch_ref_scalar.so" if scalar else "libsplotch_ref.so"
        path = REF_DIR / name
        if not path.exists():
            raise FileNotFoundError(path)
        lib = C.CDLL(str(path))
        vp, i32, i64, f32 = C.c_void_p, C.c_int, C.c_long, C.c_float
        lib.ref_simd_branch.restype = i32
        lib.ref_project_colorize.restype = i32
        lib.ref_project_colorize.argtypes = [vp, vp, i32, vp, i64, vp, vp, vp, vp, i32, vp, vp, vp,
                                             f32, i32]
        lib.ref_render_new.restype = i32
        lib.ref_render_new.argtypes = [vp, i32, i32, i32, i32, f32, i32, vp]
        lib.ref_particle_sort.restype = i32
        lib.ref_particle_sort.argtypes = [vp, i32, i32]
        lib.ref_host_rendering.restype = i32
        lib.ref_host_rendering.argtypes = [vp, vp, i32, vp, i64, vp, vp, vp, vp, i32, vp, vp, vp,
                                           f32, i32, i32, vp]
        lib.ref_postprocess.restype = i32
        lib.ref_postprocess.argtypes = [vp, vp, i32, vp, i32, i32, i32, i32, vp, vp, vp]
        lib.ref_write_image.restype = i32
        lib.ref_write_image.argtypes = [vp, i32, i32, i32, C.c_char_p]
        lib.ref_particle_normalize.restype = i32
        lib.ref_particle_normalize.argtypes = [vp, vp, i32, vp, i64, i32, vp]
        self.lib = lib
        self.simd = bool(lib.ref_simd_branch())

    @staticmethod
    def _kv(params: dict):
        keys = [k.encode() for k in params]
        vals = [str(v).encode() for v in params.values()]
        ka = (C.c_char_p * len(keys))(*keys)
        va = (C.c_char_p * len(vals))(*vals)
        return ka, va, len(keys)

    @staticmethod
    def _cam(rc):
        return [np.ascontiguousarray(a, np.float64) for a in (rc.campos, rc.lookat, rc.sky,
                                                             rc.centerpos)]

    @staticmethod
    def _pals(rc, ntypes):
        n = (C.c_int * ntypes)()
        xs = (C.c_void_p * ntypes)()
        rgbs = (C.c_void_p * ntypes)()
        keep = []
        for t in range(ntypes):
            pal = rc.amap[t] if t < len(rc.amap) else None
            if pal is None:
                n[t] = 0
                continue
            x = np.ascontiguousarray(pal.x, np.float64)
            rgb = np.ascontiguousarray(pal.rgb, np.float32)
            keep += [x, rgb]
            n[t], xs[t], rgbs[t] = len(x), x.ctypes.data, rgb.ctypes.data
        return n, xs, rgbs, keep

    def project_colorize(self, params: dict, rc, p: np.ndarray, colorize: bool = True) -> None:
        ka, va, nkv = self._kv(params)
        cams = self._cam(rc)
        nt = int(params.get("ptypes", 1))
        n, xs, rgbs, keep = self._pals(rc, nt)
        if self.lib.ref_project_colorize(ka, va, nkv, _vp(p), len(p), *[_vp(c) for c in cams],
                                         nt, n, xs, rgbs, float(rc.b_brightness), int(colorize)):
            raise RuntimeError("reference particle_project failed")

    def render_new(self, p, xres, yres, a_eq_e, gray, T) -> np.ndarray:
        pic = np.zeros((xres, yres, 3), dtype=np.float32)
        if self.lib.ref_render_new(_vp(p), len(p), xres, yres, int(a_eq_e), float(gray), T,
                                   _vp(pic)):
            raise RuntimeError("reference render_new failed")
        return pic

    def particle_sort(self, p, sort_type: int) -> None:
        if self.lib.ref_particle_sort(_vp(p), len(p), sort_type):
            raise RuntimeError("reference particle_sort failed")

    def host_rendering(self, params: dict, rc, p: np.ndarray) -> np.ndarray:
        ka, va, nkv = self._kv(params)
        cams = self._cam(rc)
        nt = int(params.get("ptypes", 1))
        n, xs, rgbs, keep = self._pals(rc, nt)
        xres = int(params.get("xres", 800))
        yres = int(params.get("yres", xres))
        pic = np.zeros((xres, yres, 3), dtype=np.float32)
        if self.lib.ref_host_rendering(ka, va, nkv, _vp(p), len(p), *[_vp(c) for c in cams], nt,
                                       n, xs, rgbs, float(rc.b_brightness), xres, yres, _vp(pic)):
            raise RuntimeError("reference host_rendering failed")
        return pic

    def postprocess(self, params: dict, rc, pic: np.ndarray, a_eq_e: bool) -> np.ndarray:
        """splotch.cc:272-291 on a copy of the x-major image."""
        ka, va, nkv = self._kv(params)
        nt = int(params.get("ptypes", 1))
        n, xs, rgbs, keep = self._pals(rc, nt)
        out = np.ascontiguousarray(pic, np.float32).copy()
        if self.lib.ref_postprocess(ka, va, nkv, _vp(out), out.shape[0], out.shape[1],
                                    int(a_eq_e), nt, n, xs, rgbs):
            raise RuntimeError("reference post-processing failed")
        return out

    def particle_normalize(self, params: dict, p: np.ndarray) -> dict:
        """sceneMaker::particle_normalize in place; the range/clamp keys it sets."""
        ka, va, nkv = self._kv(params)
        nt = int(params.get("ptypes", 1))
        out = np.zeros((nt, 4))
        if self.lib.ref_particle_normalize(ka, va, nkv, _vp(p), len(p), nt, _vp(out)):
            raise RuntimeError("reference particle_normalize failed")
        return {"range_min": list(out[:, 0]), "range_max": list(out[:, 1]),
                "clamp_min": list(out[:, 2]), "clamp_max": list(out[:, 3])}

    def image_bytes(self, pic: np.ndarray, pictype: int, tmpdir) -> bytes:
        """The file LS_Image writes (splotch.cc:295-323)."""
        path = str(Path(tmpdir) / f"ref_image_{pictype}")
        p = np.ascontiguousarray(pic, np.float32)
        if self.lib.ref_write_image(_vp(p), p.shape[0], p.shape[1], pictype, path.encode()):
            raise RuntimeError("reference image output failed")
        return Path(path).read_bytes()


def rel_linf(a: np.ndarray, b: np.ndarray, floor_frac: float = 1e-6) -> float:
    """max |a-b| / max(|b|, floor), floor = floor_frac * max|b| (per image)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    m = float(np.max(np.abs(b))) if b.size else 0.0
    floor = max(floor_frac * m, 1e-30)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if b.size else 0.0


class LegFrame(C.Structure):
    _fields_ = [("mat", C.c_float * 12), ("projection", C.c_int), ("xres", C.c_int),
                ("yres", C.c_int), ("fovfct", C.c_float), ("dist", C.c_float),
                ("xfac", C.c_float), ("minrad_pix", C.c_float), ("xshift", C.c_double),
                ("yshift", C.c_double), ("ptypes", C.c_int), ("col_vector", C.c_int * 8),
                ("brightness", C.c_float * 8), ("smooth_fac", C.c_float * 8),
                ("inorm_min", C.c_float * 8), ("inorm_max", C.c_float * 8),
                ("cnorm_min", C.c_float * 8), ("cnorm_max", C.c_float * 8)]


class LegacyGPU:
    """The reference's legacy GPU renderer (cuda/: k_range, k_process and the
    full-atomics k_render), compiled from its sources to PTX by build_ref.sh
    and driven by legacy_gpu.cc the way cuda_rendering drives it for one
    chunk.  Additive frames only, as that path renders them.  Its
    normalisation needs intensity_min/max and color_min/max per type
    (cuda/cuda_utils.cu:56-59); render() passes [0, 1] for both, so inputs
    pre-clamped to [0, 1] render as the plain path renders them."""

    def __init__(self):
        if not LEGACY_PTX.exists():
            raise FileNotFoundError(f"{LEGACY_PTX} is absent (built by build_ref.sh where "
                                    "the reference sources are)")
        build_legacy()
        self.lib = C.CDLL(str(LEGACY_LIB))
        self.lib.leg_open.restype = C.c_int
        self.lib.leg_open.argtypes = [C.c_char_p]
        self.lib.leg_render.restype = C.c_int
        self.lib.leg_render.argtypes = [C.POINTER(LegFrame), C.c_void_p, C.c_int64, C.c_void_p,
                                        C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        rc = self.lib.leg_open(str(LEGACY_PTX).encode())
        if rc:
            raise RuntimeError(f"loading the legacy kernels failed ({rc})")

    def frame(self, port: "Port", params: dict, rc) -> tuple:
        """The constant block's inputs (cu_get_trans_params, cu_init_transform)
        and the colour map (setup_colormap) of one frame."""
        cam = port.camera(params, rc)
        f = LegFrame()
        f.mat[:] = list(cam.mat)
        f.projection = 1 if _get(params, "projection", True) else 0
        f.xres = _get(params, "xres", 800)
        f.yres = _get(params, "yres", f.xres)
        f.fovfct, f.xfac = cam.fovfct, cam.xfac
        d = np.asarray(rc.centerpos, np.float64) - np.asarray(rc.lookat, np.float64)
        f.dist = float(np.float32(np.sqrt((d * d).sum())))
        f.minrad_pix = float(_get(params, "minrad_pix", 1.0))
        f.xshift, f.yshift = cam.xshift, cam.yshift
        f.ptypes = _get(params, "ptypes", 1)
        vals, points = [], []
        for t in range(f.ptypes):
            f.col_vector[t] = 1 if _get(params, f"color_is_vector{t}", False) else 0
            f.brightness[t] = float(np.float32(_get(params, f"brightness{t}", 1.0) *
                                               float(getattr(rc, "b_brightness", 1.0))))
            f.smooth_fac[t] = float(_get(params, f"smooth_factor{t}", 1.0))
            f.inorm_min[t], f.inorm_max[t], f.cnorm_min[t], f.cnorm_max[t] = 0.0, 1.0, 0.0, 1.0
            points.append(len(vals))
            pal = rc.amap[t] if t < len(rc.amap) else None
            if pal is not None:
                for x, c in zip(pal.x, pal.rgb):
                    vals.append((np.float32(x), c[0], c[1], c[2]))
        cmap = np.ascontiguousarray(np.array(vals, dtype=np.float32).reshape(-1, 4))
        return f, cmap, np.ascontiguousarray(np.array(points, dtype=np.int32))

    def render(self, port: "Port", params: dict, rc, particles: np.ndarray,
               frame=None) -> tuple:
        """(image x-major float32, stage milliseconds dict)."""
        f, cmap, points = frame if frame is not None else self.frame(port, params, rc)
        pic = np.zeros((f.xres, f.yres, 3), np.float32)
        ms = np.zeros(6)
        p = np.ascontiguousarray(particles)
        rc_ = self.lib.leg_render(C.byref(f), _vp(p), len(p), _vp(cmap), len(cmap),
                                  _vp(points), _vp(pic), _vp(ms))
        if rc_:
            raise RuntimeError(f"legacy render failed ({rc_})")
        keys = ("copy_in", "k_range", "k_process", "k_render", "copy_out", "total")
        return pic, dict(zip(keys, ms.tolist()))
