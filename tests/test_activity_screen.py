"""The activity pass's float screen (screen_activity, splotch_gb300/csrc/
spl_project.cu) restated in numpy float32, against the oracle's exact
particle_project activity (splotch/splotch_host.cc:118-176).

The screen decides a particle only when the footprint test (and the z cut)
holds or fails for every value within its error bounds; everything else goes
through the exact float-float path.  These cases check the bounds on CPU: no
particle the screen calls active or inactive may be the other way round in the
exact computation, and the undecided share stays small.  (The GPU tests compare
the kernel itself: visiting order and bins with the screen against the FP64
hook, and footprint edges placed within 0.02 pixel of the image borders.)
"""
import ctypes as C

import numpy as np
import pytest

import splotch_gb300 as sg
from splotch_gb300 import _abi, synth

f32 = np.float32


def _fma(a, b, c):
    # a*b is exact in double for float operands; one rounding of the sum to
    # float32 stands in for the fused multiply-add (the bounds cover the rest)
    return (np.asarray(a, np.float64) * b + c).astype(f32)


def screen(desc, p) -> np.ndarray:
    """-1 undecided, 0 surely inactive, 1 surely active, per particle."""
    cam = _abi.Camera()
    assert _abi.load().spl_camera_setup(C.byref(desc), C.byref(cam)) == 0
    m = np.array(cam.mat[:], dtype=f32)
    res2, fovfct = f32(cam.res2), f32(cam.fovfct)
    xs = f32(np.float64(cam.res2) + cam.xshift)
    ys = f32((np.float64(cam.res2) + cam.yshift) + np.float64(cam.ycorr))
    zmin, zmax = f32(max(desc.zmin, 0.0)), f32(desc.zmax)
    minrad2 = f32(f32(desc.minrad_pix) * f32(desc.minrad_pix))
    x, y, z, r = (p[k].astype(f32) for k in ("x", "y", "z", "r"))
    t = p["type"].astype(np.int64)
    smooth = np.array(desc.smooth_factor[:], dtype=f32)[np.clip(t, 0, _abi.SPL_MAX_TYPES - 1)]
    dec = np.full(len(p), -1, np.int8)
    with np.errstate(all="ignore"):
        am = np.maximum(np.maximum(np.abs(x), np.abs(y)), np.abs(z))
        zf = _fma(m[10], z, _fma(m[9], y, _fma(m[8], x, m[11])))
        ez = (f32(2.0**-20) * _fma(f32(abs(m[8]) + abs(m[9]) + abs(m[10])), am, abs(m[11])))
        nz = -zf
        zcut = (nz + ez <= zmin) | (nz - ez >= zmax)
        ok = ((nz - ez > zmin) & (nz - ez > f32(1e-30)) & (nz + ez < zmax) &
              (nz + ez < f32(1e30)))
        den = (fovfct * nz).astype(f32)
        ok &= (den > f32(1e-30)) & (den < f32(1e30))
        xc = _fma(m[2], z, _fma(m[1], y, _fma(m[0], x, m[3])))
        yc = _fma(m[6], z, _fma(m[5], y, _fma(m[4], x, m[7])))
        sx = _fma(f32(abs(m[0]) + abs(m[1]) + abs(m[2])), am, abs(m[3]))
        sy = _fma(f32(abs(m[4]) + abs(m[5]) + abs(m[6])), am, abs(m[7]))
        k = (res2 / den).astype(f32)
        ek = (ez / (nz - ez) + f32(2.0**-18)).astype(f32)
        X = _fma(xc, k, xs)
        Y = _fma(yc, k, ys)
        r2 = (f32(2) * r * k * smooth).astype(f32)
        R = np.sqrt(r2 * r2 + minrad2).astype(f32)
        e = (f32(4) * ek + f32(2.0**-16)).astype(f32)
        mX = ((np.abs(xs) + np.abs(xc * k) + R) * e + sx * k * f32(2.0**-19) + f32(2.0**-6))
        mY = ((np.abs(ys) + np.abs(yc * k) + R) * e + sy * k * f32(2.0**-19) + f32(2.0**-6))
        ext = (f32(0.75) * R).astype(f32)
        fin = ((np.abs(X) < 1e30) & (np.abs(Y) < 1e30) & (mX < 1e30) & (mY < 1e30) &
               (ext < 1e30))
        off = ((X + ext + mX < 0) | (X - ext - mX + 1 >= desc.xres) | (Y + ext + mY < 0) |
               (Y - ext - mY + 1 >= desc.yres))
        r_ok = (r > f32(1e-30)) & (r < f32(1e30)) & (r2 > f32(1e-20)) & (smooth > 0)
        ax = np.maximum(np.floor(X - ext + 1 + mX), 0)
        bx = np.minimum(np.floor(X + ext + 1 - mX), desc.xres)
        ay = np.maximum(np.floor(Y - ext + 1 + mY), 0)
        by = np.minimum(np.floor(Y + ext + 1 - mY), desc.yres)
        inside = (ax < bx) & (ay < by)
    valid = (t >= 0) & (t < desc.ptypes)
    dec[valid & zcut] = 0
    live = valid & ~zcut & ok & fin
    dec[live & off] = 0
    dec[live & ~off & r_ok & inside] = 1
    return dec


def _tilted(w, seed, box):
    rng = np.random.default_rng(seed)
    c = np.full(3, 0.5 * box)
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    w.rc.campos = c + d * box * float(rng.uniform(0.9, 2.0))
    w.rc.centerpos = w.rc.campos.copy()
    w.rc.lookat = c + rng.normal(size=3) * 0.05 * box
    w.rc.sky = np.array([0.0, 1.0, 0.0]) if abs(d[1]) < 0.9 else np.array([1.0, 0.0, 0.0])
    return w


CASES = {
    "absorption_bench_camera": lambda: synth.plain_absorption(n_gas=240_000, n_star=60_000),
    "additive": lambda: synth.plain_additive(n=200_000),
    "large_shape": lambda: synth.large(n=300_000),
    "absorption_tilted": lambda: _tilted(synth.plain_absorption(n_gas=160_000, n_star=40_000),
                                         7, 500.0),
    "additive_tilted": lambda: _tilted(synth.plain_additive(n=150_000), 8, 100.0),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_screen_decides_as_the_exact_projection(name, port):
    w = CASES[name]()
    prm = dict(w.params.params)
    keep: list = []
    desc = sg.frame_desc(sg.ParamFile(prm), w.rc, keep)
    p = w.particles.copy()
    dec = screen(desc, p)
    ref = p.copy()
    port.project_colorize(prm, w.rc, ref)
    act = ref["active"].astype(bool)
    assert not (act & (dec == 0)).any(), "screened out an active particle"
    assert not (~act & (dec == 1)).any(), "screened in an inactive particle"
    undecided = float((dec < 0).mean())
    print(name, "active", act.mean(), "undecided", undecided)
    assert undecided < 0.01
