"""The ray-sphere renderer on the GPU (spl_render_rays; host_rendering with
new_renderer=true, splotch/new_renderer.cc:522-641) against the FP64 oracle
restatement and the reference's own images.

Tolerance: 1e-4 relative L-infinity (per pixel, floor 1e-6 of the image's
largest magnitude), against the FP64 restatement (exact exp, double sums, the
reference's culling and coverage decisions) and against the reference's
images (whose exptable weights sit within 3e-5 of exact ones).
"""
import json
from pathlib import Path

import numpy as np
import pytest

import splotch_gb300 as sg
from oracle.oracle import PARTICLE_DTYPE, rel_linf
from splotch_gb300 import Palette, RenderContext, synth

pytestmark = pytest.mark.gpu

TOL = 1e-4
GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("rays_*.npz"))


def load(name):
    z = np.load(GOLDEN / f"{name}.npz")
    meta = json.loads(bytes(z["meta"]).decode())
    rc = RenderContext(campos=np.array(meta["campos"]), centerpos=np.array(meta["centerpos"]),
                       lookat=np.array(meta["lookat"]), sky=np.array(meta["sky"]),
                       amap=[None if p is None else Palette(np.array(p["x"]),
                                                            np.array(p["rgb"], np.float32))
                             for p in meta["palettes"]],
                       b_brightness=meta["b_brightness"])
    return z, meta["params"], rc


def gpu_rays(renderer, params: dict, rc, particles) -> np.ndarray:
    pf = sg.ParamFile(dict(params, new_renderer="T"))
    rcx = RenderContext(campos=rc.campos, centerpos=rc.centerpos, lookat=rc.lookat, sky=rc.sky,
                        amap=rc.amap, b_brightness=rc.b_brightness)
    parts = np.ascontiguousarray(particles).copy()
    left = sg.host_rendering(pf, parts, rcx, renderer=renderer)
    assert len(left) == 0  # the reference empties its particle vector
    assert np.array_equal(parts.view(np.uint8), np.ascontiguousarray(particles).view(np.uint8))
    return rcx.pic


def with_camera_spheres(w, k: int, seed: int):
    p = w.particles
    rng = np.random.default_rng(seed)
    cam = np.asarray(w.rc.campos, np.float64)
    for i in rng.choice(len(p), k, replace=False):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        dist = rng.uniform(0.5, 5.0)
        p["x"][i], p["y"][i], p["z"][i] = cam + d * dist
        p["r"][i] = dist * rng.uniform(0.3, 2.0)
    return w


@pytest.mark.parametrize("name", CASES)
def test_golden_frames(name, renderer):
    z, prm, rc = load(name)
    p = z["particles_in"].view(PARTICLE_DTYPE)
    pic = gpu_rays(renderer, prm, rc, p)
    assert rel_linf(pic, z["render_fp64"]) <= TOL
    for branch in ("simd", "scalar"):
        assert rel_linf(pic, z[f"host_rendering_{branch}"]) <= TOL
    st = renderer.stats()
    assert st["n_active"] == z["stats"][1] + z["stats"][2]  # level grids + around the camera


@pytest.mark.parametrize("extra", [
    {},                                         # plane, 800x800, seven levels
    {"dome": "T"},                              # fisheye
    {"fov": "33.3", "minrad_pix": "2.5", "yres": "600"},
    {"zmax": "180"},                            # distance cut
])
def test_against_fp64_oracle(extra, renderer, port):
    w = with_camera_spheres(synth.plain_additive(n=120_000, seed=40), 12, 41)
    prm = dict(w.params.params, new_renderer="T", **extra)
    pic = gpu_rays(renderer, prm, w.rc, w.particles)
    want, st = port.render_rays(prm, w.rc, w.particles, exact=True)
    assert st["fragments"] > 0
    assert rel_linf(pic, want) <= TOL


@pytest.mark.parametrize("res", [3, 9, 65, 127])
def test_odd_dome_resolutions(res, renderer, port):
    """Odd fisheye sizes, where the middle pixel's direction can be exactly the
    zenith: the reference's 0/0 there gives a NaN direction, which its
    exptable turns into weight 1 for every sphere listed in the pixel's
    region, and which add_overlap2's erfc passes on (a NaN pixel when spheres
    enclose the camera, as every sphere does at 3x3)."""
    w = synth.plain_additive(n=20_000, xres=res, seed=42)
    prm = dict(w.params.params, new_renderer="T", dome="T")
    pic = gpu_rays(renderer, prm, w.rc, w.particles)
    want, _ = port.render_rays(prm, w.rc, w.particles, exact=True)
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(pic), nan)
    assert rel_linf(np.where(nan, 0, pic), np.where(nan, 0, want)) <= TOL


def test_soa_device_inputs_match_aos(renderer, port):
    torch = pytest.importorskip("torch")
    w = synth.plain_additive(n=50_000, xres=320, yres=256, seed=43)
    prm = dict(w.params.params, new_renderer="T")
    pic = gpu_rays(renderer, prm, w.rc, w.particles)
    keep: list = []
    pf = sg.ParamFile(dict(prm))
    desc = sg.frame_desc(pf, w.rc, keep)
    soa = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda()
           for k, v in synth.soa_from_aos(w.particles).items()}
    out = torch.zeros((desc.xres, desc.yres, 3), dtype=torch.float32, device="cuda")
    renderer.render_rays(desc, sg.rays_desc(pf), soa, out, device=True)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), pic)


def test_repeat_and_camera_change(renderer, port):
    """The region trees are kept while the geometry holds: a repeat gives the
    same bits, a moved camera a new (correct) frame."""
    w = synth.plain_additive(n=40_000, xres=256, seed=44)
    prm = dict(w.params.params, new_renderer="T")
    a = gpu_rays(renderer, prm, w.rc, w.particles)
    b = gpu_rays(renderer, prm, w.rc, w.particles)
    assert np.array_equal(a, b)
    w.rc.campos = np.array([60.0, 45.0, 240.0])
    w.rc.centerpos = w.rc.campos
    c = gpu_rays(renderer, prm, w.rc, w.particles)
    want, _ = port.render_rays(prm, w.rc, w.particles, exact=True)
    assert rel_linf(c, want) <= TOL
    assert not np.array_equal(a, c)


def test_empty_and_culled_frames(renderer):
    w = synth.plain_additive(n=5_000, xres=64, seed=45)
    prm = dict(w.params.params, new_renderer="T")
    pic = gpu_rays(renderer, prm, w.rc, w.particles[:0])
    assert pic.shape == (64, 64, 3) and not pic.any()
    pic = gpu_rays(renderer, dict(prm, zmax="1.0"), w.rc, w.particles)  # all beyond zmax
    assert not pic.any()


def test_errors(renderer):
    w = synth.plain_additive(n=1_000, xres=48, yres=40, seed=46)
    prm = dict(w.params.params, new_renderer="T")
    with pytest.raises(sg.SplotchError):
        gpu_rays(renderer, dict(prm, a_eq_e="F"), w.rc, w.particles)  # planck_assert(a_eq_e)
    with pytest.raises(sg.SplotchError):
        gpu_rays(renderer, dict(prm, dome="T"), w.rc, w.particles)  # 48 x 40 dome
    bad = w.particles.copy()
    bad["type"][7] = 3
    with pytest.raises(sg.SplotchError):
        gpu_rays(renderer, prm, w.rc, bad)
    # the context stays usable
    pic = gpu_rays(renderer, prm, w.rc, w.particles)
    assert pic.any()


def test_full_size_1080p(renderer, port):
    """4M particles at 1920x1080 (seven levels, ~40M leaf entries, a billion
    covered pairs) against the FP64 restatement."""
    w = with_camera_spheres(synth.plain_additive(n=4_000_000, seed=47), 20, 48)
    prm = dict(w.params.params, new_renderer="T", xres="1920", yres="1080")
    pic = gpu_rays(renderer, prm, w.rc, w.particles)
    want, st = port.render_rays(prm, w.rc, w.particles, exact=True)
    assert st["levels"] == 7 and st["n_overlap"] > 0
    assert renderer.stats()["n_entries"] > 10_000_000
    assert rel_linf(pic, want) <= TOL
