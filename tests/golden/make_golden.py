"""Generate the golden fixtures from the reference's own compiled code.

Runs where the reference sources are available: builds oracle/_ref with
oracle/build_ref.sh, runs the reference's particle_project + particle_colorize,
render_new and host_rendering on small seeded inputs, and stores inputs and
outputs under tests/golden/*.npz.  The CPU tests pin the oracle restatement to
these files; the GPU tests compare the CUDA path with them.

    python tests/golden/make_golden.py          # every fixture
    python tests/golden/make_golden.py rays     # the ray-sphere renderer's only
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle  # noqa: E402
from splotch_gb300 import RenderContext, synth  # noqa: E402

OUT = Path(__file__).resolve().parent


def cases():
    yield "additive", synth.plain_additive(n=3000, xres=96, yres=80, tile=16)
    yield "absorption", synth.plain_absorption(n_gas=2400, n_star=600, xres=96, yres=54,
                                               tile=16, order="btf")
    w = synth.plain_additive(n=2500, xres=72, yres=90, tile=12, seed=7)
    w.params.params.update({"projection": "F", "zmin": "185.0", "zmax": "232.5",
                            "minrad_pix": "2.5", "smooth_factor0": "1.7",
                            "brightness0": "0.6", "fov": "38.0"})
    w.rc.b_brightness = 1.3
    yield "variants_orthographic", w
    w = synth.plain_absorption(n_gas=2000, n_star=500, xres=80, yres=80, tile=10, seed=9)
    w.rc.campos = np.array([620.0, 430.0, -180.0])
    w.rc.centerpos = np.array([600.0, 420.0, -170.0])
    w.rc.lookat = np.array([250.0, 240.0, 260.0])
    w.rc.sky = np.array([0.1, 1.0, 0.2])
    w.params.params.update({"gray_absorption": "0.35", "brightness1": "2.0"})
    yield "tilted_camera_center", w


def main() -> int:
    if not oracle.build_ref():
        print("reference sources not available; fixtures unchanged")
        return 1
    if sys.argv[1:] == ["rays"]:
        rays_cases(oracle.Ref(scalar=False), oracle.Ref(scalar=True), oracle.Port())
        return 0
    refs = {"simd": oracle.Ref(scalar=False), "scalar": oracle.Ref(scalar=True)}
    port = oracle.Port()
    for name, w in cases():
        prm = dict(w.params.params)
        rc: RenderContext = w.rc
        xres, yres = int(prm["xres"]), int(prm.get("yres", prm["xres"]))
        T = int(float(prm["tile_size_cpu"]))
        a_eq_e = prm.get("a_eq_e", "T") in ("T", "True", "true")
        gray = float(prm.get("gray_absorption", 0.2))
        out = {"particles_in": w.particles.view(np.uint8).copy()}
        proj = w.particles.copy()
        refs["simd"].project_colorize(prm, rc, proj)
        out["projected"] = proj.view(np.uint8).copy()
        perm = port.sort_perm(proj, int(prm.get("sort_type", 1))) if not a_eq_e else None
        ordered = proj[perm].copy() if perm is not None else proj.copy()
        if perm is not None:
            out["stable_perm"] = perm
        for br, ref in refs.items():
            out[f"render_new_{br}"] = ref.render_new(ordered.copy(), xres, yres, a_eq_e, gray, T)
            out[f"host_rendering_{br}"] = ref.host_rendering(prm, rc, w.particles.copy())
        pic64, frags = port.render_fp64(proj, perm, xres, yres, T, a_eq_e, gray)
        out["render_fp64"] = pic64
        out["fragments"] = np.array(frags)
        meta = {"params": prm, "campos": list(rc.campos), "centerpos": list(rc.centerpos),
                "lookat": list(rc.lookat), "sky": list(rc.sky), "b_brightness": rc.b_brightness,
                "palettes": [None if p is None else {"x": p.x.tolist(), "rgb": p.rgb.tolist()}
                             for p in rc.amap]}
        out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        np.savez_compressed(OUT / f"{name}.npz", **out)
        print(f"{name}: {len(w.particles)} particles, {int(proj['active'].sum())} active, "
              f"{frags} fragments")
    post_cases(refs["simd"])
    norm_cases(refs["simd"])
    rays_cases(refs["simd"], refs["scalar"], port)
    return 0


def with_camera_spheres(w, k: int, seed: int):
    """k particles moved next to the camera with radii that enclose it: the
    spheres host_rendering_new renders through add_overlap2."""
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


def rays_inputs():
    """Seeded frames for host_rendering with new_renderer=true
    (new_renderer.cc:522-641): plane and dome projectors, spheres around the
    camera, a tilted camera with centerpos != campos, a distance cut and two
    particle types, and a grid smaller than one leaf region."""
    w = with_camera_spheres(synth.plain_additive(n=4000, xres=96, yres=80, tile=16, seed=21), 6,
                            31)
    w.params.params.update({"fov": "33.3", "minrad_pix": "1.5"})
    yield "rays_plane", w
    w = with_camera_spheres(synth.plain_additive(n=4000, xres=72, tile=16, seed=22), 6, 32)
    w.rc.sky = np.array([0.1, 2.0, 0.3])
    w.params.params.update({"dome": "T"})
    yield "rays_dome", w
    w = synth.plain_absorption(n_gas=3000, n_star=1000, xres=80, yres=64, tile=16, seed=23)
    w.rc.campos = np.array([620.0, 430.0, -180.0])
    w.rc.centerpos = np.array([600.0, 420.0, -170.0])
    w.rc.lookat = np.array([250.0, 240.0, 260.0])
    w.rc.sky = np.array([0.1, 1.0, 0.2])
    w.rc.b_brightness = 0.7
    w.params.params.update({"a_eq_e": "T", "zmax": "900.0", "brightness1": "2.0",
                            "fov": "41.5"})
    yield "rays_two_types", w
    w = synth.plain_additive(n=1500, xres=7, yres=5, tile=16, seed=24)
    yield "rays_tiny", w


def rays_cases(ref, ref_scalar, port) -> None:
    """The reference's own host_rendering_new (both compiled branches) and the
    FP64 restatement on the same inputs."""
    for name, w in rays_inputs():
        prm = dict(w.params.params)
        prm["new_renderer"] = "T"
        rc: RenderContext = w.rc
        out = {"particles_in": w.particles.view(np.uint8).copy()}
        out["host_rendering_simd"] = ref.host_rendering(prm, rc, w.particles.copy())
        out["host_rendering_scalar"] = ref_scalar.host_rendering(prm, rc, w.particles.copy())
        pic64, st = port.render_rays(prm, rc, w.particles, exact=True)
        out["render_fp64"] = pic64
        out["stats"] = np.array([st[k] for k in ("n_used", "n_grid", "n_overlap", "levels",
                                                 "fragments")])
        meta = {"params": prm, "campos": list(rc.campos), "centerpos": list(rc.centerpos),
                "lookat": list(rc.lookat), "sky": list(rc.sky), "b_brightness": rc.b_brightness,
                "palettes": [None if p is None else {"x": p.x.tolist(), "rgb": p.rgb.tolist()}
                             for p in rc.amap]}
        out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        np.savez_compressed(OUT / f"{name}.npz", **out)
        print(f"{name}: {len(w.particles)} particles, {st}")


NORM_VARIANTS = {
    "plain": {},
    "logs": {"intensity_log0": "T", "intensity_log1": "T", "color_log0": "T"},
    "asinh_overrides": {"color_asinh0": "T", "color_asinh1": "T", "intensity_min0": "-1.5",
                        "color_max1": "0.8"},
    "vector_log": {"color_log1": "T", "color_min0": "0.25", "intensity_max1": "2.0"},
}


def norm_inputs():
    """A two-type set with zero / negative values where the logs must skip them."""
    w = synth.plain_absorption(n_gas=6000, n_star=2000, xres=96, yres=54, tile=16, seed=5)
    p = w.particles.copy()
    p["I"][::97] = 0.0
    p["er"][::89] = -0.5
    p["eg"][-50:] = 0.0
    return dict(w.params.params), p


def norm_cases(ref) -> None:
    """sceneMaker::particle_normalize (scenemaker.cc:40-296) from the reference's
    own code: normalised particles and the range/clamp keys it sets."""
    base, p = norm_inputs()
    out = {"particles_in": p.view(np.uint8).copy()}
    for var, extra in NORM_VARIANTS.items():
        prm = dict(base)
        prm.update(extra)
        q = p.copy()
        res = ref.particle_normalize(prm, q)
        out[f"particles_{var}"] = q.view(np.uint8).copy()
        out[f"ranges_{var}"] = np.array([res[k] for k in ("range_min", "range_max",
                                                          "clamp_min", "clamp_max")])
        out[f"params_{var}"] = np.frombuffer(json.dumps(prm).encode(), dtype=np.uint8)
    np.savez_compressed(OUT / "norm_absorption.npz", **out)
    print("norm_absorption:", len(p), "particles")


POST_VARIANTS = {
    "plain": {},
    "adjusted": {"pic_gamma": "0.8", "pic_brightness": "0.05", "pic_contrast": "1.3",
                 "colorbar": "T"},
}


def post_cases(ref) -> None:
    """splotch.cc:272-323 after host_rendering: -expm1 (additive frames),
    colour_adjust, colour bar, and the TGA / PPM / run-length TGA bytes of the
    result, from the reference's own code on the host_rendering images above."""
    import tempfile

    for name in ("additive", "absorption"):
        g = np.load(OUT / f"{name}.npz")
        meta = json.loads(bytes(g["meta"]).decode())
        prm = dict(meta["params"])
        a_eq_e = prm.get("a_eq_e", "T") in ("T", "True", "true")
        pic = g["host_rendering_simd"].astype(np.float32)
        if a_eq_e:  # a few pre-exp values across the whole exptable range
            rng = np.random.default_rng(11)
            pic[:3] = rng.uniform(-25.0, 0.0, pic[:3].shape).astype(np.float32)
            pic[3:5] = rng.uniform(-0.005, 0.0, pic[3:5].shape).astype(np.float32)
        rc = _rc_from_meta(meta)
        out = {"pic_in": pic, "meta": g["meta"]}
        with tempfile.TemporaryDirectory() as d:
            for var, extra in POST_VARIANTS.items():
                q = dict(prm)
                q.update(extra)
                res = ref.postprocess(q, rc, pic, a_eq_e)
                out[f"post_{var}"] = res
                for pt in (0, 2, 3):
                    out[f"bytes_{var}_{pt}"] = np.frombuffer(ref.image_bytes(res, pt, d),
                                                             dtype=np.uint8)
        np.savez_compressed(OUT / f"post_{name}.npz", **out)
        print(f"post_{name}: {pic.shape[0]}x{pic.shape[1]}")


def _rc_from_meta(meta) -> RenderContext:
    from splotch_gb300 import Palette

    pals = [None if p is None else Palette(np.array(p["x"]), np.array(p["rgb"], np.float32))
            for p in meta["palettes"]]
    return RenderContext(campos=np.array(meta["campos"]), centerpos=np.array(meta["centerpos"]),
                         lookat=np.array(meta["lookat"]), sky=np.array(meta["sky"]), amap=pals,
                         b_brightness=meta["b_brightness"])


if __name__ == "__main__":
    sys.exit(main())
