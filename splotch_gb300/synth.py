"""Seeded synthetic particle sets ("halo mixture") and the workload configs.

The reference's demo snapshot is not available, so every workload is drawn
from one generator: 64 halo centres uniform in [0,L]^3 with sigma log-uniform
in [0.5,5]*L/100; 70% of the particles sit in a halo chosen uniformly at
random (isotropic normal around its centre), 30% are uniform in the box.
numpy ``Generator(PCG64(seed))`` throughout, so the CPU oracle and the GPU
path read identical inputs.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import PARTICLE_DTYPE, Palette, ParamFile, RenderContext


def halo_positions(rng: np.random.Generator, n: int, L: float) -> np.ndarray:
    centres = rng.uniform(0.0, L, size=(64, 3))
    sig = np.exp(rng.uniform(np.log(0.5), np.log(5.0), size=64)) * (L / 100.0)
    nh = int(round(0.7 * n))
    which = rng.integers(0, 64, size=nh)
    pos = np.empty((n, 3), dtype=np.float32)
    pos[:nh] = centres[which] + rng.standard_normal((nh, 3)) * sig[which, None]
    pos[nh:] = rng.uniform(0.0, L, size=(n - nh, 3))
    return pos


def blue_white_palette(n: int = 256) -> Palette:
    """n-entry linear blue (0,0,1) -> white (1,1,1), as a .pal file would store it."""
    v = np.round(np.linspace(0, 255, n))
    return Palette.from_rgb255(np.stack([v, v, np.full(n, 255.0)], axis=1))


def five_stop_palette(n: int = 256) -> Palette:
    """n entries interpolated through 5 stops: black, deep blue, cyan, orange, white."""
    stops = np.array([[0, 0, 0], [20, 30, 150], [40, 200, 230], [255, 170, 40], [255, 255, 255]],
                     dtype=np.float64)
    t = np.linspace(0, 4, n)
    i = np.minimum(t.astype(int), 3)
    f = (t - i)[:, None]
    return Palette.from_rgb255(np.round(stops[i] * (1 - f) + stops[i + 1] * f))


@dataclass
class Workload:
    name: str
    particles: np.ndarray
    params: ParamFile
    rc: RenderContext
    notes: dict = field(default_factory=dict)


def _rc(campos, lookat, amap, b_brightness=1.0, sky=(0.0, 1.0, 0.0)) -> RenderContext:
    c = np.asarray(campos, dtype=np.float64)
    return RenderContext(campos=c, centerpos=c.copy(), lookat=np.asarray(lookat, np.float64),
                         sky=np.asarray(sky, np.float64), amap=amap, b_brightness=b_brightness)


def plain_additive(n: int = 1_000_000, seed: int = 0, xres: int = 800, yres: int | None = None,
                   tile: int = 16) -> Workload:
    """Plain render, additive: halo mixture in [0,100]^3, hsml ~ lognormal(ln 0.3, 0.5),
    I ~ lognormal(0,1), colour value U[0,1] through a 256-entry blue->white palette,
    camera (50,50,250) -> (50,50,50), fov 30."""
    rng = np.random.Generator(np.random.PCG64(seed))
    p = np.zeros(n, dtype=PARTICLE_DTYPE)
    pos = halo_positions(rng, n, 100.0)
    p["x"], p["y"], p["z"] = pos[:, 0], pos[:, 1], pos[:, 2]
    p["r"] = rng.lognormal(np.log(0.3), 0.5, n).astype(np.float32)
    p["I"] = rng.lognormal(0.0, 1.0, n).astype(np.float32)
    p["er"] = rng.uniform(0.0, 1.0, n).astype(np.float32)
    yres = xres if yres is None else yres
    params = ParamFile({"xres": xres, "yres": yres, "fov": 30.0, "a_eq_e": True,
                        "brightness0": 1.0, "tile_size_cpu": tile, "ptypes": 1})
    return Workload("plain_additive", p, params,
                    _rc((50, 50, 250), (50, 50, 50), [blue_white_palette()]))


def plain_absorption(n_gas: int = 40_000_000, n_star: int = 10_000_000, seed: int = 1,
                     xres: int = 1920, yres: int = 1080, tile: int = 16,
                     order: str = "ftb") -> Workload:
    """Plain render, ordered emission-absorption: gas (type 0) + stars (type 1) in
    [0,500]^3.  Gas hsml ~ lognormal(0,0.7), I ~ lognormal(0,1), colour value U[0,1]
    through a 256-entry 5-stop palette; stars hsml 0.2, RGB U[0,1]^3 (colour vector),
    I ~ lognormal(0,1).  Camera (250,250,-50) -> (250,250,250), sky +y, fov 45."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = n_gas + n_star
    p = np.zeros(n, dtype=PARTICLE_DTYPE)
    pos = halo_positions(rng, n, 500.0)
    p["x"], p["y"], p["z"] = pos[:, 0], pos[:, 1], pos[:, 2]
    p["r"][:n_gas] = rng.lognormal(0.0, 0.7, n_gas).astype(np.float32)
    p["r"][n_gas:] = np.float32(0.2)
    p["I"] = rng.lognormal(0.0, 1.0, n).astype(np.float32)
    p["er"][:n_gas] = rng.uniform(0.0, 1.0, n_gas).astype(np.float32)
    rgb = rng.uniform(0.0, 1.0, (n_star, 3)).astype(np.float32)
    p["er"][n_gas:], p["eg"][n_gas:], p["eb"][n_gas:] = rgb[:, 0], rgb[:, 1], rgb[:, 2]
    p["type"][n_gas:] = 1
    params = ParamFile({"xres": xres, "yres": yres, "fov": 45.0, "a_eq_e": False,
                        "sort_type": 1, "gray_absorption": 0.2, "ptypes": 2,
                        "color_is_vector0": False, "color_is_vector1": True,
                        "brightness0": 1.0, "brightness1": 1.0, "tile_size_cpu": tile,
                        "gpu_order": order})
    return Workload("plain_absorption", p, params,
                    _rc((250, 250, -50), (250, 250, 250), [five_stop_palette(), None]))


def differentiable(n: int = 4_000_000, mode: str = "additive", seed: int = 3, xres: int = 1024,
                   yres: int | None = None, tile: int = 16, order: str = "ftb") -> Workload:
    """Differentiable render: halo mixture in [0,100]^3, hsml ~ lognormal(ln 0.3, 0.5),
    I ~ lognormal(0,1); three quarters of the particles take a colour value U[0,1]
    through the 256-entry blue->white palette (type 0), one quarter a per-particle
    RGB U[0,1]^3 (type 1, colour vector).  Camera (50,50,250) -> (50,50,50), fov 30.
    notes["target"] holds the target particle set: I scaled by lognormal(0,0.2)
    noise and positions moved by N(0, 0.1*hsml)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    p = np.zeros(n, dtype=PARTICLE_DTYPE)
    pos = halo_positions(rng, n, 100.0)
    p["x"], p["y"], p["z"] = pos[:, 0], pos[:, 1], pos[:, 2]
    p["r"] = rng.lognormal(np.log(0.3), 0.5, n).astype(np.float32)
    p["I"] = rng.lognormal(0.0, 1.0, n).astype(np.float32)
    nv = n // 4
    p["type"][n - nv:] = 1
    p["er"] = rng.uniform(0.0, 1.0, n).astype(np.float32)
    rgb = rng.uniform(0.0, 1.0, (nv, 2)).astype(np.float32)
    p["eg"][n - nv:], p["eb"][n - nv:] = rgb[:, 0], rgb[:, 1]
    t = p.copy()
    t["I"] = (p["I"] * rng.lognormal(0.0, 0.2, n)).astype(np.float32)
    for ax in ("x", "y", "z"):
        t[ax] = (p[ax] + rng.standard_normal(n) * 0.1 * p["r"]).astype(np.float32)
    yres = xres if yres is None else yres
    additive = mode == "additive"
    params = ParamFile({"xres": xres, "yres": yres, "fov": 30.0, "a_eq_e": additive,
                        "sort_type": 1, "gray_absorption": 0.2, "ptypes": 2,
                        "color_is_vector0": False, "color_is_vector1": True,
                        "brightness0": 1.0, "brightness1": 1.0, "tile_size_cpu": tile,
                        "gpu_order": order})
    return Workload(f"differentiable_{mode}", p, params,
                    _rc((50, 50, 250), (50, 50, 50), [blue_white_palette(), None]),
                    notes={"target": t})


def large(n: int = 400_000_000, seed: int = 4, xres: int = 4096, tile: int = 16,
          order: str = "ftb", chunk: int = 25_000_000) -> Workload:
    """Large render, forward+backward: halo mixture in [0,1000]^3, ordered
    absorption, per-particle RGB U[0,1]^3 (colour vector), I ~ lognormal(0,1),
    hsml ~ Pareto(alpha=1.5, x_min=0.1) clipped so that no particle's pixel
    radius exceeds a quarter of the image width at its depth.  Camera
    (500,500,2500) -> (500,500,500), fov 30, xres x xres: ~3.8 pixels per unit
    at the box centre, so about 0.1% of the particles (hsml > ~10) cover more
    than 10^4 pixels.  Generated in chunks to bound host memory."""
    rng = np.random.Generator(np.random.PCG64(seed))
    p = np.zeros(n, dtype=PARTICLE_DTYPE)
    res2 = 0.5 * xres
    fovfct = np.tan(np.radians(30.0) / 2)
    for lo in range(0, n, chunk):
        m = min(chunk, n - lo)
        pos = halo_positions(rng, m, 1000.0)
        s = p[lo:lo + m]
        s["x"], s["y"], s["z"] = pos[:, 0], pos[:, 1], pos[:, 2]
        h = 0.1 * (1.0 - rng.uniform(0.0, 1.0, m)) ** (-1.0 / 1.5)  # Pareto(1.5, 0.1)
        depth = np.maximum(2500.0 - pos[:, 2].astype(np.float64), 1.0)
        hmax = (xres / 4) * fovfct * depth / (2.0 * res2)  # R = 2 h res2/(fovfct depth)
        s["r"] = np.minimum(h, hmax).astype(np.float32)
        s["I"] = rng.lognormal(0.0, 1.0, m).astype(np.float32)
        rgb = rng.uniform(0.0, 1.0, (m, 3)).astype(np.float32)
        s["er"], s["eg"], s["eb"] = rgb[:, 0], rgb[:, 1], rgb[:, 2]
    params = ParamFile({"xres": xres, "yres": xres, "fov": 30.0, "a_eq_e": False,
                        "sort_type": 1, "gray_absorption": 0.2, "ptypes": 1,
                        "color_is_vector0": True, "brightness0": 1.0, "tile_size_cpu": tile,
                        "gpu_order": order})
    return Workload("large", p, params, _rc((500, 500, 2500), (500, 500, 500), [None]),
                    notes={"hsml": "Pareto(1.5, 0.1), pixel radius <= xres/4"})


BATCH_RESOLUTIONS = ((512, 512), (1024, 1024), (1920, 1080), (2048, 2048))


@dataclass
class BatchWorkload:
    sets: list            # particle_sim arrays, one per set
    frames: list          # (set index, ParamFile, RenderContext)
    notes: dict = field(default_factory=dict)


def batched(n_sets: int = 8, poses: int = 12, seed: int = 2, scale: float = 1.0,
            tile: int = 16, order: str = "ftb",
            resolutions=BATCH_RESOLUTIONS) -> BatchWorkload:
    """Batched rendering: n_sets particle sets with N log-uniform in [1M, 32M]
    (times scale), alternating additive / ordered absorption, each from the halo
    mixture in [0,100]^3 (hsml ~ lognormal(ln 0.3, 0.5), I ~ lognormal(0,1);
    three quarters colour value through a palette -- blue->white for additive
    sets, 5-stop for ordered ones --, one quarter per-particle RGB), and
    `poses` camera poses per set on a circular orbit of radius 2L = 200 in the
    xz plane around the box centre, looking at the centre (sky +y), fov
    U[30, 60] degrees, resolution drawn from `resolutions`."""
    rng = np.random.Generator(np.random.PCG64(seed))
    L = 100.0
    centre = np.array([L / 2, L / 2, L / 2])
    sets, frames = [], []
    for s in range(n_sets):
        n = max(1, int(round(np.exp(rng.uniform(np.log(1e6), np.log(32e6))) * scale)))
        additive = s % 2 == 0
        prng = np.random.Generator(np.random.PCG64(seed * 1000 + s))
        p = np.zeros(n, dtype=PARTICLE_DTYPE)
        pos = halo_positions(prng, n, L)
        p["x"], p["y"], p["z"] = pos[:, 0], pos[:, 1], pos[:, 2]
        p["r"] = prng.lognormal(np.log(0.3), 0.5, n).astype(np.float32)
        p["I"] = prng.lognormal(0.0, 1.0, n).astype(np.float32)
        nv = n // 4
        p["type"][n - nv:] = 1
        p["er"] = prng.uniform(0.0, 1.0, n).astype(np.float32)
        rgb = prng.uniform(0.0, 1.0, (nv, 2)).astype(np.float32)
        p["eg"][n - nv:], p["eb"][n - nv:] = rgb[:, 0], rgb[:, 1]
        sets.append(p)
        pal = blue_white_palette() if additive else five_stop_palette()
        phase = rng.uniform(0.0, 2 * np.pi)
        for k in range(poses):
            a = phase + 2 * np.pi * k / poses
            campos = centre + 2 * L * np.array([np.sin(a), 0.0, np.cos(a)])
            xres, yres = resolutions[int(rng.integers(0, len(resolutions)))]
            fov = float(rng.uniform(30.0, 60.0))
            params = ParamFile({"xres": xres, "yres": yres, "fov": fov, "a_eq_e": additive,
                                "sort_type": 1, "gray_absorption": 0.2, "ptypes": 2,
                                "color_is_vector0": False, "color_is_vector1": True,
                                "brightness0": 1.0, "brightness1": 1.0, "tile_size_cpu": tile,
                                "gpu_order": order})
            frames.append((s, params, _rc(campos, centre, [pal, None])))
    return BatchWorkload(sets, frames, notes={"particles": sum(len(p) for p in sets)})


def soa_from_aos(p: np.ndarray) -> dict:
    """Split a particle_sim array into the SoA fields the C ABI takes."""
    return {"x": np.ascontiguousarray(p["x"]), "y": np.ascontiguousarray(p["y"]),
            "z": np.ascontiguousarray(p["z"]), "r": np.ascontiguousarray(p["r"]),
            "I": np.ascontiguousarray(p["I"]), "cr": np.ascontiguousarray(p["er"]),
            "cg": np.ascontiguousarray(p["eg"]), "cb": np.ascontiguousarray(p["eb"]),
            "type": np.ascontiguousarray(p["type"])}
