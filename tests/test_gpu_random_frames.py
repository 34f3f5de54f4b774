"""Seeded random frames against the oracle.

Each case draws a resolution (odd sizes, partial edge tiles), a tile size, the
mode (additive, or ordered emission-absorption with a sort type and a
compositing order), a camera around the box and a particle mixture: the halo
generator's particles, a few very large ones (the many-tile path), a few behind
the camera and a few far off-screen.  Projection, visiting order, tile bins and
the fragment count must equal the oracle's bit for bit and the image must be
within the stated tolerance of the FP64 oracle -- the same bar as the other
parity tests, over combinations the hand-written cases do not reach.
"""
import numpy as np
import pytest

from splotch_gb300 import synth

from .helpers import assert_parity, gpu_frame, oracle_frame

pytestmark = pytest.mark.gpu


def _case(seed: int):
    rng = np.random.default_rng(1000 + seed)
    xres = int(rng.integers(33, 301))
    yres = int(rng.integers(33, 301))
    tile = int(rng.choice([8, 12, 16, 32]))
    additive = bool(rng.random() < 0.4)
    if additive:
        w = synth.plain_additive(n=6000, seed=seed, xres=xres, yres=yres, tile=tile)
        box = 100.0
    else:
        w = synth.plain_absorption(n_gas=5000, n_star=1000, seed=seed, xres=xres, yres=yres,
                                   tile=tile, order=str(rng.choice(["ftb", "btf"])))
        box = 500.0
    prm = dict(w.params.params)
    if not additive:
        prm["sort_type"] = int(rng.choice([1, 2, 3, 4]))
    prm["fov"] = float(rng.uniform(25.0, 70.0))
    # camera on a sphere around the box centre, looking near the centre
    c = np.full(3, 0.5 * box)
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    w.rc.campos = c + d * box * float(rng.uniform(0.9, 2.0))
    w.rc.centerpos = w.rc.campos.copy()
    w.rc.lookat = c + rng.normal(size=3) * 0.05 * box
    w.rc.sky = np.array([0.0, 1.0, 0.0]) if abs(d[1]) < 0.9 else np.array([1.0, 0.0, 0.0])
    p = w.particles
    k = len(p)
    big = rng.choice(k, 6, replace=False)
    p["r"][big] *= np.float32(rng.uniform(30.0, 120.0))  # many-tile footprints
    far = rng.choice(k, 6, replace=False)
    p["x"][far] += np.float32(5.0 * box)  # off-screen or behind the camera
    return prm, w.rc, p


@pytest.mark.parametrize("seed", range(16))
def test_random_frame(seed, renderer, port):
    prm, rc, p = _case(seed)
    g = gpu_frame(renderer, prm, rc, p)
    o = oracle_frame(port, prm, rc, p, fp32=False)
    assert_parity(g, o)
