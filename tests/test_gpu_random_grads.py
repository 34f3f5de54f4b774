"""Gradients of seeded random differentiable frames against the oracle's FP64
adjoint.

Each case draws a resolution, a tile size, the mode (additive, or ordered
absorption rendered front to back with the relative cut) and a camera around
the box; the forward keeps optical depths and stop positions, the backward of
L = sum((pic - target)^2) must match the FP64 adjoint field by field within the
bounds of test_gpu_grad (max-normalised L-inf, median and floored element
error), and the camera-position gradient within the same L-inf bound.
"""
import numpy as np
import pytest

from splotch_gb300 import synth

from .test_gpu_grad import (FIELDS, GRAD_TOL, _frame, _gpu_matrix, _oracle_inputs,
                            check_field, describe)

pytestmark = pytest.mark.gpu


def _case(seed: int):
    rng = np.random.default_rng(2000 + seed)
    mode = str(rng.choice(["additive", "absorption"]))
    xres = int(rng.integers(96, 257))
    yres = int(rng.integers(96, 257))
    tile = int(rng.choice([8, 12, 16, 32]))
    w = synth.differentiable(n=20_000, mode=mode, seed=seed, xres=xres, yres=yres, tile=tile)
    c = np.full(3, 50.0)  # the differentiable workload's box is [0,100]^3
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    w.rc.campos = c + d * float(rng.uniform(120.0, 220.0))
    w.rc.centerpos = w.rc.campos.copy()
    w.rc.lookat = c + rng.normal(size=3) * 3.0
    w.rc.sky = np.array([0.0, 1.0, 0.0]) if abs(d[1]) < 0.9 else np.array([1.0, 0.0, 0.0])
    return mode, w


@pytest.mark.parametrize("seed", range(6))
def test_random_frame_gradients(seed, renderer, port):
    mode, w = _case(seed)
    _, _, gpic, grads = _frame(renderer, w, w.notes["target"])
    prm, raw, cov, order = _oracle_inputs(port, w)
    g64, gc64 = port.grad_fp64(prm, w.rc, raw, cov, order, gpic.astype(np.float64))
    g32 = _gpu_matrix(grads, len(raw))
    act = cov["active"].astype(bool)
    assert act.sum() >= 200, act.sum()
    assert np.all(g32[~act] == 0.0)
    bad = []
    for j, f in enumerate(FIELDS):
        print(seed, mode, f, describe(g32[act, j], g64[act, j]))
        bad += check_field(g32[act, j], g64[act, j], f)
    assert not bad, bad
    ec = np.abs(grads["campos"] - gc64).max() / np.abs(gc64).max()
    assert ec <= GRAD_TOL, ec
