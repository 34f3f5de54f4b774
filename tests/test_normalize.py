"""sceneMaker::particle_normalize (splotch/scenemaker.cc:40-296), the step
before host_rendering: log10 / asinh transforms, per-type ranges, overrides,
normAndClamp.

CPU: the oracle's restatement against golden fixtures from the reference's own
sceneMaker (tests/golden/make_golden.py), bit for bit.  GPU: spl_particle_
normalize against the same fixtures: bit for bit where no logarithm is taken.
Where log10f / log come in (CUDA's math library against the host's, an ulp
apart at most), the normalised values in [0,1] agree to 2.4e-7 absolute (two
ulps of 1.0: an ulp of the logarithm divided by the range) and the ranges to
3e-7 relative.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import splotch_gb300 as sg
from oracle.oracle import PARTICLE_DTYPE, Port

GOLDEN = Path(__file__).resolve().parent / "golden"
VARIANTS = ("plain", "logs", "asinh_overrides", "vector_log")
FIELDS = ("I", "er", "eg", "eb")


def _golden():
    return np.load(GOLDEN / "norm_absorption.npz")


def _particles(raw):
    return np.frombuffer(raw.tobytes(), dtype=PARTICLE_DTYPE).copy()


@pytest.mark.parametrize("var", VARIANTS)
def test_oracle_normalize_matches_reference(var, built):
    g = _golden()
    prm = json.loads(bytes(g[f"params_{var}"]).decode())
    p = _particles(g["particles_in"])
    res = Port().particle_normalize(prm, p)
    want = _particles(g[f"particles_{var}"])
    for f in FIELDS + ("x", "y", "z", "r", "type"):
        assert np.array_equal(p[f], want[f], equal_nan=True) if p[f].dtype.kind == "f" \
            else np.array_equal(p[f], want[f]), (var, f)
    rng = g[f"ranges_{var}"]  # range_min, range_max, clamp_min, clamp_max (text round trip)
    got = np.array([res[k] for k in ("range_min", "range_max", "clamp_min", "clamp_max")])
    np.testing.assert_allclose(got, rng, rtol=1e-7)


@pytest.mark.gpu
@pytest.mark.parametrize("var", VARIANTS)
def test_gpu_normalize_matches_reference(var, renderer):
    g = _golden()
    prm = json.loads(bytes(g[f"params_{var}"]).decode())
    p = _particles(g["particles_in"])
    params = sg.ParamFile(prm)
    res = sg.particle_normalize(params, p, renderer)
    want = _particles(g[f"particles_{var}"])
    uses_log = any(k.startswith(("intensity_log", "color_log", "color_asinh")) for k in prm)
    for f in FIELDS:
        if uses_log:
            d = np.abs(p[f].astype(np.float64) - want[f].astype(np.float64))
            assert np.nanmax(d) <= 2.4e-7, (var, f, float(np.nanmax(d)))
            assert np.array_equal(np.isnan(p[f]), np.isnan(want[f])), (var, f)
        else:
            assert np.array_equal(p[f], want[f]), (var, f)
    for f in ("x", "y", "z", "r", "type"):
        assert np.array_equal(p[f], want[f]), (var, f)
    rng = g[f"ranges_{var}"]
    got = np.array([res[k] for k in ("range_min", "range_max", "clamp_min", "clamp_max")])
    finite = np.isfinite(rng)
    np.testing.assert_allclose(got[finite], rng[finite], rtol=3e-7)
    assert np.array_equal(np.isfinite(got), finite)
    assert params.find("clamp_max0", 0.0) == pytest.approx(res["clamp_max"][0])


@pytest.mark.gpu
def test_gpu_normalize_device_soa_equals_host_aos(renderer):
    torch = pytest.importorskip("torch")
    g = _golden()
    prm = json.loads(bytes(g["params_logs"]).decode())
    p = _particles(g["particles_in"])
    dev = torch.from_numpy(p.view(np.uint8).copy()).cuda()
    torch.cuda.synchronize()
    sg.particle_normalize(sg.ParamFile(dict(prm)), dev, renderer, device=True)
    sg.particle_normalize(sg.ParamFile(dict(prm)), p, renderer)
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy(), p.view(np.uint8))
