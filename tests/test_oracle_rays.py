"""The oracle restatement of the ray-sphere renderer (oracle/spl_oracle_rays.c,
host_rendering_new of splotch/new_renderer.cc:522-641) pinned to the
reference's own outputs in tests/golden/rays_*.npz.

Bit-exact: the whole image in the reference's arithmetic (exptable<double>
weights, float sums) against both compiled branches of the reference.  The
FP64 restatement (exact exp, double sums) stays within the reference's own
table error of it.  CPU only."""
import json
import platform
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import PARTICLE_DTYPE, rel_linf
from splotch_gb300 import Palette, RenderContext

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("rays_*.npz"))
X86 = platform.machine() in ("x86_64", "AMD64")


def load(name):
    z = np.load(GOLDEN / f"{name}.npz")
    meta = json.loads(bytes(z["meta"]).decode())
    rc = RenderContext(campos=np.array(meta["campos"]), centerpos=np.array(meta["centerpos"]),
                       lookat=np.array(meta["lookat"]), sky=np.array(meta["sky"]),
                       amap=[None if p is None else Palette(np.array(p["x"]), np.array(p["rgb"]))
                             for p in meta["palettes"]],
                       b_brightness=meta["b_brightness"])
    return z, meta["params"], rc


def test_fixtures_present():
    assert set(CASES) >= {"rays_plane", "rays_dome", "rays_two_types", "rays_tiny"}


@pytest.mark.parametrize("branch", ["simd", "scalar"])
@pytest.mark.parametrize("name", CASES)
def test_reference_arithmetic_bitexact(name, branch, port):
    z, prm, rc = load(name)
    p = z["particles_in"].view(PARTICLE_DTYPE)
    pic, st = port.render_rays(prm, rc, p, exact=False)
    want = z[f"host_rendering_{branch}"]
    if X86:
        assert np.array_equal(pic.view(np.uint32), want.view(np.uint32))
    else:  # libm tan/sin/cos/atan2/erfc may round differently off x86
        assert rel_linf(pic, want) <= 1e-6
    assert list(z["stats"]) == [st[k] for k in ("n_used", "n_grid", "n_overlap", "levels",
                                                "fragments")]


@pytest.mark.parametrize("name", CASES)
def test_fp64_restatement(name, port):
    z, prm, rc = load(name)
    p = z["particles_in"].view(PARTICLE_DTYPE)
    pic64, _ = port.render_rays(prm, rc, p, exact=True)
    assert rel_linf(pic64, z["render_fp64"]) <= (0.0 if X86 else 1e-12)
    # the reference's exptable quantisation (20/2^20 in the exponent) bounds
    # its own distance from exact weights
    assert rel_linf(z["host_rendering_simd"], pic64) <= 3e-5


def test_overlap_and_levels_exercised():
    """The fixtures reach the paths that matter: spheres around the camera,
    several pyramid levels, a grid smaller than one leaf region."""
    st = {n: np.load(GOLDEN / f"{n}.npz")["stats"] for n in CASES}
    assert st["rays_plane"][2] > 0 and st["rays_dome"][2] > 0
    assert st["rays_plane"][3] > 1 and st["rays_two_types"][3] > 1
    assert st["rays_two_types"][0] < 4000  # the distance cut removed some


def test_errors(port):
    z, prm, rc = load("rays_plane")
    p = z["particles_in"].view(PARTICLE_DTYPE)
    with pytest.raises(ValueError):
        port.render_rays(dict(prm, a_eq_e="F"), rc, p)
    with pytest.raises(ValueError):
        port.render_rays(dict(prm, dome="T"), rc, p)  # 96 x 80 dome
