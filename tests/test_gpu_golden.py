"""The CUDA path against the golden fixtures made from the reference's own
compiled code (tests/golden/make_golden.py): bit-exact projection and
colourisation, the stable visiting order of active particles, the exact
fragment count, and the image within 1e-4 of the FP64 oracle image."""
import numpy as np
import pytest

import splotch_gb300 as sg
from oracle.oracle import PARTICLE_DTYPE, rel_linf

from .helpers import IMAGE_TOL
from .test_oracle_golden import CASES, load

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("order", ["btf", "ftb"])
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_golden(name, order, renderer):
    z, prm, rc = load(name)
    prm = dict(prm, gpu_order=order)
    parts = z["particles_in"].view(PARTICLE_DTYPE).copy()
    keep: list = []
    desc = sg.frame_desc(sg.ParamFile(prm), rc, keep)
    pic = np.zeros((desc.xres, desc.yres, 3), np.float32)
    renderer.render_aos(desc, parts, pic)
    proj = renderer.projected(len(parts))
    assert np.array_equal(proj.view(np.uint8), z["projected"])
    want = z["projected"].view(PARTICLE_DTYPE)
    full = z["stable_perm"] if "stable_perm" in z else np.arange(len(parts), dtype=np.uint32)
    assert np.array_equal(renderer.order(len(parts)), full[want["active"][full].astype(bool)])
    assert renderer.fragments() == int(z["fragments"])
    assert rel_linf(pic, z["render_fp64"]) <= IMAGE_TOL


@pytest.mark.parametrize("name", CASES)
def test_host_rendering_writeback_matches_golden(name, renderer):
    """host_rendering's in-place side effects: the particle array comes back
    projected, colourised and (absorption) stably z-sorted."""
    z, prm, rc = load(name)
    parts = z["particles_in"].view(PARTICLE_DTYPE).copy()
    rcx = sg.RenderContext(campos=rc.campos, centerpos=rc.centerpos, lookat=rc.lookat,
                           sky=rc.sky, amap=rc.amap, b_brightness=rc.b_brightness)
    sg.host_rendering(sg.ParamFile(dict(prm)), parts, rcx, renderer=renderer)
    want = z["projected"].view(PARTICLE_DTYPE)
    if "stable_perm" in z:
        want = want[z["stable_perm"]]
    assert np.array_equal(parts.view(np.uint8), want.view(np.uint8))
    assert rel_linf(rcx.pic, z["render_fp64"]) <= IMAGE_TOL
