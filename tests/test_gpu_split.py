"""spl_context_set_split_tiles: heavy tiles cut into list segments, one GPU
block per segment, results folded per pixel in list order.

The halo-centred frames here have tiles whose lists are many times the mean,
so the split path is taken (more kernel launches).  A split render regroups
each pixel's float sums, so it is compared with the unsplit render within
1e-5 (per-pixel relative L-infinity with the oracle's floor), and with the
FP64 oracle within the usual 1e-4.
"""
import numpy as np
import pytest

import splotch_gb300 as sg
from oracle.oracle import rel_linf
from splotch_gb300 import _abi, synth

from .helpers import oracle_frame

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["additive", "absorption"])
def test_split_tiles_match_unsplit_and_oracle(renderer, port, mode):
    w = synth.differentiable(n=300_000, mode=mode, xres=384, tile=16, order="ftb")
    keep: list = []
    desc = sg.frame_desc(w.params, w.rc, keep)
    shape = (desc.xres, desc.yres, 3)
    plain = np.zeros(shape, np.float32)
    renderer.set_split_tiles(False)
    renderer.render_aos(desc, w.particles.copy(), plain)
    launches_plain = renderer.stats()["kernel_launches"]
    split = np.zeros(shape, np.float32)
    renderer.set_split_tiles(True)
    try:
        renderer.render_aos(desc, w.particles.copy(), split)
        launches_split = renderer.stats()["kernel_launches"]
    finally:
        renderer.set_split_tiles(_abi.SPL_SPLIT_ADDITIVE)
    assert launches_split > launches_plain
    assert rel_linf(split, plain) <= 1e-5
    o = oracle_frame(port, dict(w.params.params), w.rc, w.particles, fp32=False)
    assert rel_linf(split, o.pic64) <= 1e-4


def test_split_tiles_leave_differentiable_ordered_frames_whole(renderer):
    w = synth.differentiable(n=200_000, mode="absorption", xres=256, tile=16, order="ftb")
    keep: list = []
    desc = sg.frame_desc(w.params, w.rc, keep)
    pic = np.zeros((desc.xres, desc.yres, 3), np.float32)
    renderer.set_differentiable(True)
    renderer.render_aos(desc, w.particles.copy(), pic)
    want = pic.copy()
    renderer.set_split_tiles(True)
    try:
        renderer.render_aos(desc, w.particles.copy(), pic)
    finally:
        renderer.set_split_tiles(_abi.SPL_SPLIT_ADDITIVE)
        renderer.set_differentiable(False)
    assert np.array_equal(pic, want)  # the same unsplit render


@pytest.mark.parametrize("mode", ["additive", "absorption"])
def test_split_tiles_on_sparse_frames(renderer, port, mode):
    """A frame with many empty tiles, split in both modes: every empty tile
    still writes its zeros, and the image is the oracle's."""
    from .helpers import assert_parity, gpu_frame

    w = synth.differentiable(n=300, mode=mode, xres=320, yres=200, tile=16, order="ftb")
    prm = dict(w.params.params)
    renderer.set_split_tiles(True)
    try:
        g = gpu_frame(renderer, prm, w.rc, w.particles)
    finally:
        renderer.set_split_tiles(_abi.SPL_SPLIT_ADDITIVE)
    ntiles = (320 // 16) * (200 // 16 + 1)
    assert (np.diff(g.tile_start) == 0).sum() > ntiles // 4, "expected many empty tiles"
    assert_parity(g, oracle_frame(port, prm, w.rc, w.particles, fp32=False))
