"""Failure detection on the GPU, without faulting, trapping or hanging it.

The reference stops on errors through planck_fail -> PlanckError
(cxxsupport/error_handling.h:69-80) and aborts on a device allocation error
(cuda/cuda_splotch.cc:105).  Here every C-ABI call returns a status instead,
and a failed call leaves its context usable.  Two failures are made on
purpose, both in bounded, in-range ways:

* a look-back wait that runs out: the depth sort's first scatter pass is
  launched without its first tile, so the next tile finds that status
  unpublished and gives up after a short spin limit (every write of the pass
  stays in bounds); spl_render must return SPL_ERR_TIMEOUT before anything
  uses the invalid permutation, and the next frame must be exact;
* a bin entry past its particle's counted tiles (a count stored one short by
  a test hook): the emission stores nothing outside the particle's slots and
  spl_render must return SPL_ERR_CAPACITY, the next frame exact;
* a device allocation that fails: spl_debug_fail_alloc makes the n-th buffer
  allocation fail without calling cudaMalloc; the call must return
  SPL_ERR_ALLOC, and the next call must allocate what is missing and render
  exactly (plain frames) or build the batch (batched rendering).
"""
import numpy as np
import pytest

import splotch_gb300 as sg
from splotch_gb300 import _abi, synth

from .helpers import assert_parity, gpu_frame, oracle_frame

pytestmark = pytest.mark.gpu


def _absorption():
    return synth.plain_absorption(n_gas=400_000, n_star=100_000, xres=320, yres=180, tile=16,
                                  order="ftb")


def test_lookback_timeout_is_reported_and_the_context_recovers(renderer, port):
    w = _absorption()
    prm = dict(w.params.params)
    o = oracle_frame(port, prm, w.rc, w.particles, fp32=False)
    # two or more scatter tiles of 4096 keys: a tile that waits on the first
    assert o.projected["active"].sum() > 2 * 4096
    renderer.set_debug(_abi.SPL_DEBUG_LOOKBACK_STALL)
    try:
        with pytest.raises(_abi.SplotchError) as e:
            gpu_frame(renderer, prm, w.rc, w.particles)
    finally:
        renderer.set_debug(0)
    assert e.value.code == _abi.SPL_ERR_TIMEOUT, e.value
    assert "look-back" in str(e.value)
    # the same context renders the frame exactly afterwards
    g = gpu_frame(renderer, prm, w.rc, w.particles)
    assert_parity(g, o)


def test_tile_count_mismatch_is_reported_and_the_context_recovers(renderer, port):
    """Bin emission checks every entry against its particle's counted tiles: with
    the first active particle's count stored one short (a test hook), the extra
    passing tile is not stored and spl_render returns SPL_ERR_CAPACITY."""
    from .test_gpu_parity import _edge_setup, _particles
    prm, rc = _edge_setup(a_eq_e=False, gpu_order="ftb")
    # particle 0 sits on a tile corner: four tiles; then a few others
    specs = [(16.0, 16.0, 6.0, 0.0, 1.0, 0.5)] + [
        (10.0 + 9.0 * k, 40.0 + 3.0 * (k % 4), 4.0 + k % 3, 0.1 * k, 1.0, 0.1 * k)
        for k in range(8)]
    p = _particles(prm, specs)
    o = oracle_frame(port, prm, rc, p, fp32=False)
    assert 2 <= np.count_nonzero(o.entries == 0) <= 64  # the first active particle
    renderer.set_debug(_abi.SPL_DEBUG_SHORT_COUNT)
    try:
        with pytest.raises(_abi.SplotchError) as e:
            gpu_frame(renderer, prm, rc, p)
    finally:
        renderer.set_debug(0)
    assert e.value.code == _abi.SPL_ERR_CAPACITY, e.value
    assert "more tiles than" in str(e.value)
    assert_parity(gpu_frame(renderer, prm, rc, p), o)


@pytest.mark.parametrize("nth", [1, 3, 8, 17])
def test_allocation_failure_is_reported_and_the_context_recovers(nth, port):
    lib = _abi.load()
    w = _absorption()
    prm = dict(w.params.params)
    r = sg.Renderer(0)  # a fresh context allocates every buffer on its first frame
    try:
        _abi.check(lib.spl_debug_fail_alloc(nth))
        with pytest.raises(_abi.SplotchError) as e:
            gpu_frame(r, prm, w.rc, w.particles)
        assert e.value.code == _abi.SPL_ERR_ALLOC, e.value
        assert "injected" in str(e.value)
        g = gpu_frame(r, prm, w.rc, w.particles)
        assert_parity(g, oracle_frame(port, prm, w.rc, w.particles, fp32=False))
    finally:
        lib.spl_debug_fail_alloc(0)
        r.close()


def test_batch_allocation_failure_is_reported(renderer):
    torch = pytest.importorskip("torch")
    lib = _abi.load()
    bw = synth.batched(n_sets=2, poses=2, scale=0.003,
                       resolutions=((96, 96), (160, 120)))
    sets = [{k: torch.from_numpy(v).cuda() for k, v in synth.soa_from_aos(p).items()}
            for p in bw.sets]
    keep: list = []
    frames = []
    for s, params, rc in bw.frames:
        desc = sg.frame_desc(params, rc, keep)
        frames.append((s, desc, torch.zeros((desc.xres, desc.yres, 3), dtype=torch.float32,
                                            device="cuda")))
    torch.cuda.synchronize()
    opt = {"tile_size": 16, "splat_config_additive": 0, "splat_config_absorption": 2}
    try:
        _abi.check(lib.spl_debug_fail_alloc(2))
        with pytest.raises(_abi.SplotchError) as e:
            sg.Batch(renderer, sets, frames, **opt)
        assert e.value.code == _abi.SPL_ERR_ALLOC, e.value
    finally:
        lib.spl_debug_fail_alloc(0)
    b = sg.Batch(renderer, sets, frames, **opt)
    try:
        b.render()
        torch.cuda.synchronize()
        for s, desc, pic in frames:
            want = torch.zeros_like(pic)
            d = type(desc).from_buffer_copy(desc)
            d.tile_size, d.splat_config = 16, 0 if desc.a_eq_e else 2
            renderer.set_split_tiles(False)  # the batch renders every tile whole
            try:
                renderer.render_soa(d, sets[s], want, device=True)
            finally:
                renderer.set_split_tiles(_abi.SPL_SPLIT_ADDITIVE)
            torch.cuda.synchronize()
            assert np.array_equal(pic.cpu().numpy(), want.cpu().numpy())
    finally:
        b.close()
