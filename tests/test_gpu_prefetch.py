"""spl_prefetch: host particle arrays copied ahead of the spl_render that reads
them.  Every render from a prefetched copy must equal the same render copying
its inputs itself, bit for bit; prefetches are consumed in order, a render of
other arrays drops them, and at most two may be pending."""
import ctypes

import numpy as np
import pytest

import splotch_gb300 as sg
from splotch_gb300 import _abi, synth

pytestmark = pytest.mark.gpu


def _frame(seed: int):
    w = synth.plain_absorption(n_gas=160_000, n_star=40_000, xres=320, yres=180, tile=16,
                               seed=seed)
    keep: list = []
    desc = sg.frame_desc(w.params, w.rc, keep)
    return w.particles.copy(), desc, keep


def _plain(renderer, desc, parts):
    pic = np.zeros((desc.xres, desc.yres, 3), np.float32)
    renderer.render_aos(desc, parts, pic)
    return pic


def test_prefetched_render_equals_plain(renderer):
    a, desc, _keep = _frame(11)
    want = _plain(renderer, desc, a)
    for _ in range(2):  # the copy-ahead slots are reused
        renderer.prefetch_aos(a)
        got = np.zeros_like(want)
        renderer.render_aos(desc, a, got)
        assert np.array_equal(got, want)


def test_two_pending_in_order_and_third_refused(renderer):
    a, desc_a, _ka = _frame(12)
    b, desc_b, _kb = _frame(13)
    want_a, want_b = _plain(renderer, desc_a, a), _plain(renderer, desc_b, b)
    renderer.prefetch_aos(a)
    renderer.prefetch_aos(b)
    with pytest.raises(_abi.SplotchError):
        renderer.prefetch_aos(a)  # two already pending
    got = np.zeros_like(want_a)
    renderer.render_aos(desc_a, a, got)
    assert np.array_equal(got, want_a)
    got = np.zeros_like(want_b)
    renderer.render_aos(desc_b, b, got)
    assert np.array_equal(got, want_b)


def test_render_of_other_arrays_drops_the_queue(renderer):
    a, desc_a, _ka = _frame(14)
    b, desc_b, _kb = _frame(15)
    want_a, want_b = _plain(renderer, desc_a, a), _plain(renderer, desc_b, b)
    renderer.prefetch_aos(a)
    got = np.zeros_like(want_b)
    renderer.render_aos(desc_b, b, got)  # not the prefetched arrays
    assert np.array_equal(got, want_b)
    got = np.zeros_like(want_a)
    renderer.render_aos(desc_a, a, got)  # the queue was dropped: a plain copy
    assert np.array_equal(got, want_a)


def test_device_view_is_a_no_op(renderer):
    torch = pytest.importorskip("torch")
    a, desc, _keep = _frame(16)
    dev = torch.from_numpy(a.view(np.uint8).copy()).cuda()
    p = _abi.Particles(n=len(a), layout=_abi.SPL_LAYOUT_AOS, memspace=_abi.SPL_MEM_DEVICE,
                       aos=_abi.ptr(dev))
    _abi.check(renderer.lib.spl_prefetch(renderer.ctx, ctypes.byref(p)))
