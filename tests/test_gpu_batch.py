"""Batched rendering (spl_batch_*) on the GPU.

Every frame of a batch must equal, bit for bit, the image spl_render gives for
that frame at the batch's tile size and launch configuration (the batch only
regroups the same per-frame work), and so stays within 1e-4 of the FP64
oracle.  Covered: mixed additive / ordered frames, uneven set sizes and
resolutions, the autotuner's choice, the captured graph, re-planning when the
measured capacities are exceeded, repeated renders.
"""
import numpy as np
import pytest

import splotch_gb300 as sg
from oracle.oracle import rel_linf
from splotch_gb300 import _abi, synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SMALL_RES = ((96, 96), (160, 120), (200, 64), (128, 128))


def _device_sets(bw):
    return [{k: torch.from_numpy(v).cuda() for k, v in synth.soa_from_aos(p).items()}
            for p in bw.sets]


def _batch(renderer, bw, sets, **opt):
    keep: list = []
    frames = []
    for s, params, rc in bw.frames:
        desc = sg.frame_desc(params, rc, keep)
        pic = torch.full((desc.xres, desc.yres, 3), float("nan"), dtype=torch.float32,
                         device="cuda")
        frames.append((s, desc, pic))
    torch.cuda.synchronize()  # the batch runs on its own stream
    b = sg.Batch(renderer, sets, frames, **opt)
    return b, frames, keep


def _plain(renderer, sets, s, desc, T, cfg):
    d = type(desc).from_buffer_copy(desc)
    d.tile_size = T
    d.splat_config = cfg
    pic = torch.zeros((d.xres, d.yres, 3), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    # the batch renders every tile whole: so does its per-frame counterpart
    renderer.set_split_tiles(False)
    try:
        renderer.render_soa(d, sets[s], pic, device=True)
    finally:
        renderer.set_split_tiles(_abi.SPL_SPLIT_ADDITIVE)
    torch.cuda.synchronize()
    return pic.cpu().numpy()


def _check_equal_plain(renderer, sets, frames, info):
    for s, desc, pic in frames:
        cfg = info["splat_config_additive"] if desc.a_eq_e else info["splat_config_absorption"]
        want = _plain(renderer, sets, s, desc, info["tile_size"], cfg)
        got = pic.cpu().numpy()
        assert np.array_equal(got, want), (s, desc.xres, desc.yres, desc.a_eq_e)


def test_batch_equals_plain_frames_fixed_tile(renderer):
    bw = synth.batched(n_sets=4, poses=3, scale=0.004, resolutions=SMALL_RES)
    sets = _device_sets(bw)
    b, frames, _ = _batch(renderer, bw, sets, tile_size=16, splat_config_additive=0,
                          splat_config_absorption=2)
    try:
        b.render()
        torch.cuda.synchronize()
        info = b.info()
        assert info["graph"] == 1 and info["tile_size"] == 16
        assert info["n_active"] > 0 and info["n_entries"] > 0
        _check_equal_plain(renderer, sets, frames, info)
        first = [p.cpu().numpy().copy() for _, _, p in frames]
        b.render()
        for (_, _, p), f in zip(frames, first):
            assert np.array_equal(p.cpu().numpy(), f)
    finally:
        b.close()


def test_batch_mixed_orders_and_palettes(renderer):
    """Ordered frames compositing front-to-back and back-to-front in one batch
    (the splat queue chooses the form per item), and a set whose frames do not
    all share a palette (no per-set palette cache for it)."""
    bw = synth.batched(n_sets=4, poses=3, scale=0.004, resolutions=SMALL_RES)
    for i, (s, params, rc) in enumerate(bw.frames):
        if not params.params["a_eq_e"] and i % 2:
            params.params["gpu_order"] = "btf"
        if s == 0 and i % 3 == 1:  # another palette for one frame of set 0
            rc.amap = [synth.five_stop_palette(), None]
    sets = _device_sets(bw)
    b, frames, _ = _batch(renderer, bw, sets, tile_size=16, splat_config_additive=2,
                          splat_config_absorption=2)
    try:
        b.render()
        torch.cuda.synchronize()
        _check_equal_plain(renderer, sets, frames, b.info())
    finally:
        b.close()


def test_batch_autotuned_matches_plain_and_oracle(renderer, port):
    bw = synth.batched(n_sets=2, poses=2, scale=0.003, resolutions=SMALL_RES)
    sets = _device_sets(bw)
    b, frames, _ = _batch(renderer, bw, sets)
    try:
        b.render()
        info = b.info()
        assert info["tile_size"] in (8, 16, 32) and info["tune_ms"] > 0
        _check_equal_plain(renderer, sets, frames, info)
        # one frame of each mode against the FP64 oracle at the chosen tile size
        for want_add in (True, False):
            k = next(i for i, (_, d, _) in enumerate(frames) if bool(d.a_eq_e) == want_add)
            s, params, rc = bw.frames[k]
            prm = dict(params.params)
            prm["tile_size_cpu"] = str(info["tile_size"])
            p = bw.sets[s].copy()
            port.project_colorize(prm, rc, p)
            order = None if want_add else port.sort_perm(p, 1)
            xres, yres = int(prm["xres"]), int(prm["yres"])
            pic64, _ = port.render_fp64(p, order, xres, yres, info["tile_size"], want_add, 0.2)
            assert rel_linf(frames[k][2].cpu().numpy(), pic64) <= 1e-4
    finally:
        b.close()


def test_batch_replans_when_capacity_is_exceeded(renderer):
    bw = synth.batched(n_sets=2, poses=2, scale=0.003, resolutions=SMALL_RES)
    sets = _device_sets(bw)
    b, frames, _ = _batch(renderer, bw, sets, tile_size=16, splat_config_additive=0,
                          splat_config_absorption=2, capacity_margin=0.5)
    try:
        b.render()
        info = b.info()
        assert info["replans"] >= 1
        assert info["cap_active"] >= info["n_active"]
        assert info["cap_entries"] >= info["n_entries"]
        _check_equal_plain(renderer, sets, frames, info)
    finally:
        b.close()


def test_batch_eager_equals_graph(renderer):
    bw = synth.batched(n_sets=2, poses=2, scale=0.003, resolutions=SMALL_RES)
    sets = _device_sets(bw)
    ga, fa, _ = _batch(renderer, bw, sets, tile_size=16, splat_config_additive=0,
                       splat_config_absorption=2)
    ea, fe, _ = _batch(renderer, bw, sets, tile_size=16, splat_config_additive=0,
                       splat_config_absorption=2, use_graph=False)
    try:
        ga.render()
        ea.render()
        assert ga.info()["graph"] == 1 and ea.info()["graph"] == 0
        for (_, _, p), (_, _, q) in zip(fa, fe):
            assert np.array_equal(p.cpu().numpy(), q.cpu().numpy())
    finally:
        ga.close()
        ea.close()


def test_autotuner_cache(renderer):
    """A second batch of the same shape (per frame: resolution, mode class and
    the size bucket of its set) takes the tuned choice from the cache and times
    nothing; another shape is tuned afresh; tune_cache=0 always searches."""
    bw = synth.batched(n_sets=2, poses=2, scale=0.003, resolutions=((88, 72), (120, 96)))
    sets = _device_sets(bw)
    made = []
    try:
        b0, f0, _ = _batch(renderer, bw, sets, tune_cache=False)
        made.append(b0)
        i0 = b0.info()
        assert i0["tune_cached"] == 0 and i0["tune_ms"] > 0
        b1, _, _ = _batch(renderer, bw, sets)  # searches (or hits) and fills the cache
        made.append(b1)
        b2, f2, _ = _batch(renderer, bw, sets)
        made.append(b2)
        i1, i2 = b1.info(), b2.info()
        assert i2["tune_cached"] == 1 and i2["tune_ms"] == 0.0 and i2["plan_ms"] > 0
        for k in ("tile_size", "splat_config_additive", "splat_config_absorption"):
            assert i2[k] == i1[k], k
        b2.render()
        torch.cuda.synchronize()
        _check_equal_plain(renderer, sets, f2, b2.info())
        # another shape: one frame at another resolution
        s, params, rc = bw.frames[0]
        params.params["xres"] = "104"
        b3, _, _ = _batch(renderer, bw, sets)
        made.append(b3)
        assert b3.info()["tune_cached"] == 0
    finally:
        for b in made:
            b.close()
