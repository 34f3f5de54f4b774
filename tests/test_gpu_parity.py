"""Parity of the CUDA path with the oracle, stage by stage.

Bit-exact: projected particles (x, y, z, r, I, e, active), the visiting order
(stable sort permutation), tile ranges and tile bin entries.  Images: per-pixel
relative L-inf <= 1e-4 against the FP64 oracle (floor 1e-6 * max|pixel|).
"""
import numpy as np
import pytest

import splotch_gb300 as sg
from oracle.oracle import rel_linf
from splotch_gb300 import synth

from .helpers import IMAGE_TOL, assert_parity, gpu_frame, oracle_frame

pytestmark = pytest.mark.gpu


def _additive(**kw):
    return synth.plain_additive(**kw)


def _absorption(**kw):
    return synth.plain_absorption(**kw)


CASES = {
    "add_T16": lambda: _additive(n=40000, xres=160, yres=120, tile=16),
    "add_T50": lambda: _additive(n=40000, xres=200, yres=150, tile=50),
    "add_T7_odd": lambda: _additive(n=20000, xres=101, yres=77, tile=7),
    "add_T32": lambda: _additive(n=40000, xres=256, yres=200, tile=32),
    "add_T64": lambda: _additive(n=20000, xres=200, yres=130, tile=64),
    "abs_btf_T16": lambda: _absorption(n_gas=40000, n_star=10000, xres=192, yres=108, tile=16,
                                       order="btf"),
    "abs_ftb_T16": lambda: _absorption(n_gas=40000, n_star=10000, xres=192, yres=108, tile=16,
                                       order="ftb"),
    "abs_btf_T50": lambda: _absorption(n_gas=40000, n_star=10000, xres=192, yres=108, tile=50,
                                       order="btf"),
    "abs_ftb_T32": lambda: _absorption(n_gas=40000, n_star=10000, xres=256, yres=144, tile=32,
                                       order="ftb"),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_stage_parity(name, renderer, port):
    w = CASES[name]()
    prm = dict(w.params.params)
    g = gpu_frame(renderer, prm, w.rc, w.particles)
    o = oracle_frame(port, prm, w.rc, w.particles)
    info = assert_parity(g, o)
    assert o.frags > 0
    print(name, info)


@pytest.mark.parametrize("mode", ["add", "btf", "ftb"])
@pytest.mark.parametrize("tile", [8, 12, 16, 32, 50])
def test_every_splat_config(tile, mode, renderer, port):
    """Every launch configuration that covers the tile size gives a parity image."""
    from splotch_gb300 import _abi

    lib = _abi.load()
    if mode == "add":
        w = _additive(n=20000, xres=120, yres=88, tile=tile)
    else:
        w = _absorption(n_gas=16000, n_star=4000, xres=128, yres=72, tile=tile, order=mode)
    prm = dict(w.params.params)
    o = oracle_frame(port, prm, w.rc, w.particles, fp32=False)
    ran = 0
    for cfg in range(lib.spl_splat_config_count()):
        if not lib.spl_splat_config_valid(cfg, tile):
            continue
        prm["gpu_splat_config"] = str(cfg)
        assert_parity(gpu_frame(renderer, prm, w.rc, w.particles), o)
        ran += 1
    assert ran >= 1


def _edge_setup(xres=96, yres=80, tile=16, a_eq_e=True, **extra):
    rc = sg.RenderContext(campos=np.array([0.0, 0.0, 100.0]),
                          centerpos=np.array([0.0, 0.0, 100.0]), lookat=np.zeros(3),
                          sky=np.array([0.0, 1.0, 0.0]), amap=[synth.blue_white_palette()])
    prm = {"xres": xres, "yres": yres, "fov": 45.0, "a_eq_e": a_eq_e, "tile_size_cpu": tile,
           "ptypes": 1, "sort_type": 1}
    prm.update(extra)
    return sg.ParamFile(prm).params, rc


def _place(prm, px, py, rpix, zw=0.0):
    """World position / hsml that lands near pixel (px, py) with radius rpix
    for the edge-case camera (campos (0,0,100) looking at the origin)."""
    xres, yres = int(prm["xres"]), int(prm["yres"])
    res2 = 0.5 * xres
    fovfct = np.tan(np.radians(45.0) / 2)
    xfac2 = res2 / (fovfct * (100.0 - zw))
    ycorr = 0.5 * (yres - xres)
    return (px - res2) / xfac2, (py - res2 - ycorr) / xfac2, rpix / (2 * xfac2)


def _particles(prm, specs):
    p = sg.make_particles(len(specs))
    for i, (px, py, rpix, zw, I, c) in enumerate(specs):
        x, y, h = _place(prm, px, py, rpix, zw)
        p[i]["x"], p[i]["y"], p[i]["z"], p[i]["r"] = x, y, zw, h
        p[i]["I"], p[i]["er"] = I, c
    return p


EDGE = {
    "single_centre": [(40.0, 40.0, 6.0, 0.0, 1.0, 0.5)],
    "tile_edge_straddle": [(16.0 + d, 16.0 + d, 5.0, 0.0, 1.0, 0.3) for d in (-0.5, 0.0, 0.49)]
    + [(31.5, 47.99, 3.0, 0.0, 2.0, 0.7)],
    "clipped_borders": [(-3.0, 10.0, 8.0, 0.0, 1.0, 0.2), (95.5, 79.7, 6.0, 0.0, 1.0, 0.9),
                        (50.0, -7.5, 9.0, 0.0, 1.0, 0.4), (120.0, 40.0, 10.0, 0.0, 1.0, 0.5)],
    "minrad_floor": [(20.3 + 3 * i, 30.7 + 2 * i, 0.05 * (i + 1), 0.0, 1.0, 0.5) for i in range(12)],
    "huge_wide_path": [(48.0, 40.0, 400.0, 0.0, 0.3, 0.6), (10.0, 70.0, 150.0, 1.0, 0.2, 0.1)],
    "equal_z_ties": [(30.0 + i, 35.0 + (i % 3), 7.0, 5.0, 1.0 + 0.1 * i, i / 20) for i in range(20)],
    "behind_camera": [(40.0, 40.0, 5.0, 150.0, 1.0, 0.5), (41.0, 40.0, 5.0, 99.999, 1.0, 0.5)],
}


@pytest.mark.parametrize("mode", ["add", "btf", "ftb"])
@pytest.mark.parametrize("name", sorted(EDGE))
def test_edge_cases(name, mode, renderer, port):
    prm, rc = _edge_setup(a_eq_e=(mode == "add"), gpu_order=mode if mode != "add" else "btf")
    p = _particles(prm, EDGE[name])
    g = gpu_frame(renderer, prm, rc, p)
    o = oracle_frame(port, prm, rc, p)
    assert_parity(g, o)


@pytest.mark.parametrize("tile", [8, 16, 32])
@pytest.mark.parametrize("mode", ["add", "ftb"])
def test_bins_across_footprint_sizes(tile, mode, renderer, port):
    """Bin emission deals each warp's candidate tiles across its lanes and hands
    particles of more than 64 tiles to the warp-per-particle path: footprints
    from one tile to well past 64 (both paths in every warp), partial tiles at
    the right and bottom edges, three tile sizes; bins bit-exact."""
    rng = np.random.default_rng(11 + tile)
    xres, yres = (203, 137) if tile < 32 else (403, 297)  # more than 64 tiles either way
    prm, rc = _edge_setup(xres=xres, yres=yres, tile=tile, a_eq_e=(mode == "add"),
                          gpu_order="ftb")
    # radius in pixels reaching ~1 to ~100 tiles at this tile size
    rmax = 7.0 * tile
    n = 600
    specs = [(float(rng.uniform(-10, xres + 10)), float(rng.uniform(-10, yres + 10)),
              float(rmax * rng.random() ** 2 + 0.3), float(rng.uniform(-20, 20)),
              float(rng.uniform(0.2, 1.5)), float(rng.random())) for _ in range(n)]
    p = _particles(prm, specs)
    g = gpu_frame(renderer, prm, rc, p)
    o = oracle_frame(port, prm, rc, p, fp32=False)
    assert_parity(g, o)
    counts = np.diff(o.tile_start.astype(np.int64))
    assert g.stats["n_wide"] > 0, "no particle took the many-tile path"
    assert len(o.entries) > n, counts.max()


@pytest.mark.parametrize("mode", ["add", "ftb"])
def test_footprints_at_the_image_edges(mode, renderer, port):
    """Footprint edges within +-0.02 pixel of each image border (where the
    activity pass's float screen cannot decide and the exact arithmetic does),
    and radii from below the minrad floor to several pixels: projection, order
    and bins bit-exact."""
    rng = np.random.default_rng(5)
    prm, rc = _edge_setup(xres=97, yres=61, a_eq_e=(mode == "add"), gpu_order="ftb")
    xres, yres = 97, 61
    specs = []
    for k in range(800):
        rpix = float(rng.choice([0.3, 1.0, 1.7, 4.0, 9.0]) * rng.uniform(0.9, 1.1))
        ext = 0.75 * float(np.sqrt(rpix * rpix + 1.0))  # radius after the minrad_pix=1 correction
        d = float(rng.uniform(-0.02, 0.02))
        side = k % 4
        if side == 0:    # x - 0.75r + 1 = xres + d
            px, py = xres + d - 1 + ext, float(rng.uniform(0, yres))
        elif side == 1:  # x + 0.75r + 1 = 1 + d
            px, py = d - ext, float(rng.uniform(0, yres))
        elif side == 2:
            px, py = float(rng.uniform(0, xres)), yres + d - 1 + ext
        else:
            px, py = float(rng.uniform(0, xres)), d - ext
        specs.append((px, py, rpix, float(rng.uniform(-5, 5)), 1.0, float(rng.random())))
    p = _particles(prm, specs)
    g = gpu_frame(renderer, prm, rc, p)
    o = oracle_frame(port, prm, rc, p, fp32=False)
    assert_parity(g, o)
    act = g.projected["active"].astype(bool)
    assert 0 < act.sum() < len(p)


def test_zmin_and_all_culled(renderer, port):
    # both particles sit at depth -z = 100 and 99.5 in camera space: zmin=100.5
    # culls them (splotch_host.cc:123, cull when -z <= zmin)
    prm, rc = _edge_setup(zmin=100.5)
    p = _particles(prm, [(40.0, 40.0, 5.0, 0.0, 1.0, 0.5), (60.0, 20.0, 5.0, 0.5, 1.0, 0.5)])
    g = gpu_frame(renderer, prm, rc, p)
    o = oracle_frame(port, prm, rc, p)
    assert_parity(g, o)
    assert not g.projected["active"].any()
    assert not g.pic.any()


def test_empty_input(renderer, port):
    prm, rc = _edge_setup(a_eq_e=False)
    p = sg.make_particles(0)
    g = gpu_frame(renderer, prm, rc, p)
    assert g.entries.size == 0 and not g.pic.any()


def test_host_rendering_mirror(built, port):
    """The drop-in: same keys/defaults, rc.pic overwritten, particles mutated in
    place (projected, colourised, stable z order) like the reference."""
    w = synth.plain_absorption(n_gas=8000, n_star=2000, xres=128, yres=96, tile=16, order="btf")
    parts = w.particles.copy()
    rc = w.rc
    sg.update_res(w.params, rc)
    sg.host_rendering(w.params, parts, rc)
    prm = dict(w.params.params)
    ref = w.particles.copy()
    port.project_colorize(prm, rc, ref)
    perm = port.sort_perm(ref, 1)
    ref = ref[perm]
    assert np.array_equal(parts.view(np.uint8), ref.view(np.uint8))
    pic64, _ = port.render_fp64(ref, None, 128, 96, 16, False, 0.2)
    assert rel_linf(rc.pic, pic64) <= IMAGE_TOL


def test_large_writeback_into_pageable_memory(renderer):
    """A write-back of 108 MB (3M particles, not a round size) into pageable
    host memory: its bytes equal the same write-back into device memory, the
    images are equal, and the array did change."""
    torch = pytest.importorskip("torch")
    w = synth.plain_absorption(n_gas=2_400_001, n_star=600_000, xres=320, yres=200, tile=16)
    keep: list = []
    desc = sg.frame_desc(w.params, w.rc, keep)
    host = w.particles.copy()
    pic = np.zeros((320, 200, 3), np.float32)
    renderer.render_aos(desc, host, pic, writeback=True)
    dev = torch.from_numpy(w.particles.copy().view(np.uint8).reshape(-1)).cuda()
    pic_d = torch.zeros((320, 200, 3), dtype=torch.float32, device="cuda")
    renderer.render_aos(desc, dev, pic_d, device=True, writeback=True)
    assert np.array_equal(host.view(np.uint8).reshape(-1), dev.cpu().numpy())
    assert np.array_equal(pic, pic_d.cpu().numpy())
    assert not np.array_equal(host.view(np.uint8), w.particles.view(np.uint8))


def test_soa_device_matches_aos(renderer):
    torch = pytest.importorskip("torch")
    w = synth.plain_additive(n=30000, xres=128, yres=128, tile=16)
    keep: list = []
    desc = sg.frame_desc(w.params, w.rc, keep)
    pic_h = np.zeros((128, 128, 3), np.float32)
    renderer.render_aos(desc, w.particles.copy(), pic_h)
    soa = {k: torch.from_numpy(v).cuda() for k, v in synth.soa_from_aos(w.particles).items()}
    pic_d = torch.zeros((128, 128, 3), dtype=torch.float32, device="cuda")
    renderer.render_soa(desc, soa, pic_d, device=True)
    torch.cuda.synchronize()
    assert np.array_equal(pic_d.cpu().numpy(), pic_h)


def test_determinism(renderer):
    w = synth.plain_absorption(n_gas=40000, n_star=10000, xres=192, yres=108, tile=16)
    keep: list = []
    desc = sg.frame_desc(w.params, w.rc, keep)
    a = np.zeros((192, 108, 3), np.float32)
    b = np.zeros_like(a)
    renderer.render_aos(desc, w.particles.copy(), a)
    renderer.render_aos(desc, w.particles.copy(), b)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("camera", ["outside", "inside_cluster"])
def test_fast_projection_equals_fp64(camera, renderer):
    """The float-float projection (with per-particle FP64 fallback) is bit-identical
    to the exact FP64 arithmetic over millions of particles, and the activity
    pass's float screen (off under the FP64 hook) selects the same particles:
    visiting order and tile bins are equal."""
    w = synth.plain_absorption(n_gas=1_600_000, n_star=400_000, xres=640, yres=360, tile=16)
    if camera == "inside_cluster":  # many particles near the camera axis and plane
        p = w.particles
        c = np.array([p["x"][0], p["y"][0], p["z"][0]], dtype=np.float64)
        w.rc.campos = c + np.array([0.3, -0.2, -2.0])
        w.rc.centerpos = w.rc.campos.copy()
        w.rc.lookat = c + np.array([1.0, 0.5, 40.0])
    keep: list = []
    desc = sg.frame_desc(w.params, w.rc, keep)
    pic = np.zeros((640, 360, 3), np.float32)
    out = {}
    ntiles = ((640 + 15) // 16) * ((360 + 15) // 16)
    for flags in (0, 1):
        renderer.set_debug(flags)
        try:
            renderer.render_aos(desc, w.particles.copy(), pic)
        finally:
            renderer.set_debug(0)
        out[flags] = (renderer.projected(len(w.particles)), renderer.stats()["n_fallback"],
                      renderer.order(len(w.particles)), renderer.bins(ntiles))
    a, b = out[0][0].view(np.uint8), out[1][0].view(np.uint8)
    assert np.array_equal(a, b)
    assert np.array_equal(out[0][2], out[1][2])
    for u, v in zip(out[0][3], out[1][3]):
        assert np.array_equal(u, v)
    assert out[1][1] == 0
    assert out[0][1] < 0.01 * len(w.particles), f"{out[0][1]} FP64 fallbacks"
    print(camera, "fallbacks", out[0][1], "of", len(w.particles))


def test_onesweep_equals_reduce_then_scan(renderer):
    """The onesweep radix sorts (decoupled look-back) and the reduce-then-scan
    sorts give the same permutation and bins on a few million keys."""
    w = synth.plain_absorption(n_gas=3_200_000, n_star=800_000, xres=960, yres=540, tile=16)
    keep: list = []
    desc = sg.frame_desc(w.params, w.rc, keep)
    pic = np.zeros((960, 540, 3), np.float32)
    ntiles = 60 * 34
    got = {}
    for flags in (0, 2):
        renderer.set_debug(flags)
        try:
            renderer.render_aos(desc, w.particles.copy(), pic)
        finally:
            renderer.set_debug(0)
        got[flags] = (renderer.order(len(w.particles)), *renderer.bins(ntiles), pic.copy())
    for a, b in zip(got[0], got[2]):
        assert np.array_equal(a, b)


def test_full_size_additive_1M(renderer, port):
    """The plain additive workload at full size (1M particles, 800x800)."""
    w = synth.plain_additive()
    prm = dict(w.params.params)
    g = gpu_frame(renderer, prm, w.rc, w.particles)
    o = oracle_frame(port, prm, w.rc, w.particles, fp32=False)
    info = assert_parity(g, o)
    print("full additive", info, g.stats)


@pytest.mark.parametrize("order", ["btf", "ftb"])
@pytest.mark.parametrize("sort_type", [0, 2, 3, 4])
def test_sort_types(sort_type, order, renderer, port):
    """Every sort_type of particle_sort (splotch/splotch_host.cc:289-321,
    comparators splotch/splotchutils.h:74-96) on an ordered frame: 0 keeps
    particle order, 2/3 sort by the colourised red channel descending /
    ascending, 4 by pixel radius descending; the stable permutation must equal
    the oracle's bit for bit (ties keep particle order)."""
    w = _absorption(n_gas=40000, n_star=10000, xres=192, yres=108, tile=16, order=order)
    prm = dict(w.params.params)
    prm["sort_type"] = str(sort_type)
    g = gpu_frame(renderer, prm, w.rc, w.particles)
    o = oracle_frame(port, prm, w.rc, w.particles, fp32=False)
    assert_parity(g, o)
    if sort_type:
        assert not np.array_equal(g.order, np.sort(g.order)), "the sort left particle order"
