"""Shared helpers of the parity tests: run one frame through the C ABI and the
same frame through the oracle, and compare stage by stage."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

import splotch_gb300 as sg
from oracle.oracle import rel_linf

IMAGE_TOL = 1e-4  # per-pixel relative L-inf vs the FP64 oracle (floor 1e-6*max)


@dataclass
class FrameResult:
    pic: np.ndarray
    projected: np.ndarray
    order: np.ndarray
    tile_start: np.ndarray
    entries: np.ndarray
    stats: dict


def gpu_frame(renderer: sg.Renderer, params: dict, rc, particles: np.ndarray) -> FrameResult:
    keep: list = []
    desc = sg.frame_desc(sg.ParamFile(dict(params)), rc, keep)
    pic = np.zeros((desc.xres, desc.yres, 3), np.float32)
    parts = particles.copy()
    renderer.render_aos(desc, parts, pic)
    T = desc.tile_size
    ntiles = ((desc.xres + T - 1) // T) * ((desc.yres + T - 1) // T)
    ts, ent = renderer.bins(ntiles)
    st = renderer.stats()
    st["fragments"] = renderer.fragments()
    return FrameResult(pic, renderer.projected(len(parts)), renderer.order(len(parts)), ts, ent,
                       st)


@dataclass
class OracleResult:
    projected: np.ndarray
    order: np.ndarray | None
    tile_start: np.ndarray
    entries: np.ndarray
    pic64: np.ndarray
    pic32: np.ndarray
    frags: int


def oracle_frame(port, params: dict, rc, particles: np.ndarray, fp32: bool = True) -> OracleResult:
    p = particles.copy()
    port.project_colorize(params, rc, p)
    a_eq_e = str(params.get("a_eq_e", "T")) in ("T", "True", "true", "1")
    st = int(params.get("sort_type", 1))
    order = port.sort_perm(p, st) if (not a_eq_e and st != 0) else None
    xres = int(params.get("xres", 800))
    yres = int(params.get("yres", xres))
    T = int(float(params.get("tile_size_cpu", 50)))
    gray = float(params.get("gray_absorption", 0.2))
    ts, ent = port.bins(p, order, xres, yres, T)
    pic64, frags = port.render_fp64(p, order, xres, yres, T, a_eq_e, gray)
    pic32 = port.render_fp32(p, order, xres, yres, T, a_eq_e, gray, simd=False)[0] if fp32 \
        else None
    return OracleResult(p, order, ts, ent, pic64, pic32, frags)


def assert_parity(g: FrameResult, o: OracleResult, tol: float = IMAGE_TOL) -> dict:
    n = len(o.projected)
    gb, ob = g.projected.view(np.uint8).reshape(n, 36), o.projected.view(np.uint8).reshape(n, 36)
    bad = np.nonzero((gb != ob).any(axis=1))[0]
    assert bad.size == 0, (f"{bad.size} projected particles differ, first {bad[:5]}: "
                           f"gpu {g.projected[bad[:2]]} oracle {o.projected[bad[:2]]}")
    full = o.order if o.order is not None else np.arange(n, dtype=np.uint32)
    want_order = full[o.projected["active"][full].astype(bool)]  # active particles, in order
    assert np.array_equal(g.order, want_order), "visiting order (sort permutation) differs"
    assert np.array_equal(g.tile_start, o.tile_start), "tile ranges differ"
    assert np.array_equal(g.entries, o.entries), "tile bin entries differ"
    assert g.stats["fragments"] == o.frags, "fragment count differs from the reference loop"
    err = rel_linf(g.pic, o.pic64)
    ref_err = rel_linf(o.pic32, o.pic64) if o.pic32 is not None else None
    assert err <= tol, f"image rel Linf vs FP64 oracle {err:.3e} > {tol:.0e} (reference FP32: {ref_err})"
    return {"gpu_err": err, "ref_fp32_err": ref_err, "frags": o.frags}
