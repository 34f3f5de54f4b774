"""Gradients of the render (spl_render_backward) on the GPU.

Checks, for the additive and the ordered absorption mode:
* against the FP64 CPU adjoint of the oracle (every active particle), given
  the same dL/dpic;
* against FP64 central finite differences (step 1e-4) of
  L = sum((pic - target)^2) on a random subset of 256 particles and for the
  camera position, coverage held at the forward's decisions; a palette kink
  between v-h and v+h excludes that colour entry;
* through torch.autograd (splotch_gb300.autograd), equal to the direct call.

Tolerance, per input field over the checked particles:
* relative L-inf normalised by the field's largest magnitude,
  max|g - g_ref| / max|g_ref| <= GRAD_TOL = 1e-3;
* median per-element relative error <= GRAD_MEDIAN = 2e-4;
* per-element relative error with a floor of 1% of the field maximum,
  |g - g_ref| / max(|g_ref|, 1e-2 * max|g_ref|) <= GRAD_ELEM = 1e-2.
Per-element errors grow where a gradient is a near-cancelling sum (dL/dz is
-(f/zc)(dL/dX*xc + dL/dY*yc) + ...): FP32 terms carry ~1e-7 relative error
each, so an element far below the field's scale is only as accurate as the
cancellation allows.
"""
import numpy as np
import pytest

import splotch_gb300 as sg
from splotch_gb300 import _abi, synth

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-3
GRAD_MEDIAN = 2e-4
GRAD_ELEM = 1e-2
FIELDS = _abi.GRAD_FIELDS  # I, cr, cg, cb, x, y, z, r


def rel_err(g, ref, floor):
    scale = np.abs(ref).max() if ref.size else 0.0
    if scale == 0.0:
        return np.abs(g).max() if g.size else 0.0
    return float((np.abs(g - ref) / np.maximum(np.abs(ref), floor * scale)).max())


def grad_errors(g, ref) -> tuple[float, float, float]:
    """(max-normalised L-inf, median element error, element error at floor 1e-2)."""
    scale = np.abs(ref).max() if ref.size else 0.0
    if scale == 0.0:
        e = float(np.abs(g).max()) if g.size else 0.0
        return e, e, e
    d = np.abs(g - ref)
    nz = np.abs(ref) > 0
    med = float(np.median(d[nz] / np.abs(ref[nz]))) if nz.any() else 0.0
    return float(d.max() / scale), med, rel_err(g, ref, 1e-2)


def check_field(g, ref, what: str) -> list:
    linf, med, elem = grad_errors(g, ref)
    bad = []
    if linf > GRAD_TOL:
        bad.append(f"{what}: L-inf/max {linf:.2e}")
    if med > GRAD_MEDIAN:
        nz = np.abs(ref) > 0
        bad.append(f"{what}: median {med:.2e} over {int(nz.sum())}/{ref.size} "
                   f"(all: {np.median(np.abs(g - ref) / np.maximum(np.abs(ref), 1e-300)):.2e})")
    if elem > GRAD_ELEM:
        bad.append(f"{what}: element {elem:.2e}")
    return bad


def describe(g, ref) -> str:
    """Error profile: worst element relative to the field maximum, the error at
    floors 1e-3 and 1e-2, the median relative error and the max-normalised error."""
    scale = np.abs(ref).max()
    if scale == 0.0:
        return "all zero"
    nz = np.abs(ref) > 0
    r = np.abs(g - ref)[nz] / np.abs(ref[nz])
    g, ref = g[nz], ref[nz]
    i = int(np.argmax(np.abs(g - ref) / np.maximum(np.abs(ref), 1e-3 * scale)))
    return (f"worst |ref|/max={abs(ref[i]) / scale:.2e} err={r[i]:.2e}; floor1e-3 "
            f"{rel_err(g, ref, 1e-3):.2e} floor1e-2 {rel_err(g, ref, 1e-2):.2e} median "
            f"{np.median(r):.2e} linf/max {np.abs(g - ref).max() / scale:.2e}")


def _frame(renderer, w, target_particles):
    """GPU forward of the target and of the frame, then backward of
    L = sum((pic - target)^2).  Returns pic, target, gpic, grads."""
    keep: list = []
    desc = sg.frame_desc(w.params, w.rc, keep)
    shape = (desc.xres, desc.yres, 3)
    target = np.zeros(shape, np.float32)
    renderer.render_aos(desc, target_particles.copy(), target)
    pic = np.zeros(shape, np.float32)
    renderer.set_differentiable(True)
    try:
        renderer.render_aos(desc, w.particles.copy(), pic)
    finally:
        renderer.set_differentiable(False)
    gpic = (2.0 * (pic - target)).astype(np.float32)
    grads = renderer.backward(gpic)
    return pic, target, gpic, grads


def _oracle_inputs(port, w):
    prm = dict(w.params.params)
    raw = w.particles.copy()
    cov = raw.copy()
    port.project_colorize(prm, w.rc, cov)
    a_eq_e = str(prm.get("a_eq_e")) in ("True", "T", "true", "1")
    order = None if a_eq_e else port.sort_perm(cov, 1)
    return prm, raw, cov, order


def _gpu_matrix(grads, n):
    return np.stack([np.asarray(grads[f], np.float64)[:n] for f in FIELDS], axis=1)


@pytest.mark.parametrize("mode", ["additive", "absorption"])
def test_backward_matches_fp64_adjoint(mode, renderer, port):
    w = synth.differentiable(n=120_000, mode=mode, xres=256, tile=16)
    _, _, gpic, grads = _frame(renderer, w, w.notes["target"])
    prm, raw, cov, order = _oracle_inputs(port, w)
    g64, gc64 = port.grad_fp64(prm, w.rc, raw, cov, order, gpic.astype(np.float64))
    g32 = _gpu_matrix(grads, len(raw))
    act = cov["active"].astype(bool)
    assert act.sum() > 10_000
    assert np.all(g32[~act] == 0.0)
    bad = []
    for j, f in enumerate(FIELDS):
        print(mode, f, "vs FP64 adjoint:", describe(g32[act, j], g64[act, j]))
        bad += check_field(g32[act, j], g64[act, j], f)
    assert not bad, bad
    ec = np.abs(grads["campos"] - gc64).max() / np.abs(gc64).max()
    print(mode, "campos", grads["campos"], gc64, ec)
    assert ec <= GRAD_TOL


@pytest.mark.parametrize("mode", ["additive", "absorption"])
@pytest.mark.parametrize("n,res", [(120_000, 256), (4_000_000, 1024)])
def test_backward_matches_finite_differences(mode, n, res, renderer, port):
    w = synth.differentiable(n=n, mode=mode, xres=res, tile=16)
    _, target, _, grads = _frame(renderer, w, w.notes["target"])
    prm, raw, cov, order = _oracle_inputs(port, w)
    act = np.nonzero(cov["active"])[0]
    sel = np.sort(np.random.default_rng(3).choice(act, size=256, replace=False))
    fd, excluded = port.fd_particles(prm, w.rc, raw, cov, order, target, sel, h=1e-4)
    g32 = _gpu_matrix(grads, len(raw))[sel]
    bad = []
    for j, f in enumerate(FIELDS):
        keep = ~excluded[:, j]
        print(mode, n, f, "vs FD:", describe(g32[keep, j], fd[keep, j]), "excluded",
              int((~keep).sum()))
        bad += check_field(g32[keep, j], fd[keep, j], f)
    assert not bad, bad
    fdc = port.fd_campos(prm, w.rc, raw, cov, order, target, h=1e-4)
    ec = np.abs(grads["campos"] - fdc).max() / np.abs(fdc).max()
    print(mode, n, "campos", grads["campos"], fdc, ec)
    assert ec <= GRAD_TOL


def test_autograd_function_equals_direct_call(renderer):
    torch = pytest.importorskip("torch")
    from splotch_gb300.autograd import render

    w = synth.differentiable(n=60_000, mode="absorption", xres=192, tile=16)
    p = w.particles
    _, target, _, direct = _frame(renderer, w, w.notes["target"])
    dev = "cuda"
    I = torch.from_numpy(p["I"].copy()).to(dev).requires_grad_()
    col = torch.from_numpy(np.stack([p["er"], p["eg"], p["eb"]], 1)).to(dev).requires_grad_()
    pos = torch.from_numpy(np.stack([p["x"], p["y"], p["z"]], 1)).to(dev).requires_grad_()
    hsml = torch.from_numpy(p["r"].copy()).to(dev).requires_grad_()
    campos = torch.tensor(np.asarray(w.rc.campos, np.float64), requires_grad=True)
    ptype = torch.from_numpy(p["type"].astype(np.int16)).to(dev)
    pic = render(I, col, pos, hsml, campos, renderer, w.params, w.rc, ptype)
    loss = ((pic - torch.from_numpy(target).to(dev)) ** 2).sum()
    loss.backward()
    torch.cuda.synchronize()
    got = {"I": I.grad, "cr": col.grad[:, 0], "cg": col.grad[:, 1], "cb": col.grad[:, 2],
           "x": pos.grad[:, 0], "y": pos.grad[:, 1], "z": pos.grad[:, 2], "r": hsml.grad}
    renderer.set_differentiable(False)
    for f in FIELDS:
        np.testing.assert_allclose(got[f].cpu().numpy(), direct[f], rtol=1e-5, atol=1e-7 *
                                   max(1.0, float(np.abs(direct[f]).max())), err_msg=f)
    np.testing.assert_allclose(campos.grad.numpy(), direct["campos"], rtol=1e-5)


def test_backward_argument_checks(renderer):
    w = synth.differentiable(n=5_000, mode="absorption", xres=64, tile=16)
    keep: list = []
    desc = sg.frame_desc(w.params, w.rc, keep)
    parts = w.particles.copy()
    pic = np.zeros((64, 64, 3), np.float32)
    renderer.render_aos(desc, parts, pic, writeback=True)
    with pytest.raises(_abi.SplotchError):
        renderer.backward(np.zeros_like(pic))
    # an ordered frame rendered without the differentiable switch
    renderer.set_differentiable(False)
    renderer.render_aos(desc, w.particles.copy(), pic)
    with pytest.raises(_abi.SplotchError):
        renderer.backward(np.zeros_like(pic))
    fresh = sg.Renderer(0)
    try:
        with pytest.raises(_abi.SplotchError):
            fresh.backward(np.zeros_like(pic))
    finally:
        fresh.close()
