"""The oracle's FP64 adjoint (model chain rule + exact reverse-mode splat)
against FP64 central finite differences of the same frozen-coverage model, on
small frames in both modes and both projections.  This pins the checker that
the GPU gradients are compared with.  The model is anchored at the render's
float-rounded projected values, so the loss is formed there too."""
import numpy as np
import pytest

from splotch_gb300 import synth


def _case(port, mode, projection, n=4000, xres=96, yres=64):
    w = synth.differentiable(n=n, mode=mode, xres=xres, yres=yres, tile=16)
    prm = dict(w.params.params)
    prm["projection"] = projection
    raw = w.particles.copy()
    cov = raw.copy()
    port.project_colorize(prm, w.rc, cov)
    order = None if mode == "additive" else port.sort_perm(cov, 1)
    tp = w.notes["target"].copy()
    port.project_colorize(prm, w.rc, tp)
    torder = None if mode == "additive" else port.sort_perm(tp, 1)
    target, _ = port.render_fp64(tp, torder, xres, yres, 16, mode == "additive", 0.2)
    target = target.astype(np.float32)
    # the loss at the render's own values (the model is anchored there)
    W = np.stack([cov[k].astype(np.float64) for k in ("x", "y", "r", "er", "eg", "eb")], 1)
    W[~cov["active"].astype(bool)] = 0.0
    pic = port.render_frozen_fp64(prm, cov, np.ascontiguousarray(W), order)
    return w, prm, raw, cov, order, target, 2.0 * (pic - target)


@pytest.mark.parametrize("projection", [True, False])
@pytest.mark.parametrize("mode", ["additive", "absorption"])
def test_oracle_adjoint_matches_finite_differences(mode, projection, port):
    w, prm, raw, cov, order, target, gpic = _case(port, mode, projection)
    grad, gc = port.grad_fp64(prm, w.rc, raw, cov, order, gpic)
    act = np.nonzero(cov["active"])[0]
    assert len(act) > 500
    sel = np.random.default_rng(1).choice(act, size=64, replace=False)
    fd, excluded = port.fd_particles(prm, w.rc, raw, cov, order, target, sel)
    for j, f in enumerate(port.GRAD_FIELDS):
        keep = ~excluded[:, j]
        a, b = grad[sel][keep, j], fd[keep, j]
        scale = np.abs(b).max()
        if scale == 0.0:
            assert np.abs(a).max() == 0.0, f
            continue
        err = (np.abs(a - b) / np.maximum(np.abs(b), 1e-4 * scale)).max()
        assert err < 1e-4, (f, err)
    fdc = port.fd_campos(prm, w.rc, raw, cov, order, target)
    np.testing.assert_allclose(gc, fdc, rtol=1e-5, atol=1e-6 * np.abs(fdc).max())


def test_inactive_particles_have_zero_gradient(port):
    w, prm, raw, cov, order, target, gpic = _case(port, "absorption", True, n=2000)
    grad, _ = port.grad_fp64(prm, w.rc, raw, cov, order, gpic)
    assert np.all(grad[~cov["active"].astype(bool)] == 0.0)
