"""Post-processing and image output after host_rendering (splotch.cc:272-323):
-expm1 with exptable<float32>(-20) for additive frames, colour_adjust, colour
bar, and LS_Image's TGA / PPM / run-length TGA bytes.

CPU: the oracle's restatement against golden fixtures made by the reference's
own code (tests/golden/make_golden.py), bit for bit.  GPU: spl_postprocess and
spl_image_encode against the same fixtures and against the oracle on the same
host.  pow() in colour_adjust comes from each machine's math library, so the
adjusted values may differ in the last bit between machines (compared within
2 float ulps there; bit for bit with the oracle on the same host).
"""
import json
from pathlib import Path

import numpy as np
import pytest

import splotch_gb300 as sg
from oracle.oracle import Port

GOLDEN = Path(__file__).resolve().parent / "golden"
VARIANTS = {"plain": {}, "adjusted": {"pic_gamma": "0.8", "pic_brightness": "0.05",
                                      "pic_contrast": "1.3", "colorbar": "T"}}


def _load(name):
    g = np.load(GOLDEN / f"post_{name}.npz")
    meta = json.loads(bytes(g["meta"]).decode())
    pals = [None if p is None else sg.Palette(np.array(p["x"]), np.array(p["rgb"], np.float32))
            for p in meta["palettes"]]
    rc = sg.RenderContext(campos=np.array(meta["campos"]), centerpos=np.array(meta["centerpos"]),
                          lookat=np.array(meta["lookat"]), sky=np.array(meta["sky"]), amap=pals,
                          b_brightness=meta["b_brightness"])
    prm = dict(meta["params"])
    a_eq_e = prm.get("a_eq_e", "T") in ("T", "True", "true")
    return g, prm, rc, a_eq_e


def _ulps(a, b):
    ia = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    ib = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return int(np.abs(ia - ib).max()) if ia.size else 0


@pytest.mark.parametrize("name", ["additive", "absorption"])
def test_oracle_post_matches_reference(name, built):
    port = Port()
    g, prm, rc, a_eq_e = _load(name)
    for var, extra in VARIANTS.items():
        q = dict(prm)
        q.update(extra)
        got = port.postprocess(q, rc, g["pic_in"], a_eq_e)
        assert np.array_equal(got, g[f"post_{var}"]), var
        for pt in (0, 2, 3):
            assert port.image_bytes(g[f"post_{var}"], pt) == g[f"bytes_{var}_{pt}"].tobytes(), \
                (var, pt)


def test_oracle_image_rejects_bad_pictype(built):
    with pytest.raises(ValueError):
        Port().image_bytes(np.zeros((4, 3, 3), np.float32), 5)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["additive", "absorption"])
def test_gpu_post_matches_reference(name, renderer):
    port = Port()
    g, prm, rc, a_eq_e = _load(name)
    for var, extra in VARIANTS.items():
        q = dict(prm)
        q.update(extra)
        pic = np.ascontiguousarray(g["pic_in"]).copy()
        sg.postprocess(sg.ParamFile(q), rc, renderer, pic)
        want = g[f"post_{var}"]
        if var == "plain":
            assert np.array_equal(pic, want)
        else:
            assert _ulps(pic, want) <= 2
            assert np.array_equal(pic, port.postprocess(q, rc, g["pic_in"], a_eq_e))
        for pt in (0, 2, 3):
            got = sg.encode_image(want, pt, renderer)
            assert got == g[f"bytes_{var}_{pt}"].tobytes(), (var, pt)


@pytest.mark.gpu
def test_gpu_write_image_and_device_input(renderer, tmp_path):
    torch = pytest.importorskip("torch")
    g, prm, rc, a_eq_e = _load("additive")
    want = g["post_adjusted"]
    dev = torch.from_numpy(want.copy()).cuda()
    torch.cuda.synchronize()
    assert sg.encode_image(dev, 3, renderer) == g["bytes_adjusted_3"].tobytes()
    rc.pic = want.copy()
    path = sg.write_image(sg.ParamFile({"pictype": 2}), rc, str(tmp_path / "frame"), renderer)
    assert Path(path).read_bytes() == g["bytes_adjusted_2"].tobytes()
    with pytest.raises(sg._abi.SplotchError):
        sg.write_image(sg.ParamFile({"pictype": 1}), rc, str(tmp_path / "x"), renderer)
