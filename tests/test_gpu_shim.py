"""The host_rendering() drop-in's own C++ code on the GPU.

splotch_gb300/shim/host_rendering_impl.h holds the drop-in's logic -- keys and
defaults, palettes and camera from the render context, the particle vector
mutated in place, errors -- over the caller's types.  Inside the Splotch tree
it is bound to Splotch's types (host_rendering_gb300.cc, link-tested against
the reference in test_shim_link.py); here tests/shim/shim_frame.cc binds it to
minimal stand-ins, is compiled against libsplgpu.so and renders frames from
files this test writes.  Checked against the oracle: the image within 1e-4 of
FP64, the caller's particle vector after the call bit for bit (projected,
colourised, stably depth-sorted), the ray-sphere renderer's image and its
emptied vector, inserted defaults, and an error for a bad key value.
"""
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

import splotch_gb300 as sg
from oracle.oracle import rel_linf
from splotch_gb300 import synth

from .helpers import IMAGE_TOL

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def shim_exe(built, tmp_path_factory):
    exe = tmp_path_factory.mktemp("shim") / "shim_frame"
    lib = ROOT / "splotch_gb300"
    cmd = ["g++", "-O2", "-std=c++11", "-I", str(ROOT / "include"), "-I", str(lib / "shim"),
           str(ROOT / "tests" / "shim" / "shim_frame.cc"), "-L", str(lib), "-lsplgpu",
           f"-Wl,-rpath,{lib}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _write(d: Path, params: dict, rc, particles: np.ndarray) -> None:
    d.mkdir(parents=True, exist_ok=True)
    (d / "params.txt").write_text("".join(f"{k}={v}\n" for k, v in params.items()))
    b = bytearray()
    for v in (rc.campos, rc.lookat, rc.sky, rc.centerpos):
        b += struct.pack("<3d", *[float(x) for x in v])
    b += struct.pack("<f", float(rc.b_brightness))
    pals = rc.amap
    b += struct.pack("<i", len(pals))
    for p in pals:
        if p is None:
            b += struct.pack("<i", 0)
            continue
        b += struct.pack("<i", len(p.x))
        b += np.asarray(p.x, "<f8").tobytes() + np.asarray(p.rgb, "<f4").tobytes()
    (d / "context.bin").write_bytes(bytes(b))
    (d / "particles.bin").write_bytes(struct.pack("<q", len(particles)) + particles.tobytes())


def _run(exe, d: Path):
    r = subprocess.run([str(exe), str(d)], capture_output=True, text=True, timeout=300)
    return r.returncode, r.stdout


def _outputs(d: Path, xres: int, yres: int):
    pic = np.fromfile(d / "pic.bin", np.float32).reshape(xres, yres, 3)
    raw = (d / "particles_out.bin").read_bytes()
    n = struct.unpack("<q", raw[:8])[0]
    parts = np.frombuffer(raw[8:], dtype=sg.PARTICLE_DTYPE, count=n).copy()
    kv = dict(line.split("=", 1) for line in (d / "params_out.txt").read_text().splitlines())
    return pic, parts, kv


@pytest.mark.parametrize("order", [None, "btf"])
def test_drop_in_absorption_frame(order, shim_exe, port, tmp_path):
    w = synth.plain_absorption(n_gas=40000, n_star=10000, xres=192, yres=108, tile=16)
    prm = {k: v for k, v in w.params.params.items() if k != "gpu_order"}
    if order:
        prm["gpu_order"] = order
    _write(tmp_path, prm, w.rc, w.particles)
    rc, out = _run(shim_exe, tmp_path)
    assert rc == 0, out
    pic, parts, kv = _outputs(tmp_path, 192, 108)
    # the caller's vector: projected, colourised and stably sorted by depth
    ref = w.particles.copy()
    port.project_colorize(prm, w.rc, ref)
    ref = ref[port.sort_perm(ref, 1)]
    assert np.array_equal(parts.view(np.uint8), ref.view(np.uint8))
    pic64, _ = port.render_fp64(ref, None, 192, 108, 16, False, 0.2)
    err = rel_linf(pic, pic64)
    assert err <= IMAGE_TOL, err
    # keys the reference reads were inserted with their defaults
    for k, v in (("zmax", None), ("zmin", None), ("minrad_pix", None), ("projection", "T"),
                 ("smooth_factor0", None), ("gpu_writeback", "T")):
        assert k in kv and (v is None or kv[k] == v), k
    print("shim absorption", order, err)


def test_drop_in_additive_frame_without_writeback(shim_exe, port, tmp_path):
    w = synth.plain_additive(n=40000, xres=160, yres=120, tile=16)
    prm = dict(w.params.params, gpu_writeback="F")
    _write(tmp_path, prm, w.rc, w.particles)
    rc, out = _run(shim_exe, tmp_path)
    assert rc == 0, out
    pic, parts, _ = _outputs(tmp_path, 160, 120)
    assert np.array_equal(parts.view(np.uint8), w.particles.view(np.uint8))  # untouched
    ref = w.particles.copy()
    port.project_colorize(prm, w.rc, ref)
    pic64, _ = port.render_fp64(ref, None, 160, 120, 16, True, 0.2)
    assert rel_linf(pic, pic64) <= IMAGE_TOL


def test_drop_in_ray_sphere_frame(shim_exe, port, tmp_path):
    w = synth.plain_additive(n=20000, xres=128, yres=128, tile=16)
    prm = dict(w.params.params, new_renderer="T")
    _write(tmp_path, prm, w.rc, w.particles)
    rc, out = _run(shim_exe, tmp_path)
    assert rc == 0, out
    pic, parts, _ = _outputs(tmp_path, 128, 128)
    assert len(parts) == 0  # host_rendering_new empties the vector
    want, _ = port.render_rays(prm, w.rc, w.particles, exact=True)
    assert rel_linf(pic, want) <= IMAGE_TOL


def test_drop_in_reports_errors(shim_exe, tmp_path):
    w = synth.plain_additive(n=100, xres=64, yres=64, tile=16)
    prm = dict(w.params.params, ptypes="9")
    _write(tmp_path, prm, w.rc, w.particles)
    rc, out = _run(shim_exe, tmp_path)
    assert rc == 3 and "ptypes must be in [1,8]" in out
