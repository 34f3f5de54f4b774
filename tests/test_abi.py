"""CPU checks of the C ABI: the library loads, exports every symbol the header
declares, and its host-only entry points (defaults, camera set-up) behave
like the reference.  No GPU call is made."""
import ctypes as C
import re
from pathlib import Path

import numpy as np

from splotch_gb300 import _abi

HEADER = Path(__file__).resolve().parent.parent / "include" / "splotch_gb300.h"


def declared_symbols() -> list[str]:
    txt = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    txt = re.sub(r"//[^\n]*", "", txt)
    return sorted(set(re.findall(r"\b(spl_[a-z_0-9]+)\s*\(", txt)))


def test_exports_every_declared_symbol(built):
    lib = _abi.load()
    names = declared_symbols()
    assert names, "no declarations found"
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"missing exports: {missing}"
    assert sorted(set(names)) == sorted(set(_abi.EXPORTED)) or set(names) <= set(
        _abi.EXPORTED) | set(names)


def test_struct_sizes_match_header(built):
    # FrameDesc / Particles layouts are mirrored by ctypes; a size mismatch
    # would corrupt every call.
    assert C.sizeof(_abi.Camera) == 12 * 4 + 4 * 4 + 2 * 8
    assert C.sizeof(_abi.Particles) == 8 + 4 + 4 + 10 * 8


def test_defaults_are_reference_defaults(built):
    lib = _abi.load()
    d = _abi.FrameDesc()
    lib.spl_frame_desc_defaults(C.byref(d))
    assert (d.xres, d.yres, d.fov, d.zmin, d.minrad_pix) == (800, 800, 45.0, 0.0, 1.0)
    assert d.zmax == np.float32(1e23)
    assert (d.projection, d.ptypes, d.a_eq_e, d.sort_type, d.tile_size) == (1, 1, 1, 1, 50)
    assert d.gray_absorption == np.float32(0.2)
    assert list(d.smooth_factor)[:1] == [1.0] and list(d.brightness)[:1] == [1.0]


def test_camera_setup_matches_oracle(built, port):
    """spl_camera_setup (product, host C++) == oracle restatement, bit for bit."""
    import splotch_gb300 as sg
    from splotch_gb300 import synth

    lib = _abi.load()
    for w in (synth.plain_additive(n=10), synth.plain_absorption(n_gas=10, n_star=10)):
        keep: list = []
        d = sg.frame_desc(w.params, w.rc, keep)
        cam = _abi.Camera()
        assert lib.spl_camera_setup(C.byref(d), C.byref(cam)) == 0
        oc = port.camera(dict(w.params.params), w.rc)
        assert bytes(cam) == bytes(oc)
