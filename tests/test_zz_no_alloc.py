"""spl_sort_pairs_noalloc, the depth sort with its scratch in a static device
array, against spl_render through the C ABI.

The active particles' depth keys of a frame, sorted with their particle
indices as values, must come out in the visiting order spl_render computed for
that frame, bit for bit, on two calls in a row (the one scratch array is reused
and nothing clears it).  Further cases: partial key widths and many ties
against a stable numpy sort, the maximum size, rejection of oversize and
invalid arguments before anything is launched, and no change of the device's
free memory across calls.
"""
import numpy as np
import pytest

import splotch_gb300 as sg
from splotch_gb300 import _abi, synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

MAX = _abi.SPL_NOALLOC_MAX_PAIRS


def _depth_keys(z: np.ndarray) -> np.ndarray:
    """Radix key of a depth: unsigned order == float order, -0 == +0."""
    b = np.ascontiguousarray(z, dtype=np.float32).view(np.uint32).copy()
    b[(b << np.uint32(1)) == 0] = 0
    return np.where(b & np.uint32(0x80000000), ~b, b | np.uint32(0x80000000)).astype(np.uint32)


def _dev(a: np.ndarray):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def _sort(lib, kd, vd, n, bits=32, out=None):
    ko, vo = out if out is not None else (torch.empty(max(n, 1), dtype=torch.int32, device="cuda"),
                                          torch.empty(max(n, 1), dtype=torch.int32, device="cuda"))
    stream = torch.cuda.current_stream().cuda_stream
    _abi.check(lib.spl_sort_pairs_noalloc(kd.data_ptr(), vd.data_ptr() if vd is not None else None,
                                          ko.data_ptr(), vo.data_ptr(), n, bits, stream))
    torch.cuda.synchronize()
    return (ko[:n].cpu().numpy().view(np.uint32).copy(),
            vo[:n].cpu().numpy().view(np.uint32).copy())


def test_noalloc_sort_gives_render_visiting_order(renderer):
    lib = _abi.load()
    w = synth.plain_absorption(n_gas=1_600_000, n_star=400_000, xres=640, yres=360, tile=16,
                               order="btf")
    keep: list = []
    desc = sg.frame_desc(w.params, w.rc, keep)
    assert desc.sort_type == 1 and not desc.a_eq_e
    pic = np.zeros((desc.xres, desc.yres, 3), np.float32)
    n = len(w.particles)
    renderer.render_aos(desc, w.particles.copy(), pic)
    proj = renderer.projected(n)
    order = renderer.order(n)
    act = np.nonzero(proj["active"])[0].astype(np.uint32)
    assert 16 * 4096 < len(act) <= MAX and len(order) == len(act)
    keys = _depth_keys(proj["z"][act])
    kd, vd = _dev(keys), _dev(act)
    for _ in range(2):  # two calls in a row on the same scratch
        ko, vo = _sort(lib, kd, vd, len(act))
        assert np.array_equal(vo, order), "order differs from spl_render's depth sort"
        assert np.array_equal(ko, np.sort(keys))
    # values NULL: the sort returns positions 0..n-1 in sorted order
    _, pos = _sort(lib, kd, None, len(act))
    assert np.array_equal(act[pos], order)


@pytest.mark.parametrize("bits", [8, 12, 16, 20, 32])  # 1, 2, 2, 3 and 4 digit passes
def test_noalloc_sort_stable_with_ties(bits):
    lib = _abi.load()
    rng = np.random.default_rng(bits)
    n = 300_001
    keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    keys[::3] = keys[0]  # many equal keys
    vals = rng.permutation(n).astype(np.uint32)
    p = np.argsort(keys & np.uint32((1 << bits) - 1 if bits < 32 else 0xFFFFFFFF), kind="stable")
    for _ in range(2):
        ko, vo = _sort(lib, _dev(keys), _dev(vals), n, bits)
        assert np.array_equal(vo, vals[p]) and np.array_equal(ko, keys[p])


def test_noalloc_sort_maximum_size_and_no_allocation():
    lib = _abi.load()
    rng = np.random.default_rng(7)
    keys = rng.integers(0, 2**32, MAX, dtype=np.uint64).astype(np.uint32)
    kd, vd = _dev(keys), _dev(np.arange(MAX, dtype=np.uint32))
    out = (torch.empty(MAX, dtype=torch.int32, device="cuda"),
           torch.empty(MAX, dtype=torch.int32, device="cuda"))
    p = np.argsort(keys, kind="stable")
    ko, vo = _sort(lib, kd, vd, MAX, out=out)  # first call: set-up and module loading
    assert np.array_equal(vo, p) and np.array_equal(ko, keys[p])
    reserved0 = torch.cuda.memory_reserved()
    # The device's free memory must not move across the calls.  Another process
    # on the same GPU could move it meanwhile, so up to three tries are allowed;
    # an allocation by the call itself would show on every try.
    same = False
    for _ in range(3):
        free0 = torch.cuda.mem_get_info()[0]
        for _ in range(2):
            ko, vo = _sort(lib, kd, vd, MAX, out=out)
            assert np.array_equal(vo, p)
        if torch.cuda.mem_get_info()[0] == free0:
            same = True
            break
    assert same, "the device's free memory changed across spl_sort_pairs_noalloc calls"
    assert torch.cuda.memory_reserved() == reserved0


def test_noalloc_sort_rejects_before_launch():
    lib = _abi.load()
    kd = torch.zeros(64, dtype=torch.int32, device="cuda")
    ko = torch.zeros(64, dtype=torch.int32, device="cuda")
    vo = torch.zeros(64, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    f = lib.spl_sort_pairs_noalloc
    # more pairs than the fixed capacity: refused, nothing touched
    assert f(kd.data_ptr(), None, ko.data_ptr(), vo.data_ptr(), MAX + 1, 32, s) == \
        _abi.SPL_ERR_CAPACITY
    assert b"capacity" in lib.spl_last_error_string()
    assert f(kd.data_ptr(), None, ko.data_ptr(), vo.data_ptr(), -1, 32, s) == _abi.SPL_ERR_INVALID
    assert f(kd.data_ptr(), None, ko.data_ptr(), vo.data_ptr(), 8, 0, s) == _abi.SPL_ERR_INVALID
    assert f(kd.data_ptr(), None, ko.data_ptr(), vo.data_ptr(), 8, 33, s) == _abi.SPL_ERR_INVALID
    # misaligned keys (input, and output: read back 16 bytes at a time when
    # three or four digit passes run), host memory, overlapping outputs
    assert f(kd.data_ptr() + 4, None, ko.data_ptr(), vo.data_ptr(), 8, 32, s) == \
        _abi.SPL_ERR_INVALID
    assert f(kd.data_ptr(), None, ko.data_ptr() + 4, vo.data_ptr(), 8, 32, s) == \
        _abi.SPL_ERR_INVALID
    assert b"keys_out" in lib.spl_last_error_string()
    host = np.zeros(64, np.uint32)
    assert f(host.ctypes.data, None, ko.data_ptr(), vo.data_ptr(), 8, 32, s) == \
        _abi.SPL_ERR_INVALID
    assert f(kd.data_ptr(), None, ko.data_ptr(), ko.data_ptr() + 16, 8, 32, s) == \
        _abi.SPL_ERR_INVALID
    assert f(kd.data_ptr(), None, kd.data_ptr(), vo.data_ptr(), 8, 32, s) == _abi.SPL_ERR_INVALID
    # empty input is a no-op
    assert f(kd.data_ptr(), None, ko.data_ptr(), vo.data_ptr(), 0, 32, s) == _abi.SPL_OK
    torch.cuda.synchronize()
    assert int(ko.abs().sum()) == 0 and int(vo.abs().sum()) == 0
