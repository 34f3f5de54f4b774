"""bench.py's output contract, checked on the CPU: the reference arm's JSON
line (run on a small sample), its silence on ranks other than 0, and the
roofline arithmetic of the GPU arm's line."""
import json
import os
import subprocess
import sys
from pathlib import Path
from types import SimpleNamespace

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def run_bench(*args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True,
                          text=True, timeout=600, env=e, cwd=ROOT)


def test_reference_arm_line(built):
    r = run_bench("--impl", "reference", "--steps", "1", "--warmup", "1", "--scale", "0.02")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["unit"] == "Mparticles/s" and d["metric"] == bench.METRIC
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference")
    assert "workload" in d["config"]


def test_reference_arm_other_ranks_are_silent(built):
    r = run_bench("--impl", "reference", "--steps", "1", "--warmup", "1", "--scale", "0.02",
                  env={"RANK": "1", "WORLD_SIZE": "2"})
    assert r.returncode == 0 and not r.stdout.strip()


def test_roofline_arithmetic():
    stages = {"project_ms": 1.0, "sort_ms": 0.5, "bin_ms": 1.5, "splat_ms": 6.0}
    pk = {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0, "source": "measured"}
    top, st = bench.roofline(stages, n=50_000_000, n_act=7_800_000, n_entries=37_000_000,
                             n_tiles=8160, frags=3_770_000_000, args=SimpleNamespace(),
                             pk=pk, a_eq_e=False, n_sm=152)
    assert top["stage"] == "splat" and top["kernel"] == "k_splat"
    # the FP32 rate follows the SM count it is given; the splat's traffic is the
    # committed capture's bytes scaled by the fragment count
    assert top["peak"] == pytest.approx(2 * 128 * 152 * 2070e6 / 1e12)
    assert top["traffic"] == pytest.approx(bench.SPLAT_CAPTURE["dram_bytes"] * 3_770_000_000 /
                                           bench.SPLAT_CAPTURE["fragments"])
    top148, _ = bench.roofline(stages, 50_000_000, 7_800_000, 37_000_000, 8160, 3_770_000_000,
                               SimpleNamespace(), pk, False, n_sm=148)
    assert top148["peak"] == pytest.approx(top["peak"] * 148 / 152)
    for v in st.values():
        assert v["frac"] == pytest.approx(v["achieved"] / v["peak"])
    assert st["project"]["achieved"] == pytest.approx(
        (50_000_000 * 34 + 7_800_000 * 32) / 1e-3 / 1e9)
    assert st["splat"]["achieved"] == pytest.approx(3_770_000_000 * 12 / 6e-3 / 1e12)
    assert st["project"]["peak"] == 6800.0
    # additive frames have no depth sort stage in the roofline
    _, st_add = bench.roofline(dict(stages, sort_ms=0.0), 1_000_000, 900_000, 5_000_000,
                               2500, 60_000_000, SimpleNamespace(), pk, True, 152)
    assert "sort" not in st_add and st_add["splat"]["ops_per_fragment"] == 7
