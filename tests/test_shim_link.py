"""The C++ drop-in (splotch_gb300/shim/host_rendering_gb300.cc) compiles
against the reference's own headers and links in place of splotch_host.o.

Runs only where the reference sources are present (they are not shipped):
builds oracle/_ref, compiles the shim and a small caller, links them with the
reference's support objects minus splotch_host.cc.o and with libsplgpu.so,
and runs the program.  Without a GPU the frame fails cleanly with a
PlanckError (exit 3); with one it renders (exit 0)."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
from oracle.oracle import ref_dir

REF = ref_dir()


@pytest.mark.skipif(not (REF / "splotch" / "splotch_host.h").exists(),
                    reason="reference sources not present")
def test_shim_links_in_place_of_splotch_host(built, tmp_path):
    from oracle import oracle

    assert oracle.build_ref()
    # splotch_host.o goes; so does new_renderer.o, whose only caller is the
    # reference host_rendering (splotch_host.cc:720)
    objs = sorted(p for p in (ROOT / "oracle" / "_ref" / "obj_libsplotch_ref").glob("*.o")
                  if p.name not in ("splotch_host.cc.o", "new_renderer.cc.o", "ref_harness.o",
                                    "scenemaker.cc.o", "ref_stubs.o"))
    exe = tmp_path / "link_check"
    inc = ["-I", str(REF), "-I", str(REF / "cxxsupport"), "-I", str(ROOT / "include")]
    cmd = (["g++", "-O2", "-std=c++11", "-fopenmp", "-w", *inc,
            str(ROOT / "splotch_gb300" / "shim" / "host_rendering_gb300.cc"),
            str(ROOT / "tests" / "shim" / "link_check.cc"), *map(str, objs),
            "-L", str(ROOT / "splotch_gb300"), "-lsplgpu",
            f"-Wl,-rpath,{ROOT / 'splotch_gb300'}", "-o", str(exe)])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    for args in ([], ["rays"]):  # the splat path, then new_renderer=true
        run = subprocess.run([str(exe), *args], capture_output=True, text=True, timeout=120)
        assert run.returncode in (0, 3), run.stdout + run.stderr
        if run.returncode == 3:
            assert "GB300 renderer" in run.stdout
        else:
            assert "rendered" in run.stdout
