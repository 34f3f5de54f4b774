#!/usr/bin/env python
"""bench.py -- throughput of the Splotch particle-render path on GB300.

Workload (one step = one frame): the plain ordered emission-absorption render,
40M gas + 10M star particles from the seeded halo-mixture generator in a
[0,500]^3 box, 1920x1080 float32 image, camera (250,250,-50) -> (250,250,250),
fov 45, depth sort on (sort_type 1), gray_absorption 0.2.  Synthetic data: the
reference's demo snapshot is not available.

value : Mparticles/s with the SoA inputs already resident in HBM (CUDA events
        on the render stream around K frames; 1.8 GB of inputs per frame, far
        larger than L2, so no flush is needed).
e2e   : the same metric through the C ABI with HOST buffers: a sequence of
        frames from particle_sim records in pinned host memory, each frame's
        records copied ahead (spl_prefetch) while the frame before it renders;
        every frame's H2D and image D2H lie inside the timed region; the median
        of three sequences.
roofline: the dominant kernel of the frame, algorithmic work / its CUDA-event
        time, against MEASURED_PEAKS.json.
cpu_baseline: the CPU restatement of the reference (bit-exact with it) timed
        on this host's cores on the whole frame; the same leg, as the checker,
        measures the timed frame's image against the FP64 oracle
        (image_rel_linf) and the reference's own FP32 arithmetic beside it, and
        times the reference's legacy GPU kernels (cuda/, additive frames) as
        the GPU floor (legacy_gpu_floor).
drop_in_default: the frame through host_rendering() with the drop-in's
        defaults (front-to-back compositing, every particle projected,
        colourised and sorted back into the caller's array), from pageable
        host memory, as a Splotch caller would make the call; and the same
        with back-to-front compositing.
large : the large render (400M particles, 4096^2, forward and
        forward+backward), batched / fwd_bwd / rays: the other workloads.

--impl reference runs that CPU implementation alone (rank 0) on the same
frame and prints its own line.  Multi-GPU (torchrun): replicas -- every rank
renders its own seeded frame, value = all ranks' particles / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mparticles/s & frames/s (plain, batched, fwd+bwd) on 1 GB300 at ≤1e-4 rel err"

# The splat's DRAM traffic and issue / shared-memory figures come from the
# committed one-kernel ncu capture (the bench itself runs no profiler); the
# traffic is scaled to the timed frame by its reference fragment count.
SPLAT_CAPTURE = {
    "source": "profiles/k_splat_ftb_10M.md",
    "fragments": 7.53e8,          # reference fragments of the captured launch
    "dram_bytes": 85.4e6,         # dram__bytes (read + write) of the launch
    "issue_frac": 0.70,           # issue slots busy per SMSP while active
    "smem_wavefront_frac": 0.274,  # L1 data-pipe (shared) wavefronts, of peak
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="absorption", choices=["absorption", "additive"])
    ap.add_argument("--tile", type=int, default=16)
    ap.add_argument("--order", default="ftb", choices=["ftb", "btf"])
    ap.add_argument("--e2e-steps", type=int, default=30,
                    help="frames in the host-memory sequence (the first frame's copy and "
                         "the last frame's render are not hidden behind another frame)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fwd-bwd", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batch-scale", type=float, default=1.0,
                    help="particle-count multiplier of the batched workload")
    ap.add_argument("--batch-steps", type=int, default=3)
    ap.add_argument("--no-rays", action="store_true")
    ap.add_argument("--no-large", action="store_true")
    ap.add_argument("--no-drop-in", action="store_true")
    ap.add_argument("--drop-in-steps", type=int, default=3)
    ap.add_argument("--rays-particles", type=int, default=1_000_000)
    ap.add_argument("--only", default="all",
                    choices=["all", "fwd_bwd", "batched", "large", "rays"],
                    help="run one section alone (profiling)")
    ap.add_argument("--large-scale", type=float, default=1.0)
    ap.add_argument("--large-steps", type=int, default=2)
    ap.add_argument("--fwd-bwd-particles", type=int, default=4_000_000)
    ap.add_argument("--split-tiles", action="store_true",
                    help="cut heavy tiles into list segments in the main workload's frames")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="particle-count multiplier (profiling runs use a smaller frame)")
    return ap.parse_args()


def make_workload(args, seed_offset: int = 0):
    from splotch_gb300 import synth

    s = args.scale
    if args.workload == "additive":
        n = int(1_000_000 * s)
        w = synth.plain_additive(n=n, seed=0 + seed_offset, tile=args.tile)
        cfg = {"workload": f"plain additive: {n} particles, 800x800, halo mixture [0,100]^3, "
                           "fov 30", "particles": n, "image": [800, 800]}
    else:
        ng, ns = int(40_000_000 * s), int(10_000_000 * s)
        w = synth.plain_absorption(n_gas=ng, n_star=ns, seed=1 + seed_offset, tile=args.tile,
                                   order=args.order)
        cfg = {"workload": f"plain ordered emission-absorption: {ng} gas + {ns} stars, "
                           "1920x1080, halo mixture [0,500]^3, fov 45, depth sort",
               "particles": ng + ns, "image": [1920, 1080]}
    cfg.update({"tile_size": args.tile, "absorption_order": args.order,
                "l2": "inputs (36 B/particle) larger than the 129 MB L2; no flush"})
    return w, cfg


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "sm_max_mhz": d.get("sm_max_mhz", 2070.0),
                "source": "measured"}
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.tmp,
                stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.tmp.flush()
        rows = [r.split(",") for r in Path(self.tmp.name).read_text().splitlines() if r.strip()]
        os.unlink(self.tmp.name)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def host_cpu() -> dict:
    """The host CPU as the reference arm sees it: model, cores, OpenMP binding."""
    model = None
    try:
        r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10)
        for line in r.stdout.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.TimeoutExpired):
        pass
    return {"cpu_model": model, "logical_cpus": os.cpu_count(),
            "omp_proc_bind": os.environ.get("OMP_PROC_BIND"),
            "omp_num_threads": os.environ.get("OMP_NUM_THREADS")}


def _oracle_port():
    """The oracle's restatement of host_rendering, loaded with every host core
    and threads bound close (set before its OpenMP runtime starts)."""
    os.environ.setdefault("OMP_PROC_BIND", "close")
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    from oracle.oracle import Port

    return Port()


def _time_host_rendering(port, w, steps: int, warmup: int) -> list:
    """Wall time of the restatement's host_rendering on the whole frame, at
    the reference's own default tile size (tile_size_cpu=50)."""
    prm = dict(w.params.params)
    prm["tile_size_cpu"] = "50"
    ts = []
    for i in range(warmup + steps):
        p = w.particles.copy()
        t0 = time.perf_counter()
        port.host_rendering(prm, w.rc, p)
        if i >= warmup:
            ts.append(time.perf_counter() - t0)
    return ts


def cpu_baseline(w, pic_gpu: np.ndarray, steps: int = 2, warmup: int = 1) -> dict:
    """The oracle's restatement of host_rendering (bit-exact with the
    reference) timed on this host's cores on the whole frame; then, as the
    checker, the FP64 oracle image of the same frame at the GPU's tile size,
    against which the GPU image and the reference's FP32 arithmetic (the
    scalar render_new branch an AArch64 host compiles) are measured."""
    from oracle.oracle import rel_linf

    port = _oracle_port()
    ts = _time_host_rendering(port, w, steps, warmup)
    t = statistics.median(ts)
    out = {"value": len(w.particles) / t / 1e6, "unit": "Mparticles/s", "cores": port.threads,
           "kind": "port", "seconds_per_frame": t, **host_cpu(),
           "sample": f"the whole frame ({len(w.particles)} particles), same image and camera, "
                     f"reference default tile_size_cpu=50; median of {steps} after {warmup} "
                     "warm-up"}
    # the checker: FP64 image of the timed frame (coverage and order as the GPU's)
    prm = dict(w.params.params)
    T = int(prm["tile_size_cpu"])
    xres, yres = int(prm["xres"]), int(prm["yres"])
    a_eq_e = prm.get("a_eq_e", "T") == "T"
    gray = float(prm.get("gray_absorption", 0.2))
    p = w.particles.copy()
    port.project_colorize(prm, w.rc, p)
    order = None if a_eq_e else port.sort_perm(p, int(prm.get("sort_type", 1)))
    pic64, _ = port.render_fp64(p, order, xres, yres, T, a_eq_e, gray)
    pic32 = port.render_fp32(p, order, xres, yres, T, a_eq_e, gray, simd=False)[0]
    out["image_check"] = {
        "image_rel_linf": rel_linf(pic_gpu, pic64),
        "reference_fp32_rel_linf": rel_linf(pic32, pic64),
        "tolerance": 1e-4, "floor": "1e-6 x max|pixel|",
        "against": f"FP64 oracle at the GPU tile size {T}, same coverage and order"}
    return out


def legacy_gpu_floor(args, local: int) -> dict:
    """The reference's legacy GPU renderer (cuda/, additive only), the GPU
    floor: its own kernels built from the reference sources (PTX, by
    oracle/build_ref.sh) under the oracle's driver, on the plain additive frame
    (1M particles, 800x800) and on the batched workload's additive frames
    (4 sets x 12 poses), inputs pre-clamped to [0, 1] as its normalisation
    requires.  Each frame as cuda_rendering makes it: particle_sim records from
    pageable host memory, three kernels, the image back; host wall time.  The
    plain path renders the same frames through the C ABI from the same
    pageable host records, timed the same way."""
    import torch

    import splotch_gb300 as sg
    from oracle.oracle import LEGACY_PTX, LegacyGPU
    from splotch_gb300 import synth

    if not LEGACY_PTX.exists():
        return {"unavailable": "the legacy kernels' PTX was not built (reference sources "
                               "absent where build() ran)"}
    port = _oracle_port()
    leg = LegacyGPU()
    r = sg.Renderer(local)

    def both(p, params, rc, reps: int) -> tuple:
        prm = dict(params.params)
        p = p.copy()
        p["I"] = np.minimum(p["I"], np.float32(1.0))
        fr = leg.frame(port, prm, rc)
        keep: list = []
        desc = sg.frame_desc(sg.ParamFile(dict(prm)), rc, keep)
        pic = np.zeros((desc.xres, desc.yres, 3), np.float32)
        leg.render(port, prm, rc, p, frame=fr)
        r.render_aos(desc, p, pic)
        lt, gt, lst = [], [], None
        for _ in range(reps):
            t0 = time.perf_counter()
            _, lst = leg.render(port, prm, rc, p, frame=fr)
            lt.append(time.perf_counter() - t0)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r.render_aos(desc, p, pic)
            gt.append(time.perf_counter() - t0)
        return statistics.median(lt), statistics.median(gt), lst

    out = {"kind": "reference", "note": "the reference's cuda/ kernels (k_range, k_process, "
           "full-atomics k_render) compiled from its sources; the host driver restates "
           "cuda_rendering for one chunk"}
    w = synth.plain_additive()
    lt, gt, lst = both(w.particles, w.params, w.rc, max(3, args.steps))
    n = len(w.particles)
    out["plain_additive_1M_800"] = {
        "legacy_ms": lt * 1e3, "legacy_mparticles_per_s": n / lt / 1e6,
        "legacy_stages_ms": {k: round(v, 3) for k, v in lst.items()},
        "ours_ms": gt * 1e3, "ours_mparticles_per_s": n / gt / 1e6, "speedup": lt / gt}
    bw = synth.batched(scale=args.batch_scale, tile=16, order=args.order)
    lsum = gsum = 0.0
    nfr = 0
    pf = 0
    for s, params, rc in bw.frames:
        if params.params.get("a_eq_e") != "T":
            continue
        lt, gt, _ = both(bw.sets[s], params, rc, 1)
        lsum += lt
        gsum += gt
        nfr += 1
        pf += len(bw.sets[s])
    r.close()
    out["batched_additive_frames"] = {
        "frames": nfr, "particle_frames": pf, "legacy_ms": lsum * 1e3,
        "legacy_frames_per_s": nfr / lsum, "ours_ms": gsum * 1e3,
        "ours_frames_per_s": nfr / gsum, "speedup": lsum / gsum}
    return out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    w, cfg = make_workload(args)
    port = _oracle_port()
    ts = _time_host_rendering(port, w, args.steps, args.warmup)
    t = sum(ts) / len(ts)
    n = len(w.particles)
    v = n / t / 1e6
    cb = {"value": v, "unit": "Mparticles/s", "cores": port.threads, "kind": "port",
          **host_cpu(),
          "sample": f"the whole frame ({n} particles) every step, at the reference's default "
                    "tile_size_cpu=50; the reference's own build cannot run on this host (its "
                    "sources do not travel and x86 binaries are removed), so its bit-exact C "
                    "restatement (oracle/spl_oracle.c) runs instead"}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Mparticles/s",
            "n_gpus": 0, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "frames_per_s": 1.0 / t, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "Mparticles/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def roofline(stage_ms: dict, n: int, n_act: int, n_entries: int, n_tiles: int, frags: int,
             args, pk: dict, a_eq_e: bool, n_sm: int) -> tuple[dict, dict]:
    """Per-stage rooflines; the top-level one is the dominant stage's.
    Algorithmic bytes: project reads every particle's SoA fields (x,y,z,r,I,
    e.r,e.g,e.b: 32 B + type 2 B) and writes the projected record of each
    active particle (x,y,r,z,rgb,I: 32 B); the depth sort reads and writes one
    (key, index) pair per active particle (16 B); binning reads x,y,r of each
    active particle (12 B), writes one 4-byte entry per (particle, tile) and
    4 B per tile."""
    hbm = pk["hbm_gbs"]
    # nominal FP32 rate: 128 FMA lanes per SM per clock at the maximum SM clock
    fp32_peak = 2 * 128 * n_sm * pk["sm_max_mhz"] * 1e6 / 1e12  # TFLOP/s
    st = {}
    proj_bytes = n * 34 + n_act * 32
    st["project"] = {"bound": "hbm", "unit": "GB/s", "algorithmic_bytes": proj_bytes,
                     "achieved": proj_bytes / (stage_ms["project_ms"] * 1e-3) / 1e9}
    if not a_eq_e and stage_ms["sort_ms"] > 0:
        sort_bytes = n_act * 16
        st["sort"] = {"bound": "hbm", "unit": "GB/s", "algorithmic_bytes": sort_bytes,
                      "achieved": sort_bytes / (stage_ms["sort_ms"] * 1e-3) / 1e9}
    bin_bytes = n_act * 12 + n_entries * 4 + n_tiles * 4
    st["bin"] = {"bound": "hbm", "unit": "GB/s", "algorithmic_bytes": bin_bytes,
                 "achieved": bin_bytes / (stage_ms["bin_ms"] * 1e-3) / 1e9}
    # splat: reference fragments x useful FP32 work per fragment
    ops = 7 if a_eq_e else 12
    flops = frags * ops
    st["splat"] = {"bound": "fp32", "unit": "TFLOP/s", "algorithmic_flops": flops,
                   "fragments": frags, "ops_per_fragment": ops,
                   "achieved": flops / (stage_ms["splat_ms"] * 1e-3) / 1e12}
    for k, v in st.items():
        v["ms"] = stage_ms[k + "_ms"]
        v["peak"] = hbm if v["bound"] == "hbm" else fp32_peak
        v["frac"] = v["achieved"] / v["peak"]
    kernels = {"project": "k_project_flags_soa4+scan_popc+k_project_dense",
               "sort": "k_os_hist+k_os_prefix+k_rs_downsweep",
               "bin": "k_gather_u32+scan+k_emit_narrow+k_emit_wide+tile sort+k_tile_ranges",
               "splat": "k_splat"}
    for k, v in st.items():
        v["kernels"] = kernels[k]
    dom = max(st, key=lambda k: st[k]["ms"])
    d = st[dom]
    top = {"kernel": kernels[dom], "stage": dom, "bound": d["bound"], "achieved": d["achieved"],
           "peak": d["peak"], "unit": d["unit"], "frac": d["frac"], "traffic": None,
           "peak_source": (f"{pk['source']} HBM copy bandwidth" if d["bound"] == "hbm"
                           else f"nominal FP32 rate, 128 lanes x {n_sm} SMs x "
                                f"{pk['sm_max_mhz']:.0f} MHz (no FP32 peak in "
                                "MEASURED_PEAKS.json)"),
           "sm_count": n_sm}
    if dom == "splat":
        c = SPLAT_CAPTURE
        top["traffic"] = c["dram_bytes"] * frags / c["fragments"]
        top["traffic_note"] = (f"DRAM read+write bytes per launch from {c['source']}, scaled "
                               "to this frame by its reference fragment count")
        top["issue_frac"] = c["issue_frac"]
        top["smem_wavefront_frac"] = c["smem_wavefront_frac"]
        top["capture"] = c["source"]
    return top, st


def fwd_bwd(args, local: int) -> dict:
    """Forward vs forward+backward on the differentiable-render workload: 4M
    particles of the halo mixture, 1024x1024, additive and ordered absorption.
    One step = render + dL/dpic of L = sum((pic - target)^2) + backward with
    respect to I, colour, position, hsml and the camera position; inputs and
    outputs resident in HBM, CUDA events on the render stream."""
    import torch

    import splotch_gb300 as sg
    from splotch_gb300 import _abi, synth

    dev = f"cuda:{local}"
    out = {}
    n = int(args.fwd_bwd_particles * min(args.scale, 1.0))
    for mode in ("additive", "absorption"):
        w = synth.differentiable(n=n, mode=mode, xres=1024, tile=args.tile, order=args.order)
        r = sg.Renderer(local)
        stream = torch.cuda.Stream(device=dev)
        r.set_stream(stream.cuda_stream)
        keep: list = []
        desc = sg.frame_desc(w.params, w.rc, keep)
        soa_t = {k: torch.from_numpy(v).to(dev) for k, v in
                 synth.soa_from_aos(w.notes["target"]).items()}
        soa = {k: torch.from_numpy(v).to(dev) for k, v in synth.soa_from_aos(w.particles).items()}
        target = torch.zeros((desc.xres, desc.yres, 3), dtype=torch.float32, device=dev)
        pic = torch.zeros_like(target)
        r.render_soa(desc, soa_t, target)
        grads = {f: torch.zeros(n, dtype=torch.float32, device=dev) for f in _abi.GRAD_FIELDS}

        def step(backward: bool):
            r.render_soa(desc, soa, pic)
            if backward:
                with torch.cuda.stream(stream):
                    gpic = 2.0 * (pic - target)
                r.backward(gpic, grads, device=True)

        res = {}
        for name, bw in (("fwd", False), ("fwd_bwd", True)):
            r.set_differentiable(bw)  # the plain forward keeps nothing extra
            for _ in range(args.warmup):
                step(bw)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            fwd_total = bwd_total = 0.0
            e0.record(stream)
            for _ in range(args.steps):
                step(bw)
                s = r.stats()
                fwd_total += s["total_ms"]
                bwd_total += s["bwd_total_ms"] if bw else 0.0
            e1.record(stream)
            torch.cuda.synchronize()
            res[name + "_ms"] = e0.elapsed_time(e1) / args.steps
            res[name + "_render_call_ms"] = fwd_total / args.steps
            if bw:
                res["backward_call_ms"] = bwd_total / args.steps
        st = r.stats()
        res["ratio_fwd_bwd_over_fwd"] = res["fwd_bwd_ms"] / res["fwd_ms"]
        res["fwd_bwd_mparticles_per_s"] = n / (res["fwd_bwd_ms"] * 1e-3) / 1e6
        res["fwd_bwd_frames_per_s"] = 1e3 / res["fwd_bwd_ms"]
        res["bwd_splat_ms"] = st["bwd_splat_ms"]
        res["bwd_project_ms"] = st["bwd_project_ms"]
        res["splat_ms"] = st["splat_ms"]
        res["particles"] = n
        res["active"] = int(st["n_active"])
        out[mode] = res
        r.close()
    return out


def rays(args, local: int) -> dict:
    """The ray-sphere renderer (host_rendering with new_renderer=true,
    splotch/new_renderer.cc:522-641) on the plain additive frame's particles
    (halo mixture in [0,100]^3, fov 30): the 800x800 plane view, the 800x800
    dome (fisheye) view, and the 1920x1080 plane view.  value: SoA inputs
    resident in HBM, CUDA events on the render stream; e2e: particle_sim
    records from pinned host memory and the image back, per frame; cpu: the
    oracle's restatement in the reference's arithmetic (bit-exact with it) on
    all host cores, on the whole frame."""
    import torch

    import splotch_gb300 as sg
    from oracle.oracle import Port
    from splotch_gb300 import synth

    dev = f"cuda:{local}"
    n = int(args.rays_particles * min(args.scale, 1.0))
    port = Port()
    out = {}
    for name, extra in (("plane_800", {}), ("dome_800", {"dome": "T"}),
                        ("plane_1920x1080", {"xres": "1920", "yres": "1080"})):
        w = synth.plain_additive(n=n, seed=0)
        prm = dict(w.params.params, new_renderer="T", **extra)
        pf = sg.ParamFile(dict(prm))
        keep: list = []
        desc = sg.frame_desc(pf, w.rc, keep)
        rd = sg.rays_desc(pf)
        r = sg.Renderer(local)
        stream = torch.cuda.Stream(device=dev)
        r.set_stream(stream.cuda_stream)
        soa = {k: torch.from_numpy(v).to(dev) for k, v in synth.soa_from_aos(w.particles).items()}
        pic = torch.zeros((desc.xres, desc.yres, 3), dtype=torch.float32, device=dev)
        for _ in range(args.warmup):
            r.render_rays(desc, rd, soa, pic, device=True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        stages = {k: 0.0 for k in ("project_ms", "sort_ms", "bin_ms", "splat_ms")}
        e0.record(stream)
        for _ in range(args.steps):
            r.render_rays(desc, rd, soa, pic, device=True)
            st = r.stats()
            for k in stages:
                stages[k] += st[k] / args.steps
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        host_aos = torch.empty(n * 36, dtype=torch.uint8, pin_memory=True)
        host_aos.numpy()[:] = w.particles.view(np.uint8)
        host_pic = torch.empty((desc.xres, desc.yres, 3), dtype=torch.float32, pin_memory=True)
        r.render_rays(desc, rd, host_aos, host_pic)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            r.render_rays(desc, rd, host_aos, host_pic)
        e2e_ms = (time.perf_counter() - t0) / args.steps * 1e3
        ts = []
        for i in range(3):
            t0 = time.perf_counter()
            _, ost = port.render_rays(prm, w.rc, w.particles, exact=False)
            if i:
                ts.append(time.perf_counter() - t0)
        cpu_s = statistics.median(ts)
        out[name] = {"particles": n, "image": [int(desc.xres), int(desc.yres)], "ms": ms,
                     "mparticles_per_s": n / (ms * 1e-3) / 1e6, "frames_per_s": 1e3 / ms,
                     "stages_ms": {"particles": stages["project_ms"],
                                   "level_sort": stages["sort_ms"],
                                   "walk_and_leaf_sort": stages["bin_ms"],
                                   "leaves": stages["splat_ms"]},
                     "e2e_ms": e2e_ms, "e2e_mparticles_per_s": n / (e2e_ms * 1e-3) / 1e6,
                     "spheres": int(st["n_active"]), "leaf_entries": int(st["n_entries"]),
                     "leaf_regions": int(st["n_tiles"]), "levels": ost["levels"],
                     "fragments": ost["fragments"],
                     "fragments_per_s": ost["fragments"] / (ms * 1e-3),
                     "cpu": {"ms": cpu_s * 1e3, "mparticles_per_s": n / cpu_s / 1e6,
                             "cores": port.threads, "kind": "port",
                             "sample": "the whole frame, reference arithmetic"},
                     "speedup_vs_cpu": cpu_s * 1e3 / ms}
        r.close()
    return out


def large(args, local: int) -> dict:
    """Large render, forward+backward (opt-in, --only large): 400M particles x
    large_scale, ordered absorption, per-particle RGB, Pareto hsml, 4096^2.
    One step = render + dL/dpic + backward, all resident in HBM."""
    import torch

    import splotch_gb300 as sg
    from splotch_gb300 import _abi, synth

    dev = f"cuda:{local}"
    n = int(400_000_000 * args.large_scale)
    t0 = time.perf_counter()
    w = synth.large(n=n, tile=args.tile, order=args.order)
    gen_s = time.perf_counter() - t0
    r = sg.Renderer(local)
    stream = torch.cuda.Stream(device=dev)
    r.set_stream(stream.cuda_stream)
    keep: list = []
    desc = sg.frame_desc(w.params, w.rc, keep)
    soa = {}
    for k, v in synth.soa_from_aos(w.particles).items():
        soa[k] = torch.from_numpy(v).to(dev)
    del w
    pic = torch.zeros((desc.xres, desc.yres, 3), dtype=torch.float32, device=dev)
    grads = {f: torch.zeros(n, dtype=torch.float32, device=dev) for f in _abi.GRAD_FIELDS}
    out = {"particles": n, "image": [desc.xres, desc.yres], "generate_s": gen_s}
    for name, bw in (("fwd", False), ("fwd_bwd", True)):
        r.set_differentiable(bw)
        for _ in range(max(1, args.warmup // 3)):
            r.render_soa(desc, soa, pic)
            if bw:
                with torch.cuda.stream(stream):
                    gpic = 2.0 * pic
                r.backward(gpic, grads, device=True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        steps = max(1, args.large_steps)
        e0.record(stream)
        for _ in range(steps):
            r.render_soa(desc, soa, pic)
            if bw:
                with torch.cuda.stream(stream):
                    gpic = 2.0 * pic
                r.backward(gpic, grads, device=True)
        e1.record(stream)
        torch.cuda.synchronize()
        out[name + "_ms"] = e0.elapsed_time(e1) / steps
        st = r.stats()
        out[name + "_stages"] = {k: st[k] for k in ("project_ms", "sort_ms", "bin_ms",
                                                    "splat_ms", "bwd_splat_ms",
                                                    "bwd_project_ms")}
    st = r.stats()
    free_b, total_b = torch.cuda.mem_get_info(dev)
    out.update({"active": int(st["n_active"]), "bin_entries": int(st["n_entries"]),
                "wide_particles": int(st["n_wide"]),
                "ratio_fwd_bwd_over_fwd": out["fwd_bwd_ms"] / out["fwd_ms"],
                "fwd_mparticles_per_s": n / (out["fwd_ms"] * 1e-3) / 1e6,
                "fwd_bwd_mparticles_per_s": n / (out["fwd_bwd_ms"] * 1e-3) / 1e6,
                # torch tensors (inputs, image, gradients) at their peak, and the
                # whole device in use with the renderer's buffers still held
                "torch_memory_peak_gb": torch.cuda.max_memory_allocated(dev) / 1e9,
                "device_memory_in_use_gb": (total_b - free_b) / 1e9})
    r.close()
    return out


def batched(args, local: int) -> dict:
    """Batched rendering vs the plain per-frame path on the same frames: 8
    particle sets (N log-uniform in [1M, 32M] x batch_scale, alternating
    additive / ordered), 12 orbit poses each, resolutions from {512^2, 1024^2,
    1920x1080, 2048^2} -> 96 frames.  Plain: one spl_render call per frame
    (tile 16, default launch configurations); batched: one spl_batch_render
    (captured graph, autotuned).  Inputs and images resident in HBM; CUDA events
    on each path's stream; frames/s = 96 / time of one whole pass."""
    import torch

    import splotch_gb300 as sg
    from splotch_gb300 import _abi, synth

    dev = f"cuda:{local}"
    bw = synth.batched(scale=args.batch_scale, tile=16, order=args.order)
    sets = [{k: torch.from_numpy(v).to(dev) for k, v in synth.soa_from_aos(p).items()}
            for p in bw.sets]
    keep: list = []
    frames = []
    for s, params, rc in bw.frames:
        desc = sg.frame_desc(params, rc, keep)
        frames.append((s, desc, torch.zeros((desc.xres, desc.yres, 3), dtype=torch.float32,
                                            device=dev)))
    torch.cuda.synchronize()
    r = sg.Renderer(local)
    stream = torch.cuda.Stream(device=dev)
    r.set_stream(stream.cuda_stream)
    nf = len(frames)
    pf_total = sum(len(bw.sets[s]) for s, _, _ in frames)
    out = {"frames": nf, "sets": len(bw.sets), "particles": bw.notes["particles"],
           "particle_frames": pf_total,
           "pixels": int(sum(d.xres * d.yres for _, d, _ in frames))}

    def plain_pass():
        for s, desc, pic in frames:
            r.render_soa(desc, sets[s], pic)

    for _ in range(max(1, args.warmup // 2)):
        plain_pass()
    torch.cuda.synchronize()
    reps = max(1, args.batch_steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        plain_pass()
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1) / reps
    # one more (untimed) plain pass: each frame's device stage times, summed
    stage_keys = ("project_ms", "sort_ms", "bin_ms", "splat_ms", "total_ms")
    plain_stages = dict.fromkeys(stage_keys, 0.0)
    for s, desc, pic in frames:
        r.render_soa(desc, sets[s], pic)
        st = r.stats()
        for k in stage_keys:
            plain_stages[k] += float(st[k])
    out["plain_stage_ms_sum"] = {k: round(v, 3) for k, v in plain_stages.items()}
    # the plain path with heavy tiles cut into list segments (an option, off by
    # default), timed the same way
    r.set_split_tiles(True)
    plain_pass()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        plain_pass()
    e1.record(stream)
    torch.cuda.synchronize()
    r.set_split_tiles(_abi.SPL_SPLIT_ADDITIVE)
    out["plain_split_tiles_ms"] = e0.elapsed_time(e1) / reps
    out["plain_split_tiles_frames_per_s"] = nf / (out["plain_split_tiles_ms"] * 1e-3)

    t0 = time.perf_counter()
    b = sg.Batch(r, sets, frames)
    create_s = time.perf_counter() - t0
    for _ in range(max(1, args.warmup // 2)):
        b.render()
    ts = []
    for _ in range(reps):
        t1 = time.perf_counter()
        b.render()
        ts.append(time.perf_counter() - t1)
    info = b.info()
    batch_ms = statistics.median(ts) * 1e3
    b.close()
    # a second batch of the same shape: the autotuner's choice from its cache
    t0 = time.perf_counter()
    b2 = sg.Batch(r, sets, frames)
    create2_s = time.perf_counter() - t0
    info2 = b2.info()
    b2.close()
    out.update({"plain_ms": plain_ms, "plain_frames_per_s": nf / (plain_ms * 1e-3),
                "batched_ms": batch_ms, "batched_device_ms": info["render_ms"],
                "batched_frames_per_s": nf / (batch_ms * 1e-3),
                "batched_mparticle_frames_per_s": pf_total / (batch_ms * 1e-3) / 1e6,
                "speedup_frames_per_s": plain_ms / batch_ms,
                "speedup_vs_plain_split_tiles": out["plain_split_tiles_ms"] / batch_ms,
                "tile_size": info["tile_size"],
                "splat_config_additive": info["splat_config_additive"],
                "splat_config_absorption": info["splat_config_absorption"],
                "graph": info["graph"], "create_s": create_s, "tune_ms": info["tune_ms"],
                "plan_ms": info["plan_ms"],
                "second_create": {"create_s": create2_s, "tune_ms": info2["tune_ms"],
                                  "tune_cached": info2["tune_cached"],
                                  "plan_ms": info2["plan_ms"]},
                "kernel_launches_per_render": info["kernel_launches"],
                "active_records": info["n_active"], "bin_entries": info["n_entries"]})
    r.close()
    return out


def drop_in_default(args, w, local: int) -> dict:
    """The frame through host_rendering() with the drop-in's defaults, the way
    a Splotch caller makes the call (splotch/splotch.cc:261): particle_sim
    records in pageable host memory, the default compositing order, and the
    reference's side effects -- every particle projected, colourised and
    stably depth-sorted back into the caller's array -- plus the image.  Wall
    time per call, copies included; the median of the timed calls.  The
    back-to-front order (gpu_order=btf) is timed the same way beside it."""
    import copy

    import torch

    import splotch_gb300 as sg

    n = len(w.particles)
    r = sg.Renderer(local)

    def calls(prm: dict) -> dict:
        ts, stages = [], None
        for i in range(1 + max(1, args.drop_in_steps)):
            pf = sg.ParamFile(dict(prm))
            rc = copy.copy(w.rc)
            rc.pic = None
            parts = w.particles.copy()  # the caller's vector (mutated in place)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            sg.host_rendering(pf, parts, rc, renderer=r)
            dt = time.perf_counter() - t0
            if i:
                ts.append(dt)
                stages = r.stats()
        t = statistics.median(ts)
        return {"ms": t * 1e3, "mparticles_per_s": n / t / 1e6, "frames_per_s": 1.0 / t,
                "calls_ms": [round(x * 1e3, 2) for x in ts],
                "stages_ms": {k: round(float(stages[k]), 3) for k in
                              ("h2d_ms", "project_ms", "sort_ms", "bin_ms", "splat_ms",
                               "d2h_ms", "total_ms")}}

    prm = dict(w.params.params)
    prm.pop("gpu_order", None)  # the drop-in's default order (front-to-back)
    out = calls(prm)
    out.update({"order": "ftb (default)",
                "writeback": "full (projected, colourised, sorted particle_sim array copied "
                             "back)",
                "input": "pageable host particle_sim records", "h2d_bytes": n * 36,
                "d2h_bytes": n * 36 + int(prm["xres"]) * int(prm["yres"]) * 12})
    out["back_to_front"] = calls(dict(prm, gpu_order="btf"))
    r.close()
    return out


def run_gpu(args):
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    import splotch_gb300 as sg
    from splotch_gb300 import synth

    if args.only != "all":  # one section alone (profiling runs); prints its own line
        torch.cuda.set_device(local)
        res = {"fwd_bwd": fwd_bwd, "batched": batched, "large": large,
               "rays": rays}[args.only](args, local)
        print(json.dumps({"section": args.only, "result": res}), flush=True)
        return 0

    w, cfg = make_workload(args, seed_offset=rank * 1000)
    cfg["parallelism"] = f"replicas x{world}" if world > 1 else "single GPU"
    n = len(w.particles)
    r = sg.Renderer(local)
    if args.split_tiles:
        r.set_split_tiles(True)
        cfg["split_tiles"] = True
    stream = torch.cuda.Stream()
    r.set_stream(stream.cuda_stream)
    keep: list = []
    desc = sg.frame_desc(w.params, w.rc, keep)
    soa = {k: torch.from_numpy(v).to(f"cuda:{local}") for k, v in synth.soa_from_aos(
        w.particles).items()}
    pic = torch.zeros((desc.xres, desc.yres, 3), dtype=torch.float32, device=f"cuda:{local}")

    for _ in range(args.warmup):
        r.render_soa(desc, soa, pic)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stages = {k: 0.0 for k in ("project_ms", "sort_ms", "bin_ms", "splat_ms")}
    launches = 0
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        r.render_soa(desc, soa, pic)
        s = r.stats()
        for k in stages:
            stages[k] += s[k]
        launches += s["kernel_launches"]
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    pic_host = pic.cpu().numpy()  # the timed frame's image, for the checker
    if dist:
        t = torch.tensor([ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    for k in stages:
        stages[k] /= args.steps
    last = r.stats()
    frags = r.fragments()

    # ---- e2e through the C ABI with host buffers --------------------------------
    host_aos = torch.empty(n * 36, dtype=torch.uint8, pin_memory=True)
    host_aos.numpy()[:] = w.particles.view(np.uint8)
    host_pic = torch.empty((desc.xres, desc.yres, 3), dtype=torch.float32, pin_memory=True)
    r.set_stream(stream.cuda_stream)

    # A sequence of frames from host memory, each frame's records copied ahead
    # (spl_prefetch) while the frame before it renders: every step's 1.8 GB
    # host->device copy and image read-back lie inside the timed region.
    def frames_from_host(steps: int) -> float:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r.prefetch_aos(host_aos)
        for k in range(steps):
            if k + 1 < steps:
                r.prefetch_aos(host_aos)
            r.render_aos(desc, host_aos, host_pic)
        return (time.perf_counter() - t0) / steps

    frames_from_host(3)  # warm-up: the AoS path and the three copy-ahead slots
    # the median of three sequences: wall-clock time over a host link that other
    # GPUs of the machine may share
    e2e_runs = [frames_from_host(args.e2e_steps) for _ in range(3)]
    e2e_s = statistics.median(e2e_runs)
    if dist:
        t = torch.tensor([e2e_s], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    pal_bytes = sum(int(desc.pal_n[t]) * 20 for t in range(desc.ptypes))
    e2e = {"value": world * n / e2e_s / 1e6, "unit": "Mparticles/s",
           "h2d_bytes_per_step": n * 36 + pal_bytes,
           "d2h_bytes_per_step": desc.xres * desc.yres * 12 + 12,
           "ms_per_step": e2e_s * 1e3,
           "sequences_ms_per_step": [round(t * 1e3, 3) for t in e2e_runs]}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    pk = peaks()
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count
    top, st = roofline(stages, n, int(last["n_active"]), int(last["n_entries"]),
                       int(last["n_tiles"]), frags, args, pk, bool(desc.a_eq_e), n_sm)
    r.close()
    del soa, host_aos, host_pic
    di = None if args.no_drop_in else drop_in_default(args, w, local)
    cb = None
    if world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(w, pic_host)
        cb["legacy_gpu_floor"] = legacy_gpu_floor(args, local)
    del w
    fb = None if args.no_fwd_bwd else fwd_bwd(args, local)
    bt = None if args.no_batched else batched(args, local)
    ry = None if args.no_rays else rays(args, local)
    lg = None if args.no_large else large(args, local)
    line = {"metric": METRIC, "value": world * n / (ms * 1e-3) / 1e6, "unit": "Mparticles/s",
            "frames_per_s": world * 1e3 / ms, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded halo mixture; no snapshot available)", "config": cfg,
            "e2e": e2e, "gpu_launches": launches, "clocks": clk, "roofline": top,
            "stages": st, "fragments": frags, "bin_entries": int(last["n_entries"]),
            "image_check": cb.pop("image_check") if cb else None,
            "cpu_baseline": cb, "drop_in_default": di, "fwd_bwd": fb, "batched": bt,
            "rays": ry, "large": lg}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
