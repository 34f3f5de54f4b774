"""Multi-rank logic on CPU with gloo, world size 2.

* Additive frames shard by particles: the images of two contiguous particle
  shares, summed by the allreduce, equal the single-rank image (the oracle
  renders each share on the CPU, so no GPU is involved).
* Batched frames shard by frame and gather on rank 0.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import torch.distributed as dist

    from oracle.oracle import Port
    from splotch_gb300 import dist as sd
    from splotch_gb300 import synth

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    port_ = Port(threads=1)
    w = synth.plain_additive(n=6000, xres=64, yres=48, tile=16)
    prm = dict(w.params.params)
    p = w.particles.copy()
    port_.project_colorize(prm, w.rc, p)
    lo, hi = sd.share(len(p), rank, world)
    part, _ = port_.render_fp64(np.ascontiguousarray(p[lo:hi]), None, 64, 48, 16, True, 0.2)
    pic = torch.from_numpy(part.copy())
    sd.composite_additive(pic)
    # batched frames: every rank renders its own frames, rank 0 collects them
    frames = {}
    for f in sd.shard_frames(5, rank, world):
        frames[f] = np.full((4, 3, 3), float(f), dtype=np.float32)
    got = sd.gather_frames(frames, 5, rank, world, (4, 3, 3))
    if rank == 0:
        full, _ = port_.render_fp64(p, None, 64, 48, 16, True, 0.2)
        np.save(os.path.join(out_dir, "sharded.npy"), pic.numpy())
        np.save(os.path.join(out_dir, "full.npy"), full)
        np.save(os.path.join(out_dir, "frames.npy"), np.stack(got))
    dist.barrier()
    dist.destroy_process_group()


def test_share_matches_calc_share_general():
    from splotch_gb300 import dist as sd

    for n in (0, 1, 7, 100, 101):
        for world in (1, 2, 3, 8):
            spans = [sd.share(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [hi - lo for lo, hi in spans]
            assert max(sizes) - min(sizes) <= 1


def test_two_rank_gloo(tmp_path):
    import torch.multiprocessing as mp

    mp.start_processes(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    sharded = np.load(tmp_path / "sharded.npy")
    full = np.load(tmp_path / "full.npy")
    np.testing.assert_allclose(sharded, full, rtol=1e-12, atol=1e-12)
    frames = np.load(tmp_path / "frames.npy")
    assert [int(f[0, 0, 0]) for f in frames] == [0, 1, 2, 3, 4]
