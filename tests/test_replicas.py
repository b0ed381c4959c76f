"""Multi-rank path of bench.py: N replicas (one per GPU) reduce only the timed
milliseconds (max) and the processed particle-updates (sum).  Run here as two
gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # uneven replicas: rank r processed 1000 (r + 1) units in 10 + r ms
        ms, units = bench.aggregate_replicas(10.0 + rank, 1000 * (rank + 1), "cpu")
        q.put((rank, ms, units, bench.dist_env()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    for rank, ms, units, env in out:
        assert ms == 11.0 and units == 3000.0
        assert env == (world, rank, rank)


def test_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate_replicas(7.5, 123, "cpu") == (7.5, 123.0)


def test_reference_arm_line():
    """`bench.py --impl reference` on a coarse sample: one JSON line with the
    contract's keys, the CPU sample described, and e2e equal to the value."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--steps", "2",
                          "--warmup", "0", "--ref-steps", "2", "--ref-budget", "20", "--cpu-cellsize", "0.8"],
                         capture_output=True, text=True, timeout=600, cwd=root)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["cpu_baseline"]["cores"] >= 1 and d["cpu_baseline"]["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
