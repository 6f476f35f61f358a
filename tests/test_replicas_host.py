"""The bench's N-replica bookkeeping on CPU with gloo, world size 2: the
timing reduction takes the maximum over ranks, and the reference arm runs on
rank 0 only while the other rank exits cleanly."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=2)
    import bench
    ws, r, _ = bench.dist_env()
    bench.barrier(ws)
    q.put((r, bench.reduce_max(1.5 + r, ws)))
    dist.destroy_process_group()


def test_reduce_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29617
    ps = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(60)
    assert got == {0: 2.5, 1: 2.5}


@pytest.mark.timeout(600)
def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, PYTHONPATH=ROOT)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", "--master-port=29623", os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--frames", "8"]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=ROOT, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1  # rank 0 prints, rank 1 exits without work
    d = json.loads(lines[0])
    from oracle import ref_cent
    want = "reference" if ref_cent.available() else "port"
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["kind"] == want
    # the line keeps our arm's metric, unit and workload, and the contract's keys
    import bench
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT and d["higher_is_better"] is True
    assert d["config"]["workload"] == bench.WORKLOAD["name"] and d["steps"] == 1 and d["warmup"] == 0
    assert d["n_gpus"] == 2 and d["scaling"] == "weak" and d["vs_baseline"] is None
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == bench.UNIT and cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e == {"value": d["value"], "unit": bench.UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["ms_per_step"] > 0
