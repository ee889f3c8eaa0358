"""The bench's multi-GPU path is replicas only (the step has no exchange):
one process per GPU, a barrier around the timed steps, the slowest replica's
time by an all-reduce MAX, and the whole-job throughput over it. These tests
run that path as two gloo ranks on the host, and the reference arm under
torchrun with two ranks (rank 0 times the CPU port and prints, rank 1 exits
without work)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    dist, r, ws = bench.dist_setup()
    assert (r, ws) == (rank, world) and dist.get_backend() == "gloo"
    bench.barrier()
    ms = bench.max_over_ranks(dist, times[rank])
    out.put((rank, ms, bench.aggregate_glups(ws, 1.0e8, 10, ms)))
    dist.destroy_process_group()


def test_max_over_ranks_and_aggregate_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    times = [12.5, 17.25]
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, glups in res:
        assert ms == max(times)
        assert glups == pytest.approx(2 * 1.0e8 * 10 / (max(times) * 1e-3) / 1e9)


@pytest.mark.timeout(600)
def test_reference_arm_two_ranks_prints_once(built_lib):
    env = dict(os.environ, OMP_NUM_THREADS=str(max(1, (os.cpu_count() or 2) // 2)))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "1", "--small"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] in ("port", "reference")
    # The line keeps the bench contract: the same keys as this library's arm,
    # a cpu_baseline describing this run and an e2e figure without copies.
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["higher_is_better"] is True and d["unit"] == "GLUPS" and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert {"value", "unit", "cores", "kind", "sample"} <= set(cb) and cb["value"] == d["value"] and cb["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
