"""The N>1 path of bench.py on CPU: ranks are independent replicas joined by a
gloo process group used only for the barrier and the max of the per-rank
times; under torchrun the reference arm runs on rank 0 alone."""
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

import pytest

from helpers import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, times, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    rep = bench.Replicas(ws)
    rep.barrier()
    t = rep.tmax(times[rank])
    out.put((rank, t, bench.whole_job_rate(ws, 1000, 10, t)))
    rep.close()


def test_replicas_report_the_slowest_rank_and_the_whole_job():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    ws, port, times = 2, _free_port(), [1.5, 2.5]
    procs = [ctx.Process(target=_rank_main, args=(r, ws, port, times, out)) for r in range(ws)]
    for p in procs:
        p.start()
    res = [out.get(timeout=120) for _ in range(ws)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, t, v in res:
        assert t == 2.5
        assert v == pytest.approx(2 * 1000 * 3 * 10 / 2.5 / 1e9)


def test_reference_arm_prints_one_line_from_rank_zero():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node",
           "2", "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--p", "1", "--ne", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
