"""The multi-process path of bench.py on CPU (gloo, world size 2): the timing
reduction over ranks and the reference arm under torchrun.  A single graph's
decomposition does not shard (replicas only), so these helpers are the whole
multi-rank logic: every rank times its own replica, rank 0 reports
ranks x E / max step time."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, port, out_dir):
    os.environ.update({"WORLD_SIZE": "2", "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    ws, r, local = bench.dist_env()
    dist = bench.dist_init(ws, "gloo")
    # each replica reports its own step time; the job's time is the slowest
    t = bench.max_over_ranks(10.0 + 5.0 * r, ws, "cpu")
    bench.barrier(ws)
    with open(os.path.join(out_dir, "rank%d.json" % r), "w") as f:
        json.dump({"ws": ws, "rank": r, "local": local, "max_t": t}, f)
    dist.destroy_process_group()


def test_max_over_ranks_and_barrier_gloo(tmp_path):
    mp.spawn(_rank_main, args=(_free_port(), str(tmp_path)), nprocs=2, join=True)
    got = [json.load(open(tmp_path / ("rank%d.json" % r))) for r in range(2)]
    assert [g["rank"] for g in got] == [0, 1]
    assert all(g["ws"] == 2 for g in got)
    assert all(g["max_t"] == 15.0 for g in got)


def test_reference_arm_under_torchrun_prints_one_line():
    """`--impl reference` launched like the GPU arm with 2 ranks: rank 0 alone
    runs the CPU reference and prints one JSON line; rank 1 exits 0."""
    pytest.importorskip("numpy")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-scale", "9"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "edges/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0
