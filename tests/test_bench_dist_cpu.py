"""bench.py's multi-rank plumbing on CPU: two gloo ranks on 127.0.0.1.

With N ranks the bench runs N independent replicas; the only cross-rank
steps are the barriers around the timed region and the reductions of the
timings (max over ranks) and launch counts (sum).  The reference arm is run
by rank 0 alone; the other ranks return without work."""
import io
import json
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    r, local, w = bench.dist_setup(False)
    assert (r, local, w) == (rank, rank, world)
    bench.barrier(w)
    res = {"max": bench.reduce_max(1.5 + rank, w), "sum": bench.reduce_sum(rank + 1, w)}
    # The reference arm on a tiny grid: rank 0 prints one JSON line, others nothing.
    cfg = dict(bench.WORKLOADS["hbp"], W=40, H=30, name="hbp_40x30_L64_5lvl_x10_icm5")

    class Args:
        steps, warmup, workload = 1, 0, "hbp"

    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(Args, cfg)
    res["ref_out"] = buf.getvalue()
    bench.barrier(w)
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(res, f)


def test_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, start_method="spawn")
    r0 = json.load(open(tmp_path / "rank0.json"))
    r1 = json.load(open(tmp_path / "rank1.json"))
    assert r0["max"] == r1["max"] == 2.5
    assert r0["sum"] == r1["sum"] == 3.0
    assert r1["ref_out"] == ""
    line = json.loads(r0["ref_out"].strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == world and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
