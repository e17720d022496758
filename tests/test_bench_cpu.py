"""bench.py's reporting on CPU: both arms print the same `config` dict for a
workload, and the parity field recognises the reference's own result (and
only it) for the plain loopy-BP workload."""
import io
import json
import os
import sys
from contextlib import redirect_stdout

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_reference_arm_prints_the_shared_config():
    import bench
    cfg = dict(bench.WORKLOADS["plain"], W=40, H=30, name="lbp_40x30_L16_50it")

    class Args:
        steps, warmup, workload = 1, 0, "plain"

    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(Args, cfg)
    line = json.loads(buf.getvalue().strip().splitlines()[-1])
    assert line["config"] == bench.bench_config("plain", cfg)
    assert line["config"] == json.loads(json.dumps(bench.bench_config("plain", cfg)))


def test_parity_field_against_the_reference_result(orc):
    import bench
    from gridinfcuda_gb300 import synth
    P = synth.workload_plain_bp()
    lab, _ = orc.hbp(P.D, P.V, P.model, 1, 50)
    e = orc.energy(P.D, P.V, lab)
    par = bench.parity_vs_golden("plain", lab, e)
    assert par["ok"] and par["labels_sha_equal"] and par["energy_rel_diff"] == 0.0
    bad = lab.copy()
    bad[5, 5] = (bad[5, 5] + 1) % 16
    assert not bench.parity_vs_golden("plain", bad, orc.energy(P.D, P.V, bad))["ok"]
    assert not bench.parity_vs_golden("plain", lab, e * (1 + 1e-9))["ok"]
    assert isinstance(np.float64(par["energy"]), np.float64)
