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


def test_warmnet_roofline_arithmetic():
    """The warm-start network's algorithmic bytes and FLOPs at 960x540x64, as
    the warmnet bench line divides them by the measured time: x read as FP32
    and written as BF16, each layer's BF16 input read and output written once
    (the last layer's output FP32), the FP32 residual read once; 2 FLOPs per
    multiply-add over 9 taps of every layer's channel pairs."""
    import bench
    pix = 960 * 540
    nbytes, flops = bench.warmnet_bytes_flops(960, 540, 64)
    want_bytes = (pix * 64 * (4 + 2)                          # x: FP32 read, BF16 write
                  + pix * (64 + 32) * 2                        # layer 1: 64 in, 32 out (BF16)
                  + 2 * pix * (32 + 32) * 2                    # layers 2, 3
                  + pix * 32 * 2 + pix * 64 * 4                # layer 4: BF16 in, FP32 out
                  + pix * 64 * 4)                              # residual x, FP32
    assert nbytes == want_bytes
    assert round(nbytes / 1e6, 1) == 729.9
    assert flops == 2 * pix * 9 * (64 * 32 + 32 * 32 + 32 * 32 + 32 * 64)
    assert round(flops / 1e9, 2) == 57.33
