"""Problem builders shared by the tests (inputs regenerated from seeds)."""
import hashlib

import numpy as np

from gridinfcuda_gb300 import synth


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def golden_problem(case):
    dt = np.int32 if case["dtype"] == "i32" else np.float32
    cmax = 20.0 if case["dtype"] == "i32" else 4.0
    return synth.random_problem(case["W"], case["H"], case["L"], case["seed"], model=case["model"],
                                scale=case["scale"], trunc=case["trunc"], dtype=dt, cost_max=cmax)


def workload(name):
    if name.startswith("plain_bp"):
        return synth.workload_plain_bp()
    if name.startswith("hbp_1920"):
        return synth.workload_hbp()
    raise KeyError(name)
