"""The C++ drop-in API (include/ginf/*.h) on the GPU: a program written the
way the reference example is written, compared with the oracle."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from gridinfcuda_gb300 import synth

pytestmark = pytest.mark.gpu


def test_cpp_program_matches_oracle(ginf, orc, built_lib, tmp_path):
    exe = tmp_path / "dropin"
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "dropin_stereo.cc"), "-o", str(exe), built_lib,
                        "-Wl,-rpath," + os.path.dirname(built_lib)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    W, H, L = 120, 90, 16
    pair = synth.stereo_pair(W, H, L, 8, 2.0, seed=17)
    D = np.minimum(np.abs(np.rint(pair.left)[None].astype(np.int32) -
                          np.stack([np.rint(pair.right[:, np.maximum(np.arange(W) - k, 0)]).astype(np.int32)
                                    for k in range(L)])), 20).astype(np.int32)
    inp, out = tmp_path / "in.raw", tmp_path / "out.raw"
    with open(inp, "wb") as f:
        np.array([W, H, L], np.int32).tofile(f)
        D.tofile(f)
    r = subprocess.run([str(exe), str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    res = np.fromfile(out, np.int32)
    n = W * H
    bp, hbp, icm, energy = res[:n].reshape(H, W), res[n:2 * n].reshape(H, W), res[2 * n:3 * n].reshape(H, W), \
        res[3 * n]
    f = res[3 * n + 1:]
    fbp, fhbp, ficma, ficmg = (f[i * n:(i + 1) * n].reshape(H, W) for i in range(4))
    fenergy = f[4 * n:4 * n + 1].view(np.float32)[0]
    ab = f[4 * n + 1:5 * n + 1].reshape(H, W)
    V = synth.sm_table(L, synth.TRUNC_LINEAR, 10, 20, dtype=np.int32)
    want_bp, _ = orc.hbp(D, V, synth.TRUNC_LINEAR, 1, 30)
    want_hbp, _ = orc.hbp(D, V, synth.TRUNC_LINEAR, 3, 6)
    assert np.array_equal(bp, want_bp)
    assert np.array_equal(hbp, want_hbp)
    assert np.array_equal(icm, orc.icm(D, V, want_bp, 2))
    assert energy == orc.energy(D, V, want_bp, exact_type=True)
    assert np.array_equal(ab, orc.alpha_beta(D, V, want_bp, 1))   # gpuDecodeAlphaBeta<int>
    # The same costs as a Grid<float>: decodeBp, gpuDecodeHbp, decodeIcmAsync, gpuDecodeIcm.
    Df = (np.float32(0.25) * D.astype(np.float32)).astype(np.float32)
    Vf = synth.sm_table(L, synth.TRUNC_LINEAR, 1.5, 3.0)
    want_fbp, _ = orc.hbp(Df, Vf, synth.TRUNC_LINEAR, 1, 12)
    assert np.array_equal(fbp, want_fbp)
    assert np.array_equal(fhbp, orc.hbp(Df, Vf, synth.TRUNC_LINEAR, 2, 5)[0])
    assert np.array_equal(ficma, orc.icm(Df, Vf, want_fbp, 2, asynchronous=True))
    assert np.array_equal(ficmg, orc.icm(Df, Vf, want_fbp, 3))
    assert fenergy == pytest.approx(orc.energy(Df, Vf, want_fbp), rel=1e-6)
