"""Alpha-beta swap on the GPU (ginf_decode_alpha_beta, through the C ABI)
against the reference's own results (golden fixtures) and the CPU oracle,
bit for bit: push-relabel in the reference's raster order as anti-diagonal
wavefronts, the state carried across label pairs, the sink-side labelling."""
import numpy as np
import pytest

from gridinfcuda_gb300 import synth
from helpers import golden_problem

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_golden_alpha_beta_cases_bit_exact(ginf, golden):
    meta, arr = golden
    cases = [(n, c) for n, c in meta["cases"].items() if c["kind"] == "alpha_beta"]
    assert len(cases) >= 5
    for name, case in cases:
        P = golden_problem(case)
        init = arr[name + "/init"].astype(np.int32)
        want = arr[name + "/labels"]
        got = ginf.decode_alpha_beta(P.D, P.V, case["model"], init, case["iters"])
        assert np.array_equal(got, want), name
        got_d = ginf.decode_alpha_beta(_dev(P.D), _dev(P.V), case["model"], _dev(init), case["iters"])
        assert np.array_equal(got_d.cpu().numpy(), want), name
        assert ginf.energy(P.D, P.V, case["model"], got) == case["energy_ref_type"], name


@pytest.mark.parametrize("W,H,L,model,scale,trunc,iters", [
    (37, 29, 2, synth.POTTS, 2, 0, 3), (50, 33, 7, synth.TRUNC_LINEAR, 2, 7, 2), (3, 41, 4, synth.TRUNC_LINEAR, 1, 3, 2),
    (61, 3, 5, synth.TRUNC_QUAD, 1, 8, 2), (2, 2, 3, synth.POTTS, 1, 0, 2), (26, 21, 6, synth.EXPLICIT, 0, 0, 1),
    (45, 38, 5, synth.TRUNC_LINEAR, 3, 9, 0)])
def test_alpha_beta_vs_oracle(ginf, orc, W, H, L, model, scale, trunc, iters):
    P = synth.random_problem(W, H, L, 3 * W + H, model=model, scale=scale, trunc=trunc, dtype=np.int32, cost_max=20)
    init = synth.Rng(W * H, 9).integers(0, L - 1, W * H).reshape(H, W).astype(np.int32)
    want = orc.alpha_beta(P.D, P.V, init, iters)
    got = ginf.decode_alpha_beta(P.D, P.V, model, init, iters)
    assert np.array_equal(got, want)


def test_alpha_beta_stereo_grid_vs_oracle(ginf, orc):
    """A 128x96 stereo grid with 16 labels, from the all-zero labelling:
    thousands of labels move, every one as the reference moves it."""
    W, H, L = 128, 96, 16
    P = synth.stereo_problem(W, H, L, seed=3, n_regions=6, sigma=2.0, planar=False, coef=1.0, cap=20.0,
                             model=synth.TRUNC_LINEAR, scale=10, trunc=20)
    D = np.round(P.D).astype(np.int32)
    V = synth.sm_table(L, synth.TRUNC_LINEAR, 10, 20, dtype=np.int32)
    init = np.zeros((H, W), np.int32)
    want = orc.alpha_beta(D, V, init, 1)
    got, st = ginf.decode_alpha_beta(_dev(D), _dev(V), synth.TRUNC_LINEAR, _dev(init), 1, want_stats=True)
    got = got.cpu().numpy()
    assert (want != init).sum() > 5000
    assert np.array_equal(got, want)
    assert st["kernel_launches"] == 1


def test_alpha_beta_rejects_float_grids(ginf):
    P = synth.random_problem(10, 8, 4, 1)
    with pytest.raises(ginf.GinfError) as e:
        ginf.decode_alpha_beta(P.D, P.V, P.model, np.zeros((8, 10), np.int32), 1)
    assert e.value.status == ginf.ERR_UNSUPPORTED
