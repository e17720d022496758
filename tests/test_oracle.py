"""The CPU oracle against the reference's own compiled code and the golden
fixtures that code produced (CPU only)."""
import numpy as np
import pytest

from gridinfcuda_gb300 import synth
from helpers import golden_problem, sha, workload


def _need_ref(orc):
    if orc.ref() is None:
        pytest.skip("reference checkout not present: the golden fixtures stand in for it")


@pytest.mark.parametrize("model,scale,d", [(synth.POTTS, 0.7, 0.0), (synth.TRUNC_LINEAR, 1.0, 1.7),
                                           (synth.TRUNC_QUAD, 1.0, 25.0), (synth.TRUNC_LINEAR, 2.5, 3.0)])
def test_tables_match_reference(orc, model, scale, d):
    _need_ref(orc)
    for L in (2, 3, 16, 17, 64, 128):
        mine = synth.sm_table(L, model, scale, d)
        ref = orc.ref_table(L, model, scale, d)
        assert np.array_equal(mine.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("W,H,L,seed,model", [(17, 13, 16, 100, 2), (9, 7, 3, 101, 2), (31, 23, 17, 102, 1),
                                               (12, 10, 8, 103, 3), (11, 9, 5, 104, 0), (2, 6, 4, 105, 2)])
def test_oracle_vs_reference(orc, W, H, L, seed, model):
    _need_ref(orc)
    P = synth.random_problem(W, H, L, seed, model=model, scale=0.8 if model == 1 else 1.0,
                             trunc=4.0 if model == 3 else 1.7)
    init = np.full((H, W), 5 % L, np.int32)
    for levels, iters in [(1, 0), (1, 1), (1, 2), (1, 7), (2, 3), (3, 5)]:
        mine, _ = orc.hbp(P.D, P.V, model, levels, iters, labels=init)
        ref = orc.ref_hbp(P.D, P.V, model, P.scale, P.trunc, levels, iters, labels=init)
        assert np.array_equal(mine, ref), (levels, iters)
    if model != synth.EXPLICIT:
        _, m = orc.hbp(P.D, P.V, model, 1, 9, want_msgs=True)
        r = orc.ref_bp_msgs(P.D, P.V, model, P.scale, P.trunc, 9)
        assert np.array_equal(m.view(np.uint32), r.view(np.uint32))
    for asyn in (False, True):
        assert np.array_equal(orc.icm(P.D, P.V, mine, 3, asynchronous=asyn),
                              orc.ref_icm(P.D, P.V, model, P.scale, P.trunc, mine, 3, asynchronous=asyn))
    assert np.float32(orc.energy(P.D, P.V, mine, exact_type=True)) == \
        np.float32(orc.ref_energy(P.D, P.V, model, P.scale, P.trunc, mine))


def test_oracle_stereo_png_vs_reference(orc, golden):
    """Real data: the reference example's stereo pair (stereo.cc:28-45 recipe:
    Grid<int>, L=16, cost min(|L - R(x-k)|, 20) for x >= L-1, TruncLinear(10, 20),
    30 iterations), decoded by the oracle and by the reference; the grey
    images and labels stored in the golden fixtures are what they give."""
    _need_ref(orc)
    import os
    from golden.png_grey import grey, stereo_costs_u8
    path = os.path.join(orc.REF_SRC, "examples", "stereo")
    if not os.path.exists(os.path.join(path, "left.png")):
        pytest.skip("stereo pair not present")
    left, right = grey(os.path.join(path, "left.png")), grey(os.path.join(path, "right.png"))
    L = 16
    D = stereo_costs_u8(left, right, L, 20)
    V = synth.sm_table(L, synth.TRUNC_LINEAR, 10, 20, dtype=np.int32)
    mine, _ = orc.hbp(D, V, synth.TRUNC_LINEAR, 1, 30)
    ref = orc.ref_hbp(D, V, synth.TRUNC_LINEAR, 10, 20, 1, 30)
    assert np.array_equal(mine, ref)
    meta, arr = golden
    case = meta["cases"]["stereo_png_384x288_L16"]
    assert np.array_equal(arr["stereo_png_384x288_L16/left"], left)
    assert np.array_equal(arr["stereo_png_384x288_L16/right"], right)
    assert sha(D) == case["cost_sha"] and sha(ref) == case["labels_sha"]


def test_oracle_matches_golden_stereo_png(orc, golden):
    """The reference example's stereo pair from the stored grey images (no
    reference checkout needed): the oracle's costs and labels equal the
    reference's (golden SHA-256)."""
    from golden.png_grey import stereo_costs_u8
    meta, arr = golden
    name = "stereo_png_384x288_L16"
    case = meta["cases"][name]
    D = stereo_costs_u8(arr[name + "/left"], arr[name + "/right"], case["L"], case["cap"])
    assert sha(D) == case["cost_sha"]
    V = synth.sm_table(case["L"], synth.TRUNC_LINEAR, case["scale"], case["trunc"], dtype=np.int32)
    lab, _ = orc.hbp(D, V, synth.TRUNC_LINEAR, 1, case["iters"])
    assert sha(lab) == case["labels_sha"]
    assert orc.energy(D, V, lab, exact_type=True) == case["energy_ref_type"]


def test_oracle_matches_golden_small(orc, golden):
    meta, arr = golden
    for name, case in meta["cases"].items():
        if case["kind"] not in ("bp", "hbp"):
            continue
        P = golden_problem(case)
        assert sha(P.D) == case["cost_sha"], f"{name}: synthetic generator drifted"
        init = arr[name + "/init"].astype(np.int32)
        lab, msgs = orc.hbp(P.D, P.V, case["model"], case["levels"], case["iters"], labels=init,
                            want_msgs=case["kind"] == "bp")
        assert np.array_equal(lab, arr[name + "/labels"]), name
        if case["kind"] == "bp":
            if "msgs_sha" in case:
                assert sha(msgs) == case["msgs_sha"], name
            else:
                assert np.array_equal(msgs.view(np.uint32), arr[name + "/msgs"].view(np.uint32)), name
            assert np.array_equal(orc.icm(P.D, P.V, lab, 3), arr[name + "/icm_sync3"]), name
            assert np.array_equal(orc.icm(P.D, P.V, lab, 2, asynchronous=True), arr[name + "/icm_async2"]), name
        e = orc.energy(P.D, P.V, lab, exact_type=True)
        assert np.float32(e) == np.float32(case["energy_ref_type"]), name


def test_oracle_matches_golden_plain_bp(orc, golden):
    meta, arr = golden
    case = meta["cases"]["plain_bp_384x288_L16"]
    P = workload("plain_bp")
    assert sha(P.D) == case["cost_sha"]
    lab, _ = orc.hbp(P.D, P.V, P.model, 1, 50)
    assert sha(lab) == case["labels_sha"]
    assert orc.energy(P.D, P.V, lab) == pytest.approx(case["energy_f64"], rel=1e-12)
    icm = orc.icm(P.D, P.V, lab, 5)
    assert sha(icm) == case["icm5_sha"]


def test_oracle_matches_golden_hbp_full(orc, golden):
    meta, _ = golden
    case = meta["cases"].get("hbp_1920x1080_L64")
    if case is None:
        pytest.skip("large golden case not generated")
    P = workload("hbp_1920")
    assert sha(P.D) == case["cost_sha"]
    lab, _ = orc.hbp(P.D, P.V, P.model, 5, 10)
    assert sha(lab) == case["labels_sha"]
    icm = orc.icm(P.D, P.V, lab, 5)
    assert sha(icm) == case["icm5_sha"]
    assert orc.energy(P.D, P.V, icm) == pytest.approx(case["icm5_energy_f64"], rel=1e-12)


def test_oracle_thread_count_invariant(orc):
    P = synth.random_problem(57, 41, 16, 7)
    a, ma = orc.hbp(P.D, P.V, P.model, 2, 6, want_msgs=True, nthreads=1)
    b, mb = orc.hbp(P.D, P.V, P.model, 2, 6, want_msgs=True, nthreads=4)
    assert np.array_equal(a, b) and np.array_equal(ma.view(np.uint32), mb.view(np.uint32))


def test_dt_quad_matches_brute_force(orc):
    rng = synth.Rng(5, 3)
    for L in (2, 3, 8, 17, 64, 128):
        for s in (0.25, 1.0, 3.0):
            f = rng.uniform(L) * 50.0
            i = np.arange(L)
            V = s * (i[None, :] - i[:, None]).astype(np.float64) ** 2
            brute = orc.minconv_brute(f, V.reshape(-1))
            assert np.allclose(orc.dt_quad(f, s), brute, rtol=0, atol=1e-9), (L, s)


def test_pyramid_ceil_halving(orc):
    P = synth.random_problem(7, 5, 3, 1)
    c = orc.pyramid(P.D)
    assert c.shape == (3, 3, 4)
    ref = np.zeros((3, 3, 4), np.float32)
    for y in range(5):
        for x in range(7):
            ref[:, y // 2, x // 2] += P.D[:, y, x]
    assert np.array_equal(c, ref)


def test_energy_fp64_close_to_reference_type(orc):
    P = synth.random_problem(40, 30, 16, 9)
    lab, _ = orc.hbp(P.D, P.V, P.model, 1, 10)
    e32 = orc.energy(P.D, P.V, lab, exact_type=True)
    e64 = orc.energy(P.D, P.V, lab)
    assert abs(e32 - e64) / abs(e64) < 1e-5


def test_fp64_standard_oracle_equals_reference_on_linear(orc):
    """For truncated-linear smoothness the standard rule is the reference rule,
    so the FP64 oracle lands on the same labels (up to FP32 rounding ties)."""
    P = synth.random_problem(48, 36, 16, 12)
    l32, _ = orc.hbp(P.D, P.V, P.model, 1, 20)
    l64, _ = orc.hbp_f64_std(P.D, P.V, P.model, 1, 20)
    assert (l32 == l64).mean() > 0.99


@pytest.mark.parametrize("W,H,L,seed,model,scale,trunc,iters", [
    (9, 7, 3, 1, synth.TRUNC_LINEAR, 1, 2, 2), (17, 13, 4, 2, synth.POTTS, 3, 0, 3),
    (20, 15, 5, 3, synth.TRUNC_LINEAR, 2, 6, 2), (12, 10, 6, 4, synth.EXPLICIT, 0, 0, 2),
    (1, 8, 3, 5, synth.TRUNC_LINEAR, 1, 3, 2), (8, 1, 2, 6, synth.POTTS, 2, 0, 2), (2, 2, 2, 7, synth.POTTS, 1, 0, 3),
    (31, 23, 8, 8, synth.TRUNC_LINEAR, 3, 9, 3), (40, 30, 4, 9, synth.TRUNC_QUAD, 1, 9, 2),
    (25, 19, 5, 10, synth.TRUNC_LINEAR, 2, 6, 0)])
def test_alpha_beta_oracle_vs_reference(orc, W, H, L, seed, model, scale, trunc, iters):
    """The C restatement of the alpha-beta swap (graphcut.cc:197-279) against
    the reference's own compiled decodeAlphaBeta<int>, bit for bit, from a
    random initial labelling."""
    _need_ref(orc)
    P = synth.random_problem(W, H, L, seed, model=model, scale=scale, trunc=trunc, dtype=np.int32, cost_max=20)
    init = synth.Rng(seed, 5).integers(0, L - 1, W * H).reshape(H, W).astype(np.int32)
    ref = orc.ref_alpha_beta(P.D, P.V, model, scale, trunc, init, iters)
    assert np.array_equal(orc.alpha_beta(P.D, P.V, init, iters), ref)


def test_oracle_matches_golden_alpha_beta(orc, golden):
    """The alpha-beta fixtures the reference wrote (tests/golden), reproduced
    by the C restatement without the reference checkout."""
    meta, arr = golden
    cases = [(n, c) for n, c in meta["cases"].items() if c["kind"] == "alpha_beta"]
    assert len(cases) >= 5
    for name, case in cases:
        P = golden_problem(case)
        assert sha(P.D) == case["cost_sha"], name
        lab = orc.alpha_beta(P.D, P.V, arr[name + "/init"].astype(np.int32), case["iters"])
        assert np.array_equal(lab, arr[name + "/labels"]), name
        assert orc.energy(P.D, P.V, lab, exact_type=True) == case["energy_ref_type"], name
