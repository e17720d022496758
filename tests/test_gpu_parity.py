"""GPU parity: the CUDA path, called through the C ABI, against the reference's
own outputs (golden fixtures) and the CPU oracle.  FP32 and int32 BP, HBP and
ICM are required to be bit-identical; FP16 / FP64 / standard-rule runs are
held to the tolerances written in each test."""
import numpy as np
import pytest

from gridinfcuda_gb300 import synth
from helpers import golden_problem, sha, workload

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _cases(meta, kind):
    return [(n, c) for n, c in meta["cases"].items() if c["kind"] == kind]


def test_golden_bp_cases_bit_exact(ginf, golden):
    meta, arr = golden
    for name, case in _cases(meta, "bp"):
        P = golden_problem(case)
        init = arr[name + "/init"].astype(np.int32)
        lab, msgs = ginf.decode_hbp(P.D, P.V, case["model"], 1, case["iters"], labels=init.copy(), want_msgs=True)
        assert np.array_equal(lab, arr[name + "/labels"]), name
        if "msgs_sha" in case:
            assert sha(msgs) == case["msgs_sha"], name
        else:
            assert np.array_equal(msgs.view(np.uint32), arr[name + "/msgs"].view(np.uint32)), name
        icm_s = ginf.decode_icm(P.D, P.V, case["model"], lab, 3)
        assert np.array_equal(icm_s, arr[name + "/icm_sync3"]), name
        icm_a = ginf.decode_icm(P.D, P.V, case["model"], lab, 2, asynchronous=True)
        assert np.array_equal(icm_a, arr[name + "/icm_async2"]), name
        e = ginf.energy(P.D, P.V, case["model"], lab)
        assert e == pytest.approx(case["energy_ref_type"], rel=1e-5, abs=1e-6), name


def test_golden_hbp_cases_bit_exact(ginf, golden):
    meta, arr = golden
    for name, case in _cases(meta, "hbp"):
        P = golden_problem(case)
        init = arr[name + "/init"].astype(np.int32)
        lab = ginf.decode_hbp(P.D, P.V, case["model"], case["levels"], case["iters"], labels=init.copy())
        assert np.array_equal(lab, arr[name + "/labels"]), name


def test_golden_cases_device_buffers(ginf, golden):
    """Same fixtures with every buffer resident on the device."""
    meta, arr = golden
    for name, case in meta["cases"].items():
        if case["kind"] not in ("bp", "hbp"):
            continue
        P = golden_problem(case)
        init = _dev(arr[name + "/init"].astype(np.int32))
        lab = ginf.decode_hbp(_dev(P.D), _dev(P.V), case["model"], case["levels"], case["iters"], labels=init)
        assert np.array_equal(lab.cpu().numpy(), arr[name + "/labels"]), name


def test_plain_bp_workload_matches_reference(ginf, golden):
    meta, _ = golden
    case = meta["cases"]["plain_bp_384x288_L16"]
    P = workload("plain_bp")
    assert sha(P.D) == case["cost_sha"]
    lab = ginf.decode_hbp(P.D, P.V, P.model, 1, 50)
    assert sha(lab) == case["labels_sha"]
    assert ginf.energy(P.D, P.V, P.model, lab) == pytest.approx(case["energy_f64"], rel=1e-12)
    icm = ginf.decode_icm(P.D, P.V, P.model, lab, 5)
    assert sha(icm) == case["icm5_sha"]


def test_hbp_workload_matches_reference(ginf, golden):
    """1920x1080, L=64, 5 levels x 10 half-sweeps, 5 ICM sweeps: labels
    bit-identical to the reference CPU code, energy in FP64."""
    meta, _ = golden
    case = meta["cases"].get("hbp_1920x1080_L64")
    if case is None:
        pytest.skip("large golden case not generated")
    P = workload("hbp_1920")
    assert sha(P.D) == case["cost_sha"]
    lab = ginf.decode_hbp(P.D, P.V, P.model, 5, 10)
    assert sha(lab) == case["labels_sha"]
    lab2, e = ginf.solve(_dev(P.D), _dev(P.V), P.model, 5, 10, 5)
    assert sha(lab2.cpu().numpy()) == case["icm5_sha"]
    assert e == pytest.approx(case["icm5_energy_f64"], rel=1e-12)


@pytest.mark.parametrize("W,H,L,levels,iters", [
    (5, 5, 2, 1, 4), (8, 3, 5, 1, 6), (47, 35, 33, 1, 7), (50, 40, 65, 2, 5), (39, 27, 100, 1, 5),
    (64, 64, 128, 3, 4), (129, 97, 16, 4, 6), (200, 3, 16, 1, 5), (3, 200, 32, 2, 5), (70, 50, 64, 1, 2)])
def test_random_vs_oracle(ginf, orc, W, H, L, levels, iters):
    P = synth.random_problem(W, H, L, W * 131 + H * 7 + L)
    want, msgs_want = orc.hbp(P.D, P.V, P.model, levels, iters, want_msgs=True)
    for tile in (0, 8, 32):
        got, msgs = ginf.decode_hbp(P.D, P.V, P.model, levels, iters, want_msgs=True, tile_nodes=tile)
        assert np.array_equal(got[1:-1, 1:-1], want[1:-1, 1:-1]), tile
        assert np.array_equal(msgs.view(np.uint32), msgs_want.view(np.uint32)), tile


def test_int_grid_vs_oracle(ginf, orc):
    P = synth.random_problem(61, 45, 16, 77, dtype=np.int32, scale=10, trunc=20, cost_max=40)
    want, mw = orc.hbp(P.D, P.V, P.model, 3, 6, want_msgs=True)
    got, mg = ginf.decode_hbp(P.D, P.V, P.model, 3, 6, want_msgs=True)
    assert np.array_equal(got, want)
    assert np.array_equal(mg, mw)


def test_reference_rule_quadratic_and_explicit(ginf, orc):
    for model in (synth.TRUNC_QUAD, synth.EXPLICIT):
        P = synth.random_problem(37, 29, 12, 5 + model, model=model, scale=1.0, trunc=9.0)
        want, mw = orc.hbp(P.D, P.V, model, 1, 4, want_msgs=True)
        got, mg = ginf.decode_hbp(P.D, P.V, model, 1, 4, want_msgs=True)
        assert np.array_equal(got, want)
        assert np.array_equal(mg.view(np.uint32), mw.view(np.uint32))


def _renorm(m):
    m = m.astype(np.float64)
    return m - m.mean(axis=-1, keepdims=True)


def _msg_rel_err(a, b):
    """max |a-b| / max|b| after re-normalising both to zero mean per message."""
    a, b = _renorm(a), _renorm(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)


def test_fp64_path_matches_fp64_oracle(ginf, orc):
    P = synth.random_problem(45, 33, 24, 31, model=synth.TRUNC_QUAD, scale=0.5, trunc=9.0)
    want, mw = orc.hbp_f64_std(P.D, P.V, P.model, 2, 6, want_msgs=True)
    got, mg = ginf.decode_hbp(P.D, P.V, P.model, 2, 6, want_msgs=True, compute_type=ginf.F64, rule=ginf.RULE_STANDARD)
    assert _msg_rel_err(mg, mw) < 1e-12
    assert (got[1:-1, 1:-1] == want[1:-1, 1:-1]).mean() == 1.0


def test_fp64_path_on_the_precision_workload_recipe(ginf, orc):
    """The FP64 path that the precision sweep measures FP32 and FP16 against,
    on that workload's own recipe (80 slanted planes, sigma 3, L = 128,
    D = 0.05 min(|dI|, 20), V = min((a-b)^2, 25)) at 384x216, for the sweep's
    full 40 half-sweeps: messages within 1e-12 of the CPU FP64 oracle and
    identical labels."""
    P = synth.workload_quad(seed=3, W=384, H=216, L=128)
    want, mw = orc.hbp_f64_std(P.D, P.V, P.model, 1, 40, want_msgs=True)
    got, mg = ginf.decode_hbp(P.D, P.V, P.model, 1, 40, want_msgs=True, compute_type=ginf.F64,
                              rule=ginf.RULE_STANDARD)
    assert _msg_rel_err(mg, mw) < 1e-12
    assert np.array_equal(got[1:-1, 1:-1], want[1:-1, 1:-1])


def test_standard_quadratic_fp32_and_fp16_vs_fp64_oracle(ginf, orc):
    """Truncated-quadratic standard BP against the FP64 oracle: messages within
    1e-4 (FP32 store) / 5e-3 (FP16 store) relative; labels agree on >= 99.9% /
    99% of nodes.  Energies within 1e-3 / 5e-3: one label flip at a near-tie
    moves this 96x72 grid's energy by an integer table step (4 / 14174 =
    2.8e-4), so the bound allows a few flips."""
    P = synth.stereo_problem(96, 72, 32, seed=4, n_regions=10, sigma=3.0, planar=True, coef=0.05, cap=20.0,
                             model=synth.TRUNC_QUAD, scale=1.0, trunc=25.0)
    want, mw = orc.hbp_f64_std(P.D, P.V, P.model, 1, 12, want_msgs=True)
    e_want = orc.energy(P.D, P.V, want)
    f32, m32 = ginf.decode_hbp(P.D, P.V, P.model, 1, 12, want_msgs=True, rule=ginf.RULE_STANDARD)
    assert _msg_rel_err(m32, mw) < 1e-4
    assert (f32[1:-1, 1:-1] == want[1:-1, 1:-1]).mean() >= 0.999
    assert abs(orc.energy(P.D, P.V, f32) - e_want) / abs(e_want) < 1e-3
    _, mw_min = orc.hbp_f64_std(P.D, P.V, P.model, 1, 12, norm=1, want_msgs=True)
    f16, m16 = ginf.decode_hbp(P.D, P.V, P.model, 1, 12, want_msgs=True, rule=ginf.RULE_STANDARD,
                               store=ginf.STORE_F16)
    assert _msg_rel_err(m16, mw_min) < 5e-3
    assert (f16[1:-1, 1:-1] == want[1:-1, 1:-1]).mean() >= 0.99
    assert abs(orc.energy(P.D, P.V, f16) - e_want) / abs(e_want) < 5e-3


def test_fp16_store_linear_vs_fp64(ginf, orc):
    P = synth.workload_plain_bp()
    want, _ = orc.hbp_f64_std(P.D, P.V, P.model, 1, 50)
    got = ginf.decode_hbp(P.D, P.V, P.model, 1, 50, store=ginf.STORE_F16)
    assert (got[1:-1, 1:-1] == want[1:-1, 1:-1]).mean() >= 0.99
    e_w, e_g = orc.energy(P.D, P.V, want), orc.energy(P.D, P.V, got)
    assert abs(e_g - e_w) / abs(e_w) < 1e-3


def test_fresh_decode_vs_oracle(ginf, orc):
    P = synth.random_problem(52, 40, 16, 3)
    want, _ = orc.hbp_f64_std(P.D, P.V, P.model, 1, 10, decode=1)
    got = ginf.decode_hbp(P.D, P.V, P.model, 1, 10, decode=ginf.DECODE_FRESH)
    assert (got[1:-1, 1:-1] == want[1:-1, 1:-1]).mean() > 0.99


def test_deterministic_and_workspace_reuse(ginf):
    P = synth.random_problem(90, 70, 32, 8)
    with ginf.Workspace() as ws:
        a, ma = ginf.decode_hbp(P.D, P.V, P.model, 3, 6, want_msgs=True, workspace=ws)
        b, mb = ginf.decode_hbp(P.D, P.V, P.model, 3, 6, want_msgs=True, workspace=ws)
        small = synth.random_problem(20, 10, 8, 2)
        ginf.decode_hbp(small.D, small.V, small.model, 1, 3, workspace=ws)
        c, mc = ginf.decode_hbp(P.D, P.V, P.model, 3, 6, want_msgs=True, workspace=ws)
    assert np.array_equal(a, b) and np.array_equal(a, c)
    assert np.array_equal(ma.view(np.uint32), mb.view(np.uint32))
    assert np.array_equal(ma.view(np.uint32), mc.view(np.uint32))


def test_solve_matches_separate_calls(ginf, orc):
    P = synth.random_problem(80, 60, 32, 21)
    lab, e = ginf.solve(P.D, P.V, P.model, 3, 6, 4)
    hbp, _ = orc.hbp(P.D, P.V, P.model, 3, 6)
    icm = orc.icm(P.D, P.V, hbp, 4)
    assert np.array_equal(lab, icm)
    assert e == pytest.approx(orc.energy(P.D, P.V, icm), rel=1e-12)


def test_border_labels_untouched(ginf):
    P = synth.random_problem(30, 20, 8, 4)
    init = np.full((20, 30), 7, np.int32)
    lab = ginf.decode_hbp(P.D, P.V, P.model, 2, 4, labels=init)
    assert (lab[0] == 7).all() and (lab[-1] == 7).all() and (lab[:, 0] == 7).all() and (lab[:, -1] == 7).all()


def test_stereo_cost_kernel_bit_exact(ginf):
    import torch
    pair = synth.stereo_pair(160, 90, 24, 5, 2.0, seed=3)
    want = synth.cost_volume(pair, 24, 0.07, 15.0)
    out = torch.empty((24, 90, 160), dtype=torch.float32, device="cuda")
    ginf.stereo_costs(_dev(pair.left), _dev(pair.right), 24, 0.07, 15.0, out)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), want.view(np.uint32))
    out2 = torch.empty_like(out)
    ginf.stereo_costs(pair.left, pair.right, 24, 0.07, 15.0, out2)
    assert torch.equal(out, out2)


def test_reference_stereo_example_end_to_end(ginf, golden):
    """The reference example on its own stereo pair (examples/stereo/stereo.cc:
    16-43): 8-bit grey images -> the integer cost volume on the GPU
    (ginf_stereo_costs_u8: min(|L(x) - R(x-k)|, 20) for x >= L-1, zero
    elsewhere) -> Grid<int> loopy BP, TruncLinear(10, 20), 30 iterations.
    Costs and labels must equal what the reference's own code produced
    (golden SHA-256), from device and from host images."""
    import torch
    meta, arr = golden
    name = "stereo_png_384x288_L16"
    case = meta["cases"][name]
    left, right = arr[name + "/left"], arr[name + "/right"]
    H, W, L = case["H"], case["W"], case["L"]
    V = _dev(synth.sm_table(L, synth.TRUNC_LINEAR, case["scale"], case["trunc"], dtype=np.int32))
    for src in ("device", "host"):
        D = torch.full((L, H, W), -1, dtype=torch.int32, device="cuda")   # every element must be written
        if src == "device":
            ginf.stereo_costs_u8(_dev(left), _dev(right), L, case["cap"], D)
        else:
            ginf.stereo_costs_u8(left, right, L, case["cap"], D)
        assert sha(D.cpu().numpy()) == case["cost_sha"], src
        lab = torch.zeros((H, W), dtype=torch.int32, device="cuda")
        ginf.decode_hbp(D, V, synth.TRUNC_LINEAR, 1, case["iters"], labels=lab)
        got = lab.cpu().numpy()
        assert sha(got) == case["labels_sha"], src
        assert np.array_equal(got, arr[name + "/labels"].astype(np.int32)), src
        e = ginf.energy(D, V, synth.TRUNC_LINEAR, lab)
        assert e == case["energy_ref_type"], src


def test_errors_are_reported_not_fatal(ginf):
    P = synth.random_problem(10, 8, 4, 1)
    with pytest.raises(ginf.GinfError) as e:
        ginf.decode_hbp(P.D, P.V, P.model, 0, 3)
    assert e.value.status == ginf.ERR_INVALID_ARGUMENT
    big = synth.random_problem(6, 5, 130, 1)
    with pytest.raises(ginf.GinfError) as e:
        ginf.decode_hbp(big.D, big.V, big.model, 1, 3)
    assert e.value.status == ginf.ERR_UNSUPPORTED
    bad = np.full((8, 10), 9, np.int32)   # labels outside [0, 4)
    with pytest.raises(ginf.GinfError) as e:
        ginf.energy(P.D, P.V, P.model, bad)
    assert e.value.status == ginf.ERR_INVALID_ARGUMENT
    with pytest.raises(ginf.GinfError) as e:
        ginf.decode_icm(P.D, P.V, P.model, bad, 2)
    assert e.value.status == ginf.ERR_INVALID_ARGUMENT
    # the library stays usable after the errors
    lab = ginf.decode_hbp(P.D, P.V, P.model, 1, 3)
    assert lab.shape == (8, 10)


def test_windowed_quadratic_equals_min_convolution(ginf):
    """The windowed truncated-quadratic transform is the exact minimum over the
    whole table: bit-identical to the O(L^2) min-convolution of the same table.
    FP32 records at L = 128 run the split kernel (two warps per eight nodes):
    radius 4 (trunc 25) and radius 7 (trunc 50) windows, the mean and the
    minimum subtracted, FP32 and FP16 messages, 37- and 70-wide grids
    (partial last tiles), two levels (the coarse-to-fine first sweep).  FP16
    cases use a table offset by V(0,0) = 0.5, which keeps them on the window
    form (an exactly quadratic table with the FP16 store runs the pass form,
    test_fp16_quadratic_pass_form_vs_min_convolution)."""
    F32, F16 = ginf.STORE_NATIVE, ginf.STORE_F16
    cases = [(128, 25.0, 37, 23, ginf.NORM_MEAN, F32), (128, 25.0, 37, 23, ginf.NORM_MIN, F32),
             (128, 50.0, 70, 41, ginf.NORM_MEAN, F32), (128, 50.0, 70, 41, ginf.NORM_MIN, F32),
             (128, 25.0, 37, 23, ginf.NORM_MIN, F16), (128, 50.0, 70, 41, ginf.NORM_MIN, F16),
             (17, 9.0, 37, 23, ginf.NORM_MEAN, F32), (64, 2.0, 37, 23, ginf.NORM_MEAN, F32),
             (64, 25.0, 37, 23, ginf.NORM_MIN, F16)]
    for L, trunc, W, H, norm, store in cases:
        P = synth.random_problem(W, H, L, 40 + L, model=synth.TRUNC_QUAD, scale=1.0, trunc=trunc, cost_max=30.0)
        V = P.V + np.float32(0.5) if store == F16 else P.V
        opt = dict(want_msgs=True, rule=ginf.RULE_STANDARD, normalize=norm, store=store)
        lq, mq = ginf.decode_hbp(P.D, V, synth.TRUNC_QUAD, 2, 5, **opt)
        lb, mb = ginf.decode_hbp(P.D, V, synth.EXPLICIT, 2, 5, **opt)
        case = (L, trunc, norm, store)
        assert np.array_equal(lq, lb), case
        assert mq.dtype == mb.dtype and np.array_equal(mq.view(np.uint8), mb.view(np.uint8)), case


def test_fp16_quadratic_pass_form_vs_min_convolution(ginf):
    """FP16 store with an exactly quadratic table V(0,k) = s k^2 (radius <= 4):
    the distance transform runs as r min-plus passes, whose sums round step by
    step, so it is held to the FP16 store's resolution against the O(L^2)
    min-convolution: messages within 2^-8 of their largest magnitude (four
    FP16 steps at the top of the range) after five half-sweeps on two levels,
    labels equal on >= 99.5 % of the interior, and each message's minimum
    exactly 0 (min-normalised)."""
    for L, trunc, W, H, scale in [(128, 25.0, 37, 23, 1.0), (64, 25.0, 37, 23, 1.0), (128, 9.0, 70, 41, 0.6),
                                  (48, 16.0, 41, 30, 1.0)]:
        P = synth.random_problem(W, H, L, 60 + L, model=synth.TRUNC_QUAD, scale=scale, trunc=trunc, cost_max=30.0)
        opt = dict(want_msgs=True, rule=ginf.RULE_STANDARD, normalize=ginf.NORM_MIN, store=ginf.STORE_F16)
        lq, mq = ginf.decode_hbp(P.D, P.V, synth.TRUNC_QUAD, 2, 5, **opt)
        lb, mb = ginf.decode_hbp(P.D, P.V, synth.EXPLICIT, 2, 5, **opt)
        a, b = mq.astype(np.float64), mb.astype(np.float64)
        case = (L, trunc, scale)
        assert np.abs(a - b).max() <= 2.0 ** -8 * np.abs(b).max(), case
        assert (lq[1:-1, 1:-1] == lb[1:-1, 1:-1]).mean() >= 0.995, case
        inner = a[1:-1, 1:-1]
        live = np.abs(inner).max(axis=-1) > 0   # slots from interior senders
        assert (inner.min(axis=-1)[live] == 0).all(), case


def test_wide_quadratic_lower_envelope_vs_fp64(ginf, orc):
    """Truncation radius beyond the window (s = 0.05, d = 25: radius 22): the
    lower-envelope transform, FP32 store within 1e-4 of the FP64 oracle."""
    P = synth.random_problem(41, 31, 64, 9, model=synth.TRUNC_QUAD, scale=0.05, trunc=25.0, cost_max=30.0)
    want, mw = orc.hbp_f64_std(P.D, P.V, P.model, 1, 8, want_msgs=True)
    got, mg = ginf.decode_hbp(P.D, P.V, P.model, 1, 8, want_msgs=True, rule=ginf.RULE_STANDARD)
    assert _msg_rel_err(mg, mw) < 1e-4
    assert (got[1:-1, 1:-1] == want[1:-1, 1:-1]).mean() >= 0.999


def test_host_costs_read_in_place_or_staged(ginf, orc):
    """Host costs read in place by the device (page-locked memory, and
    pageable memory where the device reads it coherently) or staged by a
    copy: identical labels and messages, equal to the oracle's."""
    import torch
    P = synth.random_problem(97, 61, 24, 5)
    want, msgs_want = orc.hbp(P.D, P.V, P.model, 3, 5, want_msgs=True)
    pinned = (torch.from_numpy(P.D).pin_memory(), torch.from_numpy(P.V).pin_memory())
    for D, V in ((P.D, P.V), pinned):
        for access in (ginf.HOST_AUTO, ginf.HOST_COPY):
            lab, msgs = ginf.decode_hbp(D, V, P.model, 3, 5, want_msgs=True, host_access=access)
            lab, msgs = np.asarray(lab), np.asarray(msgs)
            assert np.array_equal(lab[1:-1, 1:-1], want[1:-1, 1:-1]), (type(D), access)
            assert np.array_equal(msgs.view(np.uint32), msgs_want.view(np.uint32)), (type(D), access)
    with pytest.raises(ginf.GinfError):
        ginf.decode_hbp(P.D, P.V, P.model, 3, 5, host_access=7)


def test_stream_ordered_solve(ginf):
    """Stream-ordered ginf_solve on two workspaces and two streams, pinned
    host buffers: every frame equals the synchronous call; misuse is
    rejected."""
    import ctypes
    import torch
    P = synth.random_problem(150, 110, 32, 9)
    want_lab, want_e = ginf.solve(P.D, P.V, P.model, 3, 6, 2)
    D, V = torch.from_numpy(P.D).pin_memory(), torch.from_numpy(P.V).pin_memory()
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    wss = [ginf.Workspace(), ginf.Workspace()]
    labs = [torch.zeros((110, 150), dtype=torch.int32).pin_memory() for _ in range(4)]
    es = [ctypes.c_double() for _ in range(4)]
    for access in (ginf.HOST_COPY, ginf.HOST_AUTO):
        for i in range(4):
            ginf.solve_async(D, V, P.model, 3, 6, 2, labs[i], es[i], wss[i % 2], streams[i % 2].cuda_stream,
                             host_access=access)
        for w in wss:
            w.sync()
        for i in range(4):
            assert np.array_equal(labs[i].numpy()[1:-1, 1:-1], want_lab[1:-1, 1:-1]), (access, i)
            assert es[i].value == want_e, (access, i)
            labs[i].zero_()
            es[i].value = 0.0
    with pytest.raises(ginf.GinfError):   # no workspace
        g = ginf.make_grid(P.D, P.V, P.model)
        o = ginf.options(stream_ordered=1)
        lab = np.zeros((110, 150), np.int32)
        ginf.check(ginf.lib().ginf_decode_hbp(None, ctypes.byref(g), 3, 6, lab.ctypes.data, ctypes.byref(o), None))
    with pytest.raises(ginf.GinfError):   # stats requested
        ginf.decode_hbp(P.D, P.V, P.model, 3, 6, workspace=wss[0], want_stats=True, stream_ordered=1)
    for w in wss:
        w.close()


def test_concurrent_host_threads(ginf):
    """Calls are reentrant per workspace: four host threads, each with its own
    workspace and stream, solve different grids (label counts 16, 24, 64 and
    128, so several kernels and their launch caches are first used
    concurrently) at the same time; every result equals the single-thread
    call."""
    import threading
    import torch
    cases = [synth.random_problem(90 + 7 * k, 70 + 5 * k, L, 300 + k, model=synth.TRUNC_QUAD if L == 24 else
                                  synth.TRUNC_LINEAR) for k, L in enumerate((16, 24, 64, 128))]
    got = [None] * len(cases)
    errors = []
    start = threading.Barrier(len(cases))

    def run(k):
        try:
            P = cases[k]
            stream = torch.cuda.Stream()
            with ginf.Workspace() as ws:
                start.wait()
                res = []
                for _ in range(3):
                    res.append(ginf.solve(P.D, P.V, P.model, 3, 5, 2, workspace=ws, stream=stream.cuda_stream))
                got[k] = res
        except Exception as e:  # reported on the main thread
            errors.append(e)

    threads = [threading.Thread(target=run, args=(k,)) for k in range(len(cases))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    want = [ginf.solve(P.D, P.V, P.model, 3, 5, 2) for P in cases]
    for k, res in enumerate(got):
        for lab, e in res:
            assert np.array_equal(lab[1:-1, 1:-1], want[k][0][1:-1, 1:-1]), k
            assert e == want[k][1], k


@pytest.mark.parametrize("W,H", [(1, 1), (2, 9), (9, 2), (1, 40), (3, 3), (4, 3)])
def test_grids_without_or_with_tiny_interior(ginf, orc, W, H):
    """Grids with no interior node (nothing updates: every label stays the
    caller's) or a one-node-wide interior, through BP, HBP, ICM, solve and the
    energy, host and device buffers: equal to the oracle."""
    import torch
    P = synth.random_problem(W, H, 6, W * 17 + H)
    init = (np.arange(W * H, dtype=np.int32).reshape(H, W) % 6).astype(np.int32)
    for levels in (1, 3):
        got = ginf.decode_hbp(P.D, P.V, P.model, levels, 4, labels=init.copy())
        ref, _ = orc.hbp(P.D, P.V, P.model, levels, 4, want_msgs=True)
        if W < 3 or H < 3:
            assert np.array_equal(got, init), (levels, "no interior: labels unchanged")
        else:
            assert np.array_equal(got[1:-1, 1:-1], ref[1:-1, 1:-1]), levels
        gd = ginf.decode_hbp(_dev(P.D), _dev(P.V), P.model, levels, 4, labels=_dev(init.copy())).cpu().numpy()
        assert np.array_equal(gd, got), levels
    icm = ginf.decode_icm(P.D, P.V, P.model, init, 3)
    assert np.array_equal(icm, orc.icm(P.D, P.V, init, 3))
    lab, e = ginf.solve(P.D, P.V, P.model, 2, 4, 2, labels=init.copy())
    assert e == pytest.approx(orc.energy(P.D, P.V, lab), rel=1e-12, abs=1e-12)


def test_very_tall_grids(ginf, orc):
    """More rows than a CUDA grid's y dimension holds (65535): the layout
    transform, the fused level-1 pyramid and the sweeps walk every row."""
    for W, H, levels in ((4, 70000, 1), (5, 140000, 3)):
        P = synth.random_problem(W, H, 2, H)
        want = orc.hbp(P.D, P.V, P.model, levels, 3)[0]
        got = ginf.decode_hbp(P.D, P.V, P.model, levels, 3)
        assert np.array_equal(got[1:-1, 1:-1], want[1:-1, 1:-1]), (W, H, levels)


def test_stream_ordered_decode_and_int_grids_from_host(ginf, orc):
    """ginf_decode_hbp stream-ordered on two workspaces / two streams with
    pinned int32 grids read in place: equal to the oracle."""
    import ctypes
    import torch
    P = synth.random_problem(90, 70, 24, 12, dtype=np.int32)
    want, _ = orc.hbp(P.D, P.V, P.model, 3, 5)
    D, V = torch.from_numpy(P.D).pin_memory(), torch.from_numpy(P.V).pin_memory()
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    wss = [ginf.Workspace(), ginf.Workspace()]
    labs = [torch.zeros((70, 90), dtype=torch.int32).pin_memory() for _ in range(4)]
    g = ginf.make_grid(D, V, P.model)
    for i in range(4):
        o = ginf.options(stream=streams[i % 2].cuda_stream, stream_ordered=1)
        ginf.check(ginf.lib().ginf_decode_hbp(wss[i % 2].handle, ctypes.byref(g), 3, 5, labs[i].data_ptr(),
                                              ctypes.byref(o), None))
    for w in wss:
        w.sync()
    for i in range(4):
        assert np.array_equal(labs[i].numpy()[1:-1, 1:-1], want[1:-1, 1:-1]), i
    for w in wss:
        w.close()


def test_bounded_waits_time_out_and_the_device_stays_usable(ginf, orc):
    """The mbarrier wait and the grid barrier are driven into their time
    limit on purpose (a phase nothing completes, a barrier one block short):
    both record the timeout status and return, and a solve afterwards is
    still exact."""
    mbar, barrier = ginf.selftest_bounded_waits()
    assert mbar == 1 and barrier == 1
    P = synth.random_problem(40, 30, 8, 21)
    want, _ = orc.hbp(P.D, P.V, P.model, 2, 4)
    got = ginf.decode_hbp(P.D, P.V, P.model, 2, 4)
    assert np.array_equal(got[1:-1, 1:-1], want[1:-1, 1:-1])


@pytest.mark.parametrize("W,H,L,levels,iters", [(384, 288, 16, 1, 50), (203, 157, 32, 1, 13), (97, 71, 5, 1, 9),
                                                (130, 91, 24, 1, 7), (61, 250, 12, 2, 6), (300, 41, 31, 3, 5),
                                                (3, 3, 16, 1, 4), (4, 50, 16, 1, 3), (200, 3, 32, 1, 2),
                                                (1025, 257, 16, 1, 20), (515, 300, 32, 4, 10)])
def test_cluster_temporal_blocking_bit_exact(ginf, orc, W, H, L, levels, iters):
    """Several half-sweeps per launch on thread-block clusters (FP32, L <= 32):
    labels and messages equal the one-half-sweep-per-launch kernel for every
    halo depth tried, and the oracle."""
    P = synth.random_problem(W, H, L, 7 * W + H, model=synth.TRUNC_LINEAR if L % 2 else synth.POTTS,
                             scale=1.0 if L % 2 else 0.6, trunc=2.2)
    D, V = _dev(P.D), _dev(P.V)
    lab1, msg1 = ginf.decode_hbp(D, V, P.model, levels, iters, want_msgs=True)
    for k in (2, 3, 5, 8, 15):
        lab, msg = ginf.decode_hbp(D, V, P.model, levels, iters, want_msgs=True, sweeps_per_launch=k)
        assert np.array_equal(lab.cpu().numpy(), lab1.cpu().numpy()), k
        assert np.array_equal(msg.cpu().numpy().view(np.uint32), msg1.cpu().numpy().view(np.uint32)), k
    if W * H * L * iters <= 4e7:
        want, _ = orc.hbp(P.D, P.V, P.model, levels, iters)
        assert np.array_equal(lab1.cpu().numpy(), want)


def test_cluster_launch_schedule(ginf):
    """sweeps_per_launch = 8 runs the 384x288x16 workload's 50 half-sweeps in
    an even number of cluster launches (8), so the level ends in its own
    records; the default runs one half-sweep per launch."""
    P = synth.workload_plain_bp()
    _, st = ginf.decode_hbp(_dev(P.D), _dev(P.V), P.model, 1, 50, want_stats=True, sweeps_per_launch=8)
    assert st["level0_sweep_launches"] == 8
    _, st1 = ginf.decode_hbp(_dev(P.D), _dev(P.V), P.model, 1, 50, want_stats=True)
    assert st1["level0_sweep_launches"] == 50


def test_linear_minimum_with_negative_zero_and_infinite_costs(ginf, orc):
    """The truncated-linear update keeps the reference's (a < b) ? a : b
    minimum (GINF_MIN, utils.h:16) on every input: -0 costs give the oracle's
    messages bit for bit, and infinite costs -- which make NaN messages, where
    that minimum and min.f32 differ -- give the oracle's labels, NaN in the
    same slots and the same finite messages."""
    P = synth.random_problem(41, 29, 8, 77, model=synth.TRUNC_LINEAR, scale=1.0, trunc=2.5)
    D = P.D.copy()
    D[:, 3:9, 4:12] = np.float32(-0.0)
    lab, m = ginf.decode_hbp(_dev(D), _dev(P.V), P.model, 1, 9, want_msgs=True)
    want, mw = orc.hbp(D, P.V, P.model, 1, 9, want_msgs=True)
    assert np.array_equal(lab.cpu().numpy(), want)
    assert np.array_equal(m.cpu().numpy().view(np.uint32), mw.view(np.uint32))
    D = P.D.copy()
    D[2, 10, 7] = np.float32(np.inf)
    D[:, 20, 30] = np.float32(np.inf)
    lab, m = ginf.decode_hbp(_dev(D), _dev(P.V), P.model, 1, 9, want_msgs=True)
    want, mw = orc.hbp(D, P.V, P.model, 1, 9, want_msgs=True)
    m = m.cpu().numpy()
    assert np.isnan(mw).any()
    assert np.array_equal(lab.cpu().numpy(), want)
    assert np.array_equal(np.isnan(m), np.isnan(mw))
    fin = ~np.isnan(mw)
    assert np.array_equal(m[fin], mw[fin])
