"""ginf_decode_bp_noalloc: loopy BP for callers that cannot allocate device
memory (a real-time loop that cannot afford cudaMalloc's synchronisation, or
a plugin whose host application owns all device memory).  It keeps its
working set in a fixed 48 MiB array inside the library instead of a
workspace.  Its labels must equal those of ginf_decode_hbp (one level) -- the
same bit-exact standard as every other FP32 / int32 test -- on consecutive
calls that reuse the shared array, for every smoothness model (Potts and
truncated linear run the O(L) update; explicit tables and truncated
quadratic run the reference's O(L^2) rule, src/bp.cc:55-62), on the legacy
default stream and on a caller's stream; grids above the documented size
rule are refused, not run.

This file is collected last on purpose, and passes whether it runs alone in
a fresh process or after the other tests."""
import ctypes

import numpy as np
import pytest

from gridinfcuda_gb300 import synth

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 48 * 1024 * 1024


def _call_noalloc(capi, D, V, model, iters, labels, stream=None):
    fn = capi.lib().ginf_decode_bp_noalloc
    fn.argtypes = [ctypes.POINTER(capi.Grid), ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int32
    g = capi.make_grid(D, V, model)
    return fn(ctypes.byref(g), iters, labels.data_ptr(), stream)


def _bytes_needed(W, H, L):
    """The header's rule: a 256-byte status block, then per node one record
    of 5 * Lp four-byte elements, Lp = L rounded up to a multiple of 8."""
    Lp = (L + 7) // 8 * 8
    return 256 + W * H * 20 * Lp


def _problems():
    I32 = np.int32
    return [
        (synth.workload_plain_bp(), 50),                                          # 384x288x16, 35 MB of records
        (synth.random_problem(90, 70, 32, 4, dtype=I32, scale=10, trunc=20, cost_max=40), 7),
        (synth.random_problem(33, 17, 5, 6), 1),
        # explicit tables and truncated quadratic: the reference's O(L^2) rule
        (synth.random_problem(41, 29, 12, 31, model=synth.EXPLICIT), 6),
        (synth.random_problem(37, 23, 9, 32, model=synth.EXPLICIT, dtype=I32, cost_max=20), 5),
        (synth.random_problem(45, 31, 16, 33, model=synth.TRUNC_QUAD, scale=1.0, trunc=9.0), 8),
        (synth.random_problem(29, 35, 10, 34, model=synth.TRUNC_QUAD, dtype=I32, scale=2, trunc=30, cost_max=25), 5),
        (synth.random_problem(50, 40, 7, 35, model=synth.POTTS, scale=0.8), 9),
        (synth.workload_plain_bp(), 50),
    ]


def _want(ginf, P, iters, D, V):
    import torch
    H, W = P.D.shape[1:]
    want = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    ginf.decode_hbp(D, V, P.model, 1, iters, labels=want)
    return want


def test_noalloc_matches_decode_hbp_on_consecutive_calls(ginf):
    import torch
    for k, (P, iters) in enumerate(_problems()):
        D = torch.from_numpy(P.D).cuda()
        V = torch.from_numpy(P.V).cuda()
        H, W = P.D.shape[1:]
        want = _want(ginf, P, iters, D, V)
        got = torch.full((H, W), 0, dtype=torch.int32, device="cuda")
        st = _call_noalloc(ginf, D, V, P.model, iters, got)
        assert st == ginf.OK, ginf.lib().ginf_last_error()
        torch.cuda.synchronize()
        assert torch.equal(got, want), (k, W, H, iters)


def test_noalloc_on_a_caller_stream(ginf):
    """The call runs on the caller's (non-default) stream: inputs written on
    that stream are seen, and the labels are complete when it returns."""
    import torch
    s = torch.cuda.Stream()
    for P, iters in (_problems()[0], _problems()[3], _problems()[6]):
        H, W = P.D.shape[1:]
        want = _want(ginf, P, iters, torch.from_numpy(P.D).cuda(), torch.from_numpy(P.V).cuda())
        torch.cuda.synchronize()
        with torch.cuda.stream(s):
            D = torch.from_numpy(P.D).pin_memory().to("cuda", non_blocking=True)
            V = torch.from_numpy(P.V).pin_memory().to("cuda", non_blocking=True)
            got = torch.zeros((H, W), dtype=torch.int32, device="cuda")
            for _ in range(2):
                st = _call_noalloc(ginf, D, V, P.model, iters, got, s.cuda_stream)
                assert st == ginf.OK, ginf.lib().ginf_last_error()
                assert torch.equal(got, want)


def test_noalloc_size_rule_at_its_boundary(ginf):
    """The largest grid the documented rule admits runs and equals
    ginf_decode_hbp; one more row is refused.  L = 5 pads to Lp = 8, so the
    limit is well below 48 MiB / (20 L) nodes."""
    import torch
    W, L = 1024, 5
    H = (SCRATCH_BYTES - 256) // (W * 20 * 8)
    assert _bytes_needed(W, H, L) <= SCRATCH_BYTES < _bytes_needed(W, H + 1, L)
    assert W * (H + 1) < SCRATCH_BYTES // (20 * L)   # what a per-L estimate would have admitted
    P = synth.random_problem(W, H, L, 41)
    D, V = torch.from_numpy(P.D).cuda(), torch.from_numpy(P.V).cuda()
    want = _want(ginf, P, 4, D, V)
    got = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    assert _call_noalloc(ginf, D, V, P.model, 4, got) == ginf.OK, ginf.lib().ginf_last_error()
    torch.cuda.synchronize()
    assert torch.equal(got, want)
    P2 = synth.random_problem(W, H + 1, L, 42)
    D2, V2 = torch.from_numpy(P2.D).cuda(), torch.from_numpy(P2.V).cuda()
    lab2 = torch.zeros((H + 1, W), dtype=torch.int32, device="cuda")
    assert _call_noalloc(ginf, D2, V2, P2.model, 4, lab2) == ginf.ERR_INVALID_ARGUMENT
    assert str(_bytes_needed(W, H + 1, L)).encode() in ginf.lib().ginf_last_error()


def test_noalloc_rejects_grids_above_its_fixed_size(ginf):
    import torch
    P = synth.random_problem(256, 256, 64, 1)   # 256*256*1280 B of records > 48 MiB
    D = torch.from_numpy(P.D).cuda()
    V = torch.from_numpy(P.V).cuda()
    lab = torch.zeros((256, 256), dtype=torch.int32, device="cuda")
    st = _call_noalloc(ginf, D, V, P.model, 4, lab)
    assert st == ginf.ERR_INVALID_ARGUMENT
    assert b"maximum" in ginf.lib().ginf_last_error()
    # host buffers are refused too: the entry point never copies
    st = _call_noalloc(ginf, P.D, P.V, P.model, 4, lab)
    assert st == ginf.ERR_INVALID_ARGUMENT
