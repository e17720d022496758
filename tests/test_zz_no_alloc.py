"""ginf_decode_bp_noalloc: loopy BP for callers that cannot allocate device
memory (a real-time loop that cannot afford cudaMalloc's synchronisation, or
a plugin whose host application owns all device memory).  It keeps its
working set in a fixed 48 MiB array inside the library instead of a
workspace.  Its labels must equal those of ginf_decode_hbp (one level) -- the
same bit-exact standard as every other FP32 / int32 test -- on consecutive
calls that reuse the shared array; oversized grids are refused, not run.

This file is collected last on purpose, and passes whether it runs alone in
a fresh process or after the other tests."""
import ctypes

import numpy as np
import pytest

from gridinfcuda_gb300 import synth

pytestmark = pytest.mark.gpu


def _call_noalloc(capi, D, V, model, iters, labels, stream=None):
    fn = capi.lib().ginf_decode_bp_noalloc
    fn.argtypes = [ctypes.POINTER(capi.Grid), ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int32
    g = capi.make_grid(D, V, model)
    return fn(ctypes.byref(g), iters, labels.data_ptr(), stream)


def test_noalloc_matches_decode_hbp_on_consecutive_calls(ginf):
    import torch
    problems = [
        (synth.workload_plain_bp(), 50),                                         # 384x288x16, 35 MB of records
        (synth.random_problem(90, 70, 32, 4, dtype=np.int32, scale=10, trunc=20, cost_max=40), 7),
        (synth.random_problem(33, 17, 5, 6), 1),
        (synth.workload_plain_bp(), 50),
    ]
    for P, iters in problems:
        D = torch.from_numpy(P.D).cuda()
        V = torch.from_numpy(P.V).cuda()
        H, W = P.D.shape[1:]
        want = torch.zeros((H, W), dtype=torch.int32, device="cuda")
        ginf.decode_hbp(D, V, P.model, 1, iters, labels=want)
        got = torch.full((H, W), 0, dtype=torch.int32, device="cuda")
        st = _call_noalloc(ginf, D, V, P.model, iters, got)
        assert st == ginf.OK, ginf.lib().ginf_last_error()
        torch.cuda.synchronize()
        assert torch.equal(got, want), (W, H, iters)


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
