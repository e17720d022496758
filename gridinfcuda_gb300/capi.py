"""ctypes binding of the C ABI (include/ginf_gb300.h) for numpy and torch buffers.

Host buffers are numpy arrays (or CPU tensors); device buffers are CUDA torch
tensors.  All buffers of one call must live in the same memory kind.  Every
function raises :class:`GinfError` on a non-zero ``ginf_status``.  The shared
library is loaded from the package directory; when it has not been built the
first call raises instead of computing anything elsewhere.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import synth

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libginf_gb300.so")

# Enumerations (values as in include/ginf_gb300.h).
OK, ERR_INVALID_ARGUMENT, ERR_UNSUPPORTED, ERR_CUDA, ERR_OUT_OF_MEMORY, ERR_TIMEOUT, ERR_NO_DEVICE = range(7)
F32, I32, F64 = 0, 1, 2
HOST, DEVICE = 0, 1
HOST_AUTO, HOST_COPY = 0, 1   # ginf_options.host_access
RULE_REFERENCE, RULE_STANDARD = 0, 1
STORE_NATIVE, STORE_F16 = 0, 1
DECODE_STALE, DECODE_FRESH = 0, 1
NORM_MEAN, NORM_MIN = 0, 1
EXPLICIT, POTTS, TRUNC_LINEAR, TRUNC_QUAD = synth.EXPLICIT, synth.POTTS, synth.TRUNC_LINEAR, synth.TRUNC_QUAD

_i32 = ctypes.c_int32
_p = ctypes.c_void_p


class Grid(ctypes.Structure):
    _fields_ = [("width", _i32), ("height", _i32), ("num_labels", _i32), ("cost_type", _i32),
                ("sm_model", _i32), ("memory", _i32), ("data_costs", _p), ("sm_costs", _p)]


class Options(ctypes.Structure):
    _fields_ = [("msg_rule", _i32), ("msg_store", _i32), ("decode", _i32), ("normalize", _i32),
                ("compute_type", _i32), ("tile_nodes", _i32), ("sweeps_per_launch", _i32), ("autotune", _i32),
                ("stream", _p), ("msgs_out", _p), ("host_access", _i32), ("stream_ordered", _i32),
                ("reserved", ctypes.c_int64 * 5)]


class Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("total_ms", "upload_ms", "prepare_ms", "sweep_ms", "level0_sweep_ms",
                                               "icm_ms", "energy_ms", "download_ms")] + \
               [(n, ctypes.c_int64) for n in ("kernel_launches", "level0_sweep_launches", "node_label_iters",
                                              "h2d_bytes", "d2h_bytes", "warm_start_used", "level0_alg_bytes")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class GinfError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"ginf status {status}: {message}")
        self.status = status


_lib = None


def lib():
    """The loaded libginf_gb300.so (raises if it was never built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with gridinfcuda_gb300.build()")
        L = ctypes.CDLL(LIB_PATH)
        L.ginf_version.restype = ctypes.c_char_p
        L.ginf_last_error.restype = ctypes.c_char_p
        L.ginf_default_options.argtypes = [ctypes.POINTER(Options)]
        L.ginf_workspace_create.argtypes = [ctypes.POINTER(_p)]
        L.ginf_workspace_destroy.argtypes = [_p]
        L.ginf_workspace_sync.argtypes = [_p]
        L.ginf_decode_hbp.argtypes = [_p, ctypes.POINTER(Grid), _i32, _i32, _p, ctypes.POINTER(Options),
                                      ctypes.POINTER(Stats)]
        L.ginf_decode_icm.argtypes = [_p, ctypes.POINTER(Grid), _p, _i32, _i32, _p, ctypes.POINTER(Options),
                                      ctypes.POINTER(Stats)]
        L.ginf_energy.argtypes = [_p, ctypes.POINTER(Grid), _p, ctypes.POINTER(ctypes.c_double),
                                  ctypes.POINTER(Options)]
        L.ginf_decode_alpha_beta.argtypes = [_p, ctypes.POINTER(Grid), _p, _i32, _p, ctypes.POINTER(Options),
                                             ctypes.POINTER(Stats)]
        L.ginf_solve.argtypes = [_p, ctypes.POINTER(Grid), _i32, _i32, _i32, _p, ctypes.POINTER(ctypes.c_double),
                                 ctypes.POINTER(Options), ctypes.POINTER(Stats)]
        L.ginf_stereo_costs.argtypes = [_i32, _i32, _i32, _i32, _p, _p, ctypes.c_float, ctypes.c_float, _p, _p]
        L.ginf_stereo_costs_u8.argtypes = [_i32, _i32, _i32, _i32, _p, _p, _i32, _p, _p]
        L.ginf_batch_create.argtypes = [ctypes.POINTER(_p), ctypes.POINTER(Grid), ctypes.POINTER(_p), _i32, _i32,
                                        ctypes.POINTER(Options)]
        L.ginf_batch_run.argtypes = [_p, _p, ctypes.POINTER(Stats)]
        L.ginf_batch_config.argtypes = [_p, ctypes.POINTER(_i32), ctypes.POINTER(_i32), ctypes.POINTER(_i32)]
        L.ginf_batch_destroy.argtypes = [_p]
        L.ginf_batch_enqueue.argtypes = [_p, _p]
        L.ginf_selftest_bounded_waits.argtypes = [ctypes.POINTER(_i32), ctypes.POINTER(_i32)]
        L.ginf_batch_sync.argtypes = [_p]
        L.ginf_decode_bp_batch.argtypes = [ctypes.POINTER(Grid), ctypes.POINTER(_p), _i32, _i32,
                                           ctypes.POINTER(Options), ctypes.POINTER(Stats)]
        L.ginf_warmnet_create.argtypes = [ctypes.POINTER(_p), _i32, _i32, ctypes.c_uint64]
        L.ginf_warmnet_load.argtypes = [ctypes.POINTER(_p), ctypes.c_char_p]
        L.ginf_warmnet_save.argtypes = [_p, ctypes.c_char_p]
        L.ginf_warmnet_destroy.argtypes = [_p]
        L.ginf_warmnet_num_params.argtypes = [_p, ctypes.POINTER(ctypes.c_int64)]
        L.ginf_warmnet_get_params.argtypes = [_p, _p]
        L.ginf_warmnet_set_params.argtypes = [_p, _p]
        L.ginf_warmnet_forward.argtypes = [_p, _p, _i32, _i32, _i32, _p, _p]
        L.ginf_warmnet_gradients.argtypes = [_p, _p, _p, _i32, _i32, _i32, ctypes.POINTER(ctypes.c_float), _p, _p]
        L.ginf_warmnet_train_step.argtypes = [_p, _p, _p, _i32, _i32, _i32, ctypes.c_float,
                                              ctypes.POINTER(ctypes.c_float), _p]
        L.ginf_hbp_level_state.argtypes = [_p, ctypes.POINTER(Grid), _i32, _i32, _i32, _i32, _p, _p,
                                           ctypes.POINTER(Options)]
        L.ginf_decode_hbp_learned.argtypes = [_p, ctypes.POINTER(Grid), _i32, _i32, _i32, _i32, _i32, _p, _p,
                                              ctypes.POINTER(Options), ctypes.POINTER(Stats)]
        L.ginf_decode_hbp_warm.argtypes = [_p, ctypes.POINTER(Grid), _i32, _i32, _i32, _i32, _i32, _p, _i32, _p,
                                           ctypes.POINTER(Options), ctypes.POINTER(Stats)]
        for name in ("ginf_decode_hbp", "ginf_decode_icm", "ginf_energy", "ginf_decode_alpha_beta",
                     "ginf_solve", "ginf_stereo_costs",
                     "ginf_stereo_costs_u8",
                     "ginf_workspace_create", "ginf_workspace_destroy", "ginf_batch_create", "ginf_batch_run",
                     "ginf_batch_config", "ginf_batch_destroy", "ginf_decode_bp_batch", "ginf_warmnet_create",
                     "ginf_warmnet_load", "ginf_warmnet_save", "ginf_warmnet_destroy", "ginf_warmnet_num_params",
                     "ginf_warmnet_get_params", "ginf_warmnet_set_params", "ginf_warmnet_forward",
                     "ginf_warmnet_gradients", "ginf_warmnet_train_step", "ginf_hbp_level_state",
                     "ginf_decode_hbp_learned", "ginf_decode_hbp_warm", "ginf_workspace_sync",
                     "ginf_batch_enqueue", "ginf_batch_sync", "ginf_selftest_bounded_waits"):
            getattr(L, name).restype = _i32
        _lib = L
    return _lib


def check(status: int):
    if status != OK:
        raise GinfError(status, lib().ginf_last_error().decode())


class Workspace:
    """Reusable device buffers (``ginf_workspace``); use one per thread."""

    def __init__(self):
        h = _p()
        check(lib().ginf_workspace_create(ctypes.byref(h)))
        self.handle = h

    def sync(self):
        """Waits for this workspace's stream-ordered calls; raises a device
        error any of them recorded."""
        check(lib().ginf_workspace_sync(self.handle))

    def close(self):
        if self.handle:
            lib().ginf_workspace_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _is_torch(a):
    return type(a).__module__.startswith("torch")


def _ptr(a):
    """(address, memory kind) of a numpy array or torch tensor."""
    if a is None:
        return None, None
    if _is_torch(a):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return a.data_ptr(), (DEVICE if a.is_cuda else HOST)
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data, HOST


def _dtype_code(a):
    name = str(a.dtype)
    if name.endswith("float32"):
        return F32
    if name.endswith("int32"):
        return I32
    raise ValueError(f"costs must be float32 or int32, got {a.dtype}")


def make_grid(D, V, model):
    """ginf_grid for label-planar costs D (L, H, W) and a flat L*L table V."""
    L, H, W = D.shape
    dp, dm = _ptr(D)
    vp, vm = _ptr(V)
    if dm != vm:
        raise ValueError("D and V must live in the same memory kind")
    if V.shape[-1] * (V.shape[0] if len(V.shape) == 2 else 1) != L * L:
        raise ValueError("V must hold L*L entries")
    return Grid(W, H, L, _dtype_code(D), int(model), dm, dp, vp)


def options(rule=RULE_REFERENCE, store=STORE_NATIVE, decode=DECODE_STALE, normalize=NORM_MEAN, compute_type=-1,
            tile_nodes=0, sweeps_per_launch=0, autotune=0, stream=None, msgs_out=None, host_access=0,
            stream_ordered=0):
    o = Options()
    lib().ginf_default_options(ctypes.byref(o))
    o.msg_rule, o.msg_store, o.decode, o.normalize = rule, store, decode, normalize
    o.compute_type, o.tile_nodes = compute_type, tile_nodes
    o.sweeps_per_launch, o.autotune = sweeps_per_launch, autotune
    o.stream = stream if stream is not None else None
    o.msgs_out = msgs_out
    o.host_access = host_access
    o.stream_ordered = stream_ordered
    return o


def _new_like(D, shape, dtype):
    if _is_torch(D):
        import torch
        tdt = {np.int32: torch.int32, np.float32: torch.float32, np.float64: torch.float64}[dtype]
        return torch.zeros(shape, dtype=tdt, device=D.device)
    return np.zeros(shape, dtype=dtype)


def _msg_dtype(D, compute_type):
    ct = _dtype_code(D) if compute_type < 0 else compute_type
    return {F32: np.float32, I32: np.int32, F64: np.float64}[ct]


def decode_hbp(D, V, model, levels, iters, labels=None, *, workspace=None, want_msgs=False, want_stats=False,
               **opt):
    """Hierarchical (levels > 1) or loopy BP; returns labels [, msgs] [, stats]."""
    L, H, W = D.shape
    g = make_grid(D, V, model)
    lab = labels if labels is not None else _new_like(D, (H, W), np.int32)
    msgs = _new_like(D, (H, W, 4, L), _msg_dtype(D, opt.get("compute_type", -1))) if want_msgs else None
    o = options(msgs_out=_ptr(msgs)[0] if msgs is not None else None, **opt)
    st = Stats()
    ws = workspace.handle if workspace is not None else None
    check(lib().ginf_decode_hbp(ws, ctypes.byref(g), levels, iters, _ptr(lab)[0], ctypes.byref(o),
                                ctypes.byref(st) if want_stats else None))
    out = [lab]
    if want_msgs:
        out.append(msgs)
    if want_stats:
        out.append(st.as_dict())
    return out[0] if len(out) == 1 else tuple(out)


def decode_icm(D, V, model, initial, iters, asynchronous=False, *, workspace=None, want_stats=False, **opt):
    L, H, W = D.shape
    g = make_grid(D, V, model)
    res = _new_like(D, (H, W), np.int32)
    o = options(**opt)
    st = Stats()
    ws = workspace.handle if workspace is not None else None
    check(lib().ginf_decode_icm(ws, ctypes.byref(g), _ptr(initial)[0], iters, int(asynchronous), _ptr(res)[0],
                                ctypes.byref(o), ctypes.byref(st) if want_stats else None))
    return (res, st.as_dict()) if want_stats else res


def decode_alpha_beta(D, V, model, initial, iters, *, workspace=None, want_stats=False, **opt):
    """Alpha-beta swap (int32 grids); returns the labelling [, stats]."""
    L, H, W = D.shape
    g = make_grid(D, V, model)
    out = _new_like(D, (H, W), np.int32)
    init = initial if _ptr(initial)[1] == _ptr(D)[1] else None
    if init is None:
        raise ValueError("initial must live in the same memory kind as D")
    o = options(**opt)
    st = Stats()
    ws = workspace.handle if workspace is not None else None
    check(lib().ginf_decode_alpha_beta(ws, ctypes.byref(g), _ptr(init)[0], iters, _ptr(out)[0], ctypes.byref(o),
                                       ctypes.byref(st) if want_stats else None))
    return (out, st.as_dict()) if want_stats else out


def energy(D, V, model, labels, *, workspace=None):
    g = make_grid(D, V, model)
    e = ctypes.c_double()
    ws = workspace.handle if workspace is not None else None
    check(lib().ginf_energy(ws, ctypes.byref(g), _ptr(labels)[0], ctypes.byref(e), None))
    return e.value


def solve(D, V, model, levels, iters, icm_iters, labels=None, *, workspace=None, want_stats=False, **opt):
    """HBP + Jacobi ICM + FP64 energy in one call; returns (labels, energy[, stats])."""
    L, H, W = D.shape
    g = make_grid(D, V, model)
    lab = labels if labels is not None else _new_like(D, (H, W), np.int32)
    o = options(**opt)
    st = Stats()
    e = ctypes.c_double()
    ws = workspace.handle if workspace is not None else None
    check(lib().ginf_solve(ws, ctypes.byref(g), levels, iters, icm_iters, _ptr(lab)[0], ctypes.byref(e),
                           ctypes.byref(o), ctypes.byref(st) if want_stats else None))
    return (lab, e.value, st.as_dict()) if want_stats else (lab, e.value)


def solve_async(D, V, model, levels, iters, icm_iters, labels, energy, workspace, stream, **opt):
    """Stream-ordered ginf_solve: enqueues on `stream` (a cudaStream_t handle)
    and returns.  `labels` receives the result and the ctypes.c_double
    `energy` the FP64 energy once the stream (or workspace.sync()) is done;
    D, V, labels and energy must stay alive and unchanged until then."""
    g = make_grid(D, V, model)
    o = options(stream=stream, stream_ordered=1, **opt)
    check(lib().ginf_solve(workspace.handle, ctypes.byref(g), levels, iters, icm_iters, _ptr(labels)[0],
                           ctypes.byref(energy), ctypes.byref(o), None))


def stereo_costs(left, right, L, coef, cap, out, stream=None):
    """Device cost volume (L, H, W) float32 into the CUDA tensor ``out``."""
    H, W = left.shape
    lp, lm = _ptr(left)
    rp, _ = _ptr(right)
    op, om = _ptr(out)
    if om != DEVICE:
        raise ValueError("out must be a CUDA tensor")
    check(lib().ginf_stereo_costs(W, H, L, lm, lp, rp, coef, cap, op, stream))
    return out


def stereo_costs_u8(left, right, L, cap, out, stream=None):
    """The reference example's integer cost volume (examples/stereo/stereo.cc:28-34)
    from 8-bit grey images into the CUDA int32 tensor ``out`` (L, H, W)."""
    H, W = left.shape
    lp, lm = _ptr(left)
    rp, _ = _ptr(right)
    op, om = _ptr(out)
    if om != DEVICE:
        raise ValueError("out must be a CUDA tensor")
    check(lib().ginf_stereo_costs_u8(W, H, L, lm, lp, rp, cap, op, stream))
    return out


class Batch:
    """A captured batch solve (``ginf_batch``): grids are (D, V, model) with
    CUDA tensors, labels CUDA int32 tensors (H, W); run() replays the solve."""

    def __init__(self, problems, labels, iters, **opt):
        self._keep = (problems, labels)
        n = len(problems)
        self._grids = (Grid * n)(*[make_grid(D, V, m) for (D, V, m) in problems])
        self._labs = (_p * n)(*[_ptr(l)[0] for l in labels])
        self._opt = options(**opt)
        h = _p()
        check(lib().ginf_batch_create(ctypes.byref(h), self._grids, self._labs, n, iters, ctypes.byref(self._opt)))
        self.handle = h

    def run(self, stream=None, want_stats=False):
        st = Stats()
        check(lib().ginf_batch_run(self.handle, stream, ctypes.byref(st) if want_stats else None))
        return st.as_dict() if want_stats else None

    def enqueue(self, stream=None):
        """Stream-ordered replay (returns at once; see sync())."""
        check(lib().ginf_batch_enqueue(self.handle, stream))

    def sync(self):
        """Waits for the stream-ordered replays; raises a device error they recorded."""
        check(lib().ginf_batch_sync(self.handle))

    def config(self):
        a, b, c = _i32(), _i32(), _i32()
        check(lib().ginf_batch_config(self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"tile_nodes": a.value, "sweeps_per_launch": b.value, "tuned_now": bool(c.value)}

    def close(self):
        if getattr(self, "handle", None):
            lib().ginf_batch_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class WarmNet:
    """The warm-start network (``ginf_warmnet``).  Tensors are CUDA FP32,
    shaped (n, h, w, L)."""

    def __init__(self, num_labels=64, hidden=32, seed=0, path=None):
        h = _p()
        if path is not None:
            check(lib().ginf_warmnet_load(ctypes.byref(h), str(path).encode()))
        else:
            check(lib().ginf_warmnet_create(ctypes.byref(h), num_labels, hidden, seed))
        self.handle = h

    def num_params(self):
        n = ctypes.c_int64()
        check(lib().ginf_warmnet_num_params(self.handle, ctypes.byref(n)))
        return n.value

    def get_params(self):
        out = np.zeros(self.num_params(), np.float32)
        check(lib().ginf_warmnet_get_params(self.handle, out.ctypes.data))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        check(lib().ginf_warmnet_set_params(self.handle, p.ctypes.data))

    def forward(self, x, stream=None):
        import torch
        n, h, w, _ = x.shape
        y = torch.empty_like(x)
        check(lib().ginf_warmnet_forward(self.handle, x.data_ptr(), n, h, w, y.data_ptr(), stream))
        return y

    def gradients(self, x, target, stream=None):
        n, h, w, _ = x.shape
        loss = ctypes.c_float()
        g = np.zeros(self.num_params(), np.float32)
        check(lib().ginf_warmnet_gradients(self.handle, x.data_ptr(), target.data_ptr(), n, h, w, ctypes.byref(loss),
                                           g.ctypes.data, stream))
        return loss.value, g

    def train_step(self, x, target, lr, stream=None):
        n, h, w, _ = x.shape
        loss = ctypes.c_float()
        check(lib().ginf_warmnet_train_step(self.handle, x.data_ptr(), target.data_ptr(), n, h, w, lr,
                                            ctypes.byref(loss), stream))
        return loss.value

    def save(self, path):
        check(lib().ginf_warmnet_save(self.handle, str(path).encode()))

    def close(self):
        if getattr(self, "handle", None):
            lib().ginf_warmnet_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def level_state(D, V, model, levels, iters, level, want_beliefs=True, target=0, workspace=None, **opt):
    """(x, target) of pyramid level `level` as CUDA FP32 (H_t, W_t, L); target
    0 = the level's own beliefs, 1 = projected finest-level messages."""
    import torch
    L, H, W = D.shape
    Wt, Ht = W, H
    for _ in range(level):
        Wt, Ht = (Wt + 1) // 2, (Ht + 1) // 2
    x = torch.empty((Ht, Wt, L), dtype=torch.float32, device=D.device)
    b = torch.empty_like(x) if want_beliefs else None
    g = make_grid(D, V, model)
    o = options(**opt)
    ws = workspace.handle if workspace is not None else None
    check(lib().ginf_hbp_level_state(ws, ctypes.byref(g), levels, iters, level, target, x.data_ptr(),
                                     b.data_ptr() if b is not None else None, ctypes.byref(o)))
    return x, b


def decode_hbp_learned(D, V, model, levels, iters, warm_level, net, labels=None, *, warm_iters=None, mid_iters=-1,
                       workspace=None, want_stats=False, **opt):
    """Hierarchical BP with level `warm_level` seeded by the network `net`
    (warm_iters half-sweeps there, default `iters`; mid_iters at the levels
    between it and level 0, default `iters`) and the cold fallback."""
    L, H, W = D.shape
    g = make_grid(D, V, model)
    lab = labels if labels is not None else _new_like(D, (H, W), np.int32)
    o = options(**opt)
    st = Stats()
    ws = workspace.handle if workspace is not None else None
    wi = iters if warm_iters is None else warm_iters
    check(lib().ginf_decode_hbp_learned(ws, ctypes.byref(g), levels, iters, warm_level, wi, mid_iters, net.handle,
                                        _ptr(lab)[0], ctypes.byref(o), ctypes.byref(st) if want_stats else None))
    return (lab, st.as_dict()) if want_stats else lab


def decode_hbp_warm(D, V, model, levels, iters, warm_level, prediction, labels=None, *, warm_iters=None,
                    mid_iters=-1, fallback=True, workspace=None, want_stats=False, **opt):
    """Hierarchical BP with level `warm_level` seeded from `prediction`, a CUDA
    FP32 tensor (H_t, W_t, L) on the warm-start network's output scale."""
    import torch
    L, H, W = D.shape
    g = make_grid(D, V, model)
    lab = labels if labels is not None else _new_like(D, (H, W), np.int32)
    o = options(**opt)
    st = Stats()
    ws = workspace.handle if workspace is not None else None
    wi = iters if warm_iters is None else warm_iters
    Wt, Ht = W, H
    for _ in range(warm_level):
        Wt, Ht = (Wt + 1) // 2, (Ht + 1) // 2
    if tuple(prediction.shape) != (Ht, Wt, L) or prediction.dtype != torch.float32 or not prediction.is_cuda:
        raise ValueError(f"prediction must be a CUDA float32 tensor of shape {(Ht, Wt, L)}")
    pred = prediction.contiguous()
    check(lib().ginf_decode_hbp_warm(ws, ctypes.byref(g), levels, iters, warm_level, wi, mid_iters, pred.data_ptr(),
                                     1 if fallback else 0, _ptr(lab)[0], ctypes.byref(o),
                                     ctypes.byref(st) if want_stats else None))
    return (lab, st.as_dict()) if want_stats else lab


def selftest_bounded_waits():
    """(mbarrier status, grid-barrier status) after the library's bounded
    device waits were run into their time limit on purpose (about 2 s each)."""
    a, b = _i32(), _i32()
    check(lib().ginf_selftest_bounded_waits(ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


def version() -> str:
    return lib().ginf_version().decode()
