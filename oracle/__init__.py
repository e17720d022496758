"""ctypes bindings for the CPU oracle (and the compiled reference, when built).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline legs; the product package never imports it.

Two libraries:
  * ``oracle/_build/libginf_oracle.so`` -- the C restatement (ginf_oracle.c),
    built anywhere by ``make -C oracle``;
  * ``oracle/_ref/libginf_ref.so`` -- the reference's own CPU code behind
    ref_bridge.cc, built by ``make -C oracle ref`` only where the reference
    checkout exists.  Tests that need it skip when it is absent.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libginf_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libginf_ref.so")


def _reference_dir() -> str:
    """Where the reference checkout is looked for: $GINF_REFERENCE, else the
    default that oracle/Makefile holds (the one recipe naming a location)."""
    env = os.environ.get("GINF_REFERENCE")
    if env:
        return env
    try:
        r = subprocess.run(["make", "-s", "-C", HERE, "ref-dir"], capture_output=True, text=True, timeout=30)
        return r.stdout.strip()
    except Exception:
        return ""


REF_SRC = _reference_dir()

_i = ctypes.c_int
_p = ctypes.c_void_p
_f = ctypes.c_float
_d = ctypes.c_double


def build(with_ref: bool | None = None) -> None:
    """Compile the oracle; also the reference bridge when its sources exist."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if with_ref is None:
        with_ref = bool(REF_SRC) and os.path.isdir(os.path.join(REF_SRC, "src"))
    if with_ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}"], check=True)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _c32(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(with_ref=False)
        L = ctypes.CDLL(ORACLE_SO)
        for name in ("orc_hbp_f32", "orc_hbp_i32"):
            getattr(L, name).argtypes = [_i, _i, _i, _p, _p, _i, _i, _i, _p, _p, _i]
            getattr(L, name).restype = _i
        L.orc_hbp_f64_std.argtypes = [_i, _i, _i, _p, _p, _i, _i, _i, _i, _i, _p, _p, _i]
        L.orc_hbp_f64_std.restype = _i
        for name in ("orc_icm_sync_f32", "orc_icm_sync_i32"):
            getattr(L, name).argtypes = [_i, _i, _i, _p, _p, _p, _i, _p, _i]
            getattr(L, name).restype = _i
        for name in ("orc_icm_async_f32", "orc_icm_async_i32"):
            getattr(L, name).argtypes = [_i, _i, _i, _p, _p, _p, _i, _p]
            getattr(L, name).restype = _i
        L.orc_energy_f32_seq.argtypes = [_i, _i, _i, _p, _p, _p]
        L.orc_energy_f32_seq.restype = _f
        L.orc_energy_i32_seq.argtypes = [_i, _i, _i, _p, _p, _p]
        L.orc_energy_i32_seq.restype = ctypes.c_int32
        L.orc_energy_f64.argtypes = [_i, _i, _i, _p, _p, _p]
        L.orc_energy_f64.restype = _d
        L.orc_energy_i32_f64.argtypes = [_i, _i, _i, _p, _p, _p]
        L.orc_energy_i32_f64.restype = _d
        L.orc_alpha_beta_i32.argtypes = [_i, _i, _i, _p, _p, _p, _i, _p]
        L.orc_alpha_beta_i32.restype = _i
        L.orc_pyramid_f32.argtypes = [_i, _i, _i, _p, _p]
        L.orc_send_linear_f32.argtypes = [_i, _p, _p, _f, _f, _p]
        L.orc_dt_quad_f64.argtypes = [_i, _p, _d, _p]
        L.orc_minconv_brute_f64.argtypes = [_i, _p, _p, _p]
        _lib = L
    return _lib


def ref():
    """The compiled reference bridge, or None where it was not built."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            return None
        R = ctypes.CDLL(REF_SO)
        R.ref_table_f32.argtypes = [_i, _i, _f, _f, _p, _p]
        R.ref_table_i32.argtypes = [_i, _i, _i, _i, _p, _p]
        R.ref_hbp_f32.argtypes = [_i, _i, _i, _p, _i, _f, _f, _p, _i, _i, _p]
        R.ref_hbp_i32.argtypes = [_i, _i, _i, _p, _i, _i, _i, _p, _i, _i, _p]
        R.ref_bp_msgs_f32.argtypes = [_i, _i, _i, _p, _i, _f, _f, _p, _i, _p]
        R.ref_bp_msgs_i32.argtypes = [_i, _i, _i, _p, _i, _i, _i, _p, _i, _p]
        R.ref_icm_f32.argtypes = [_i, _i, _i, _p, _i, _f, _f, _p, _p, _i, _p, _i]
        R.ref_icm_i32.argtypes = [_i, _i, _i, _p, _i, _i, _i, _p, _p, _i, _p, _i]
        R.ref_energy_f32.argtypes = [_i, _i, _i, _p, _i, _f, _f, _p, _p]
        R.ref_energy_f32.restype = _f
        R.ref_energy_i32.argtypes = [_i, _i, _i, _p, _i, _i, _i, _p, _p]
        R.ref_energy_i32.restype = ctypes.c_int32
        R.ref_alpha_beta_i32.argtypes = [_i, _i, _i, _p, _i, _i, _i, _p, _p, _i, _p]
        _ref = R
    return _ref


def _dims(D):
    L, H, W = D.shape
    return W, H, L


def _kind(D):
    return "i32" if D.dtype == np.int32 else "f32"


# --------------------------------------------------------------------------
# Oracle (C restatement)

def hbp(D, V, model, levels, iters, labels=None, want_msgs=False, nthreads=0):
    """Reference-semantics HBP/BP; returns (labels, msgs or None)."""
    k = _kind(D)
    dt = np.int32 if k == "i32" else np.float32
    D = _c32(D, dt)
    V = _c32(V, dt)
    W, H, L = _dims(D)
    lab = np.zeros((H, W), np.int32) if labels is None else np.array(labels, dtype=np.int32, copy=True)
    msgs = np.zeros((H, W, 4, L), dt) if want_msgs else None
    rc = getattr(lib(), "orc_hbp_" + k)(W, H, L, _ptr(D), _ptr(V), model, levels, iters, _ptr(lab), _ptr(msgs),
                                        nthreads)
    assert rc == 0
    return lab, msgs


def hbp_f64_std(D, V, model, levels, iters, decode=0, norm=0, labels=None, want_msgs=False, nthreads=0):
    D = _c32(D, np.float32)
    V = _c32(V, np.float32)
    W, H, L = _dims(D)
    lab = np.zeros((H, W), np.int32) if labels is None else np.array(labels, dtype=np.int32, copy=True)
    msgs = np.zeros((H, W, 4, L), np.float64) if want_msgs else None
    rc = lib().orc_hbp_f64_std(W, H, L, _ptr(D), _ptr(V), model, levels, iters, decode, norm, _ptr(lab),
                               _ptr(msgs), nthreads)
    assert rc == 0
    return lab, msgs


def icm(D, V, initial, iters, asynchronous=False, nthreads=0):
    k = _kind(D)
    dt = np.int32 if k == "i32" else np.float32
    D = _c32(D, dt)
    V = _c32(V, dt)
    W, H, L = _dims(D)
    init = _c32(initial, np.int32)
    out = np.zeros((H, W), np.int32)
    if asynchronous:
        rc = getattr(lib(), "orc_icm_async_" + k)(W, H, L, _ptr(D), _ptr(V), _ptr(init), iters, _ptr(out))
    else:
        rc = getattr(lib(), "orc_icm_sync_" + k)(W, H, L, _ptr(D), _ptr(V), _ptr(init), iters, _ptr(out), nthreads)
    assert rc == 0
    return out


def energy(D, V, labels, exact_type=False):
    """FP64 energy (default), or the reference's own-type raster accumulation."""
    k = _kind(D)
    dt = np.int32 if k == "i32" else np.float32
    D = _c32(D, dt)
    V = _c32(V, dt)
    W, H, L = _dims(D)
    f = _c32(labels, np.int32)
    if exact_type:
        fn = lib().orc_energy_f32_seq if k == "f32" else lib().orc_energy_i32_seq
    else:
        fn = lib().orc_energy_f64 if k == "f32" else lib().orc_energy_i32_f64
    return fn(W, H, L, _ptr(D), _ptr(V), _ptr(f))


def pyramid(D):
    D = _c32(D, np.float32)
    W, H, L = _dims(D)
    out = np.zeros((L, (H + 1) // 2, (W + 1) // 2), np.float32)
    lib().orc_pyramid_f32(W, H, L, _ptr(D), _ptr(out))
    return out


def dt_quad(f, s):
    f = _c32(f, np.float64)
    out = np.zeros_like(f)
    lib().orc_dt_quad_f64(len(f), _ptr(f), s, _ptr(out))
    return out


def minconv_brute(f, V):
    f = _c32(f, np.float64)
    V = _c32(V, np.float64)
    out = np.zeros_like(f)
    lib().orc_minconv_brute_f64(len(f), _ptr(f), _ptr(V), _ptr(out))
    return out


# --------------------------------------------------------------------------
# The reference itself (only where oracle/_ref was built)

def ref_table(L, model, scale, d, V=None, dtype=np.float32):
    R = ref()
    out = np.zeros(L * L, dtype)
    Vin = _c32(V if V is not None else np.zeros(L * L), dtype)
    fn = R.ref_table_i32 if dtype == np.int32 else R.ref_table_f32
    fn(L, model, scale, d, _ptr(Vin), _ptr(out))
    return out


def ref_hbp(D, V, model, scale, d, levels, iters, labels=None):
    R = ref()
    k = _kind(D)
    dt = np.int32 if k == "i32" else np.float32
    D = _c32(D, dt)
    V = _c32(V, dt)
    W, H, L = _dims(D)
    lab = np.zeros((H, W), np.int32) if labels is None else np.array(labels, dtype=np.int32, copy=True)
    getattr(R, "ref_hbp_" + k)(W, H, L, _ptr(D), model, scale, d, _ptr(V), levels, iters, _ptr(lab))
    return lab


def ref_bp_msgs(D, V, model, scale, d, iters):
    R = ref()
    k = _kind(D)
    dt = np.int32 if k == "i32" else np.float32
    D = _c32(D, dt)
    V = _c32(V, dt)
    W, H, L = _dims(D)
    out = np.zeros((H, W, 4, L), dt)
    getattr(R, "ref_bp_msgs_" + k)(W, H, L, _ptr(D), model, scale, d, _ptr(V), iters, _ptr(out))
    return out


def ref_icm(D, V, model, scale, d, initial, iters, asynchronous=False):
    R = ref()
    k = _kind(D)
    dt = np.int32 if k == "i32" else np.float32
    D = _c32(D, dt)
    V = _c32(V, dt)
    W, H, L = _dims(D)
    out = np.zeros((H, W), np.int32)
    getattr(R, "ref_icm_" + k)(W, H, L, _ptr(D), model, scale, d, _ptr(V), _ptr(_c32(initial, np.int32)), iters,
                               _ptr(out), int(asynchronous))
    return out


def ref_alpha_beta(D, V, model, scale, d, initial, iters):
    """The reference's decodeAlphaBeta<int> (src/graphcut.cc:197-279)."""
    R = ref()
    D = _c32(D, np.int32)
    V = _c32(V, np.int32)
    W, H, L = _dims(D)
    out = np.zeros((H, W), np.int32)
    R.ref_alpha_beta_i32(W, H, L, _ptr(D), model, int(scale), int(d), _ptr(V), _ptr(_c32(initial, np.int32)),
                         iters, _ptr(out))
    return out


def alpha_beta(D, V, initial, iters):
    """Alpha-beta swap restated in C (int grids; src/graphcut.cc:197-279)."""
    D = _c32(D, np.int32)
    V = _c32(V, np.int32)
    W, H, L = _dims(D)
    out = np.zeros((H, W), np.int32)
    rc = lib().orc_alpha_beta_i32(W, H, L, _ptr(D), _ptr(V), _ptr(_c32(initial, np.int32)), iters, _ptr(out))
    assert rc == 0
    return out


def ref_energy(D, V, model, scale, d, labels):
    R = ref()
    k = _kind(D)
    dt = np.int32 if k == "i32" else np.float32
    D = _c32(D, dt)
    V = _c32(V, dt)
    W, H, L = _dims(D)
    return getattr(R, "ref_energy_" + k)(W, H, L, _ptr(D), model, scale, d, _ptr(V), _ptr(_c32(labels, np.int32)))
