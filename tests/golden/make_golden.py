"""Writes the golden fixtures of tests/golden/ from the reference's own CPU code.

Run where the reference checkout exists (``make -C oracle ref`` builds
oracle/_ref/libginf_ref.so from its unmodified src/{grid,matrix,bp,icm}.cc):

    python tests/golden/make_golden.py [--skip-large]

Every input is regenerated from a seed by gridinfcuda_gb300.synth, so the
fixtures hold only outputs (labels, messages, energies) plus a SHA-256 of
each input cost volume, which pins the generator itself across machines.
Large outputs are stored as SHA-256 digests; small ones as arrays
(golden_arrays.npz).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from gridinfcuda_gb300 import synth  # noqa: E402
from png_grey import grey, stereo_costs_u8  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


# Small single-level cases: (name, W, H, L, seed, model, scale, trunc, dtype, iters)
SMALL_BP = [
    ("lin_17x13_L16", 17, 13, 16, 0, synth.TRUNC_LINEAR, 1.0, 1.7, "f32", 9),
    ("lin_33x21_L17", 33, 21, 17, 1, synth.TRUNC_LINEAR, 0.5, 2.5, "f32", 12),
    ("lin_9x7_L3", 9, 7, 3, 2, synth.TRUNC_LINEAR, 1.0, 1.7, "f32", 5),
    ("potts_40x30_L8", 40, 30, 8, 3, synth.POTTS, 0.8, 0.0, "f32", 10),
    ("lin_64x48_L64", 64, 48, 64, 4, synth.TRUNC_LINEAR, 1.0, 4.0, "f32", 8),
    ("lin_31x29_L128", 31, 29, 128, 5, synth.TRUNC_LINEAR, 0.25, 6.0, "f32", 6),
    ("quadref_19x15_L8", 19, 15, 8, 6, synth.TRUNC_QUAD, 1.0, 4.0, "f32", 4),
    ("explicit_15x11_L5", 15, 11, 5, 7, synth.EXPLICIT, 0.0, 0.0, "f32", 4),
    ("int_lin_45x33_L16", 45, 33, 16, 8, synth.TRUNC_LINEAR, 10, 20, "i32", 11),
    ("int_potts_23x19_L7", 23, 19, 7, 9, synth.POTTS, 3, 0, "i32", 6),
    ("lin_3x3_L4", 3, 3, 4, 10, synth.TRUNC_LINEAR, 1.0, 1.7, "f32", 3),
    ("lin_1x5_L4", 1, 5, 4, 11, synth.TRUNC_LINEAR, 1.0, 1.7, "f32", 3),
    ("lin_iters1_20x14_L16", 20, 14, 16, 12, synth.TRUNC_LINEAR, 1.0, 1.7, "f32", 1),
    ("lin_iters0_20x14_L16", 20, 14, 16, 13, synth.TRUNC_LINEAR, 1.0, 1.7, "f32", 0),
]

# Hierarchical cases: (name, W, H, L, seed, model, scale, trunc, dtype, levels, iters)
SMALL_HBP = [
    ("hbp_97x71_L16_3x6", 97, 71, 16, 20, synth.TRUNC_LINEAR, 1.0, 1.7, "f32", 3, 6),
    ("hbp_60x44_L32_4x3", 60, 44, 32, 21, synth.TRUNC_LINEAR, 1.0, 3.0, "f32", 4, 3),
    ("hbp_33x29_L16_5x1", 33, 29, 16, 22, synth.TRUNC_LINEAR, 1.0, 1.7, "f32", 5, 1),
    ("hbp_int_50x38_L16_3x5", 50, 38, 16, 23, synth.TRUNC_LINEAR, 10, 20, "i32", 3, 5),
    ("hbp_41x33_L24_6x4", 41, 33, 24, 24, synth.POTTS, 1.5, 0.0, "f32", 6, 4),
]


def small_problem(W, H, L, seed, model, scale, trunc, dtype):
    dt = np.int32 if dtype == "i32" else np.float32
    cmax = 20.0 if dtype == "i32" else 4.0
    return synth.random_problem(W, H, L, seed, model=model, scale=scale, trunc=trunc, dtype=dt, cost_max=cmax)


def initial_labels(W, H, L, seed):
    rng = synth.Rng(seed, 99)
    return rng.integers(0, L - 1, W * H).reshape(H, W).astype(np.int32)


# Alpha-beta swap cases (int grids): (name, W, H, L, seed, model, scale, trunc, iters)
ALPHA_BETA = [
    ("ab_lin_23x17_L5", 23, 17, 5, 30, synth.TRUNC_LINEAR, 2, 6, 3),
    ("ab_potts_31x19_L4", 31, 19, 4, 31, synth.POTTS, 3, 0, 3),
    ("ab_quad_20x26_L6", 20, 26, 6, 32, synth.TRUNC_QUAD, 1, 9, 2),
    ("ab_explicit_15x12_L5", 15, 12, 5, 33, synth.EXPLICIT, 0, 0, 2),
    ("ab_lin_1x9_L3", 1, 9, 3, 34, synth.TRUNC_LINEAR, 1, 2, 2),
    ("ab_lin_64x48_L8", 64, 48, 8, 35, synth.TRUNC_LINEAR, 10, 20, 2),
]


def alpha_beta_cases(gold, arrays):
    """The reference's own decodeAlphaBeta<int> (src/graphcut.cc:197-279) on
    seeded int grids from a seeded initial labelling."""
    for (name, W, H, L, seed, model, scale, trunc, iters) in ALPHA_BETA:
        P = synth.random_problem(W, H, L, seed, model=model, scale=scale, trunc=trunc, dtype=np.int32, cost_max=20)
        init = initial_labels(W, H, L, seed)
        lab = oracle.ref_alpha_beta(P.D, P.V, model, scale, trunc, init, iters)
        gold["cases"][name] = dict(kind="alpha_beta", W=W, H=H, L=L, seed=seed, model=model, scale=scale,
                                   trunc=trunc, dtype="i32", iters=iters, cost_sha=sha(P.D), table_sha=sha(P.V),
                                   energy_ref_type=int(oracle.ref_energy(P.D, P.V, model, scale, trunc, lab)))
        arrays[name + "/init"] = init.astype(np.int16)
        arrays[name + "/labels"] = lab.astype(np.int16)
        print("case", name, flush=True)


def stereo_png_case(gold, arrays):
    """The reference example end to end (examples/stereo/stereo.cc:16-43):
    its own stereo pair as grey images, Grid<int> with L = 16 and costs
    min(|left(x) - right(x-k)|, 20) for x >= L-1, TruncLinear(10, 20), 30
    iterations of loopy BP by the reference's CPU code.  The grey images are
    stored (the GPU test has no reference checkout), the labels both as an
    array and as a SHA-256."""
    path = os.path.join(oracle.REF_SRC, "examples", "stereo")
    left, right = grey(os.path.join(path, "left.png")), grey(os.path.join(path, "right.png"))
    H, W = left.shape
    L = 16
    D = stereo_costs_u8(left, right, L, 20)
    V = synth.sm_table(L, synth.TRUNC_LINEAR, 10, 20, dtype=np.int32)
    lab = oracle.ref_hbp(D, V, synth.TRUNC_LINEAR, 10, 20, 1, 30)
    gold["cases"]["stereo_png_384x288_L16"] = dict(
        kind="stereo_png", W=W, H=H, L=L, levels=1, iters=30, cap=20, scale=10, trunc=20, cost_sha=sha(D),
        table_sha=sha(V), labels_sha=sha(lab), energy_ref_type=float(oracle.ref_energy(D, V, synth.TRUNC_LINEAR,
                                                                                         10, 20, lab)),
        source="examples/stereo/left.png, right.png (grey: (299 R + 587 G + 114 B + 500) / 1000)")
    arrays["stereo_png_384x288_L16/left"] = left
    arrays["stereo_png_384x288_L16/right"] = right
    arrays["stereo_png_384x288_L16/labels"] = lab.astype(np.int8)
    print("stereo PNG case done", flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--skip-large", action="store_true", help="skip the 1920x1080 reference HBP run (minutes)")
    ap.add_argument("--only-stereo-png", action="store_true",
                    help="keep every existing fixture and (re)write only the stereo PNG case")
    ap.add_argument("--only-alpha-beta", action="store_true",
                    help="keep every existing fixture and (re)write only the alpha-beta swap cases")
    args = ap.parse_args()
    oracle.build(with_ref=True)
    assert oracle.ref() is not None, "the reference bridge did not build"
    if args.only_stereo_png or args.only_alpha_beta:
        with open(os.path.join(HERE, "golden.json")) as f:
            gold = json.load(f)
        arrays = dict(np.load(os.path.join(HERE, "golden_arrays.npz")))
        if args.only_stereo_png:
            stereo_png_case(gold, arrays)
        if args.only_alpha_beta:
            alpha_beta_cases(gold, arrays)
        write(gold, arrays)
        return
    gold = {"generator": "tests/golden/make_golden.py", "cases": {}}
    arrays = {}
    stereo_png_case(gold, arrays)
    alpha_beta_cases(gold, arrays)

    for (name, W, H, L, seed, model, scale, trunc, dtype, iters) in SMALL_BP:
        P = small_problem(W, H, L, seed, model, scale, trunc, dtype)
        init = initial_labels(W, H, L, seed)
        lab = oracle.ref_hbp(P.D, P.V, model, scale, trunc, 1, iters, labels=init)
        msgs = oracle.ref_bp_msgs(P.D, P.V, model, scale, trunc, iters)
        e_ref = float(oracle.ref_energy(P.D, P.V, model, scale, trunc, lab))
        icm_s = oracle.ref_icm(P.D, P.V, model, scale, trunc, lab, 3)
        icm_a = oracle.ref_icm(P.D, P.V, model, scale, trunc, lab, 2, asynchronous=True)
        gold["cases"][name] = dict(kind="bp", W=W, H=H, L=L, seed=seed, model=model, scale=scale, trunc=trunc,
                                   dtype=dtype, levels=1, iters=iters, cost_sha=sha(P.D), table_sha=sha(P.V),
                                   energy_ref_type=e_ref)
        arrays[name + "/init"] = init.astype(np.int16)
        arrays[name + "/labels"] = lab.astype(np.int16)
        if msgs.size <= 200000:
            arrays[name + "/msgs"] = msgs
        else:
            gold["cases"][name]["msgs_sha"] = sha(msgs)
        arrays[name + "/icm_sync3"] = icm_s.astype(np.int16)
        arrays[name + "/icm_async2"] = icm_a.astype(np.int16)
        print("case", name, flush=True)

    for (name, W, H, L, seed, model, scale, trunc, dtype, levels, iters) in SMALL_HBP:
        P = small_problem(W, H, L, seed, model, scale, trunc, dtype)
        init = initial_labels(W, H, L, seed)
        lab = oracle.ref_hbp(P.D, P.V, model, scale, trunc, levels, iters, labels=init)
        gold["cases"][name] = dict(kind="hbp", W=W, H=H, L=L, seed=seed, model=model, scale=scale, trunc=trunc,
                                   dtype=dtype, levels=levels, iters=iters, cost_sha=sha(P.D), table_sha=sha(P.V),
                                   energy_ref_type=float(oracle.ref_energy(P.D, P.V, model, scale, trunc, lab)))
        arrays[name + "/init"] = init.astype(np.int16)
        arrays[name + "/labels"] = lab.astype(np.int16)
        print("case", name, flush=True)

    # Plain loopy BP workload: 384x288, L=16, 50 half-sweeps.
    P = synth.workload_plain_bp()
    t0 = time.time()
    lab = oracle.ref_hbp(P.D, P.V, P.model, P.scale, P.trunc, 1, 50)
    t_ref = time.time() - t0
    icm = oracle.ref_icm(P.D, P.V, P.model, P.scale, P.trunc, lab, 5)
    gold["cases"]["plain_bp_384x288_L16"] = dict(
        kind="workload", W=384, H=288, L=16, levels=1, iters=50, cost_sha=sha(P.D), table_sha=sha(P.V),
        labels_sha=sha(lab), energy_ref_type=float(oracle.ref_energy(P.D, P.V, P.model, P.scale, P.trunc, lab)),
        energy_f64=oracle.energy(P.D, P.V, lab), icm5_sha=sha(icm),
        icm5_energy_f64=oracle.energy(P.D, P.V, icm), reference_seconds_1core=t_ref)
    arrays["plain_bp_384x288_L16/labels"] = lab.astype(np.int8)
    print("plain BP workload done", t_ref, flush=True)

    if args.skip_large:
        # keep the previously generated large case, if any
        try:
            with open(os.path.join(HERE, "golden.json")) as f:
                old = json.load(f)["cases"].get("hbp_1920x1080_L64")
            if old is not None:
                gold["cases"]["hbp_1920x1080_L64"] = old
        except FileNotFoundError:
            pass
    else:
        P = synth.workload_hbp()
        t0 = time.time()
        lab = oracle.ref_hbp(P.D, P.V, P.model, P.scale, P.trunc, 5, 10)
        t_ref = time.time() - t0
        icm = oracle.ref_icm(P.D, P.V, P.model, P.scale, P.trunc, lab, 5)
        gold["cases"]["hbp_1920x1080_L64"] = dict(
            kind="workload", W=1920, H=1080, L=64, levels=5, iters=10, icm_iters=5, cost_sha=sha(P.D),
            table_sha=sha(P.V), labels_sha=sha(lab), icm5_sha=sha(icm),
            energy_f64=oracle.energy(P.D, P.V, lab), icm5_energy_f64=oracle.energy(P.D, P.V, icm),
            reference_seconds_1core=t_ref)
        print("HBP workload done", t_ref, flush=True)

    write(gold, arrays)


def write(gold, arrays):
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(gold, f, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "golden_arrays.npz"), **arrays)
    print("wrote", os.path.join(HERE, "golden.json"))


if __name__ == "__main__":
    main()
