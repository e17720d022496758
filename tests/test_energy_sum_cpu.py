"""The energy kernel sums FP32 terms as double-float pairs (Knuth's TwoSum,
k_energy_partial in csrc/aux_kernels.cu): a thread accumulates its terms into
(hi, lo), warps merge pairs, and only the per-warp results are converted to
FP64.  This restates that arithmetic with IEEE float32 scalars and checks it
against the exact sum (math.fsum) on terms with a wide dynamic range and heavy
cancellation: the error stays within a few units of 2^-48 of the sum of
magnitudes, far inside the 1e-12 the energy tests allow."""
import math

import numpy as np

f32 = np.float32


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    e = f32(f32(a - f32(s - bb)) + f32(b - bb))
    return s, e


def acc_add(hi, lo, x):
    s, e = two_sum(hi, x)
    return two_sum(s, f32(e + lo))


def acc_merge(a, b):
    s, e = two_sum(a[0], b[0])
    return two_sum(s, f32(e + f32(a[1] + b[1])))


def test_two_sum_is_exact():
    rng = np.random.default_rng(1)
    for _ in range(2000):
        a, b = (f32(v) for v in rng.standard_normal(2) * 10.0 ** rng.integers(-8, 8, 2))
        s, e = two_sum(a, b)
        assert math.fsum([float(s), float(e)]) == math.fsum([float(a), float(b)])


def test_thread_and_warp_sums_match_the_exact_sum():
    rng = np.random.default_rng(2)
    for trial in range(20):
        n_threads, per_thread = 32, 24
        mags = 10.0 ** rng.uniform(-3, 4, (n_threads, per_thread))
        terms = (rng.choice([-1.0, 1.0], (n_threads, per_thread)) * mags).astype(np.float32)
        if trial % 2:
            terms[:, 1::2] = -terms[:, ::2]  # exact cancellation pairs
            terms[:, 0] += f32(0.125)
        pairs = []
        for t in range(n_threads):
            hi, lo = f32(0), f32(0)
            for x in terms[t]:
                hi, lo = acc_add(hi, lo, x)
            pairs.append((hi, lo))
        # xor-butterfly merge as the warp shuffles do; lane 0's result
        for off in (16, 8, 4, 2, 1):
            pairs = [acc_merge(pairs[i], pairs[i ^ off]) for i in range(n_threads)]
        got = float(pairs[0][0]) + float(pairs[0][1])
        exact = math.fsum(float(x) for x in terms.ravel())
        scale = math.fsum(abs(float(x)) for x in terms.ravel())
        assert abs(got - exact) <= 8 * 2.0 ** -48 * scale, (trial, got, exact)
