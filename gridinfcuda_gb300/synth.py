"""Seeded synthetic stereo MRF problems (the inputs of the benchmark workloads).

The generator is bit-reproducible on any IEEE-754 host: a counter-based
SplitMix64 stream (Steele, Lea and Flood, "Fast splittable pseudorandom number
generators", OOPSLA 2014) gives exact dyadic uniforms, Gaussian noise is the
Irwin-Hall sum of twelve uniforms minus six (mean 0, variance 1; no libm
transcendental functions are involved), and every float operation is a single
correctly rounded numpy ufunc.  The same images therefore give the same cost
volume on x86-64 and on aarch64, and the GPU cost-volume kernel
(``ginf_stereo_costs``) reproduces :func:`cost_volume` bit for bit.

Problem recipe (a stand-in for a real rectified stereo pair):
  * right image R: uniform texture in [0, 255], smoothed by a 3x3 box filter
    (border pixels average over their valid neighbours);
  * disparity map: a background value plus axis-aligned rectangles, each
    either constant (integer d) or a slanted plane d = round(a x + b y + c),
    clamped to [0, L-1]; later rectangles overwrite earlier ones;
  * left image: I_L(x, y) = R(max(x - disp, 0), y) + sigma * noise;
  * data cost D(x, y, d) = coef * min(|I_L(x, y) - R(max(x - d, 0), y)|, cap),
    stored label-planar (index x + W*y + W*H*d), the layout of the
    reference's Grid data costs (src/include/grid.h:20-21, matrix.cc:52-56).
    The reference example (examples/stereo/stereo.cc:28-34) leaves columns
    x < L-1 at zero cost; clamping x - d at 0 avoids those all-zero ties.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)
_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_C1 = np.uint64(0xBF58476D1CE4E5B9)
_C2 = np.uint64(0x94D049BB133111EB)

# Smoothness models, numbered as the reference's SmoothnessFunctions enum
# (src/include/grid.h:9-14).
EXPLICIT, POTTS, TRUNC_LINEAR, TRUNC_QUAD = 0, 1, 2, 3


def _mix(z: np.ndarray) -> np.ndarray:
    z = z.astype(np.uint64, copy=True)
    z ^= z >> np.uint64(30)
    z *= _C1
    z ^= z >> np.uint64(27)
    z *= _C2
    z ^= z >> np.uint64(31)
    return z


class Rng:
    """Counter-based SplitMix64 stream: draw i of stream (seed) is mix(key + (i+1)*gamma)."""

    def __init__(self, seed: int, stream: int = 0):
        base = np.array([(seed * 0x632BE59BD9B4E019 + stream * 0x8CB92BA72F3D8DD7 + 1) & 0xFFFFFFFFFFFFFFFF],
                        dtype=np.uint64)
        self._key = _mix(base)[0]
        self._ctr = 0

    def bits(self, n: int) -> np.ndarray:
        idx = np.arange(self._ctr + 1, self._ctr + 1 + n, dtype=np.uint64)
        self._ctr += n
        with np.errstate(over="ignore"):
            return _mix(self._key + idx * _GAMMA)

    def uniform(self, n: int) -> np.ndarray:
        """Exact dyadic uniforms in [0, 1) as float64 (53 random bits)."""
        return (self.bits(n) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)

    def integers(self, lo: int, hi: int, n: int) -> np.ndarray:
        """Integers in [lo, hi] (inclusive), by exact floor of a scaled uniform."""
        return lo + np.floor(self.uniform(n) * (hi - lo + 1)).astype(np.int64)

    def normal(self, n: int) -> np.ndarray:
        """Irwin-Hall N(0, 1) approximation: sum of 12 uniforms minus 6."""
        u = self.uniform(12 * n).reshape(n, 12)
        acc = np.zeros(n, dtype=np.float64)
        for k in range(12):
            acc = acc + u[:, k]
        return acc - 6.0


def _box3(img: np.ndarray) -> np.ndarray:
    """3x3 box filter, averaging over the valid pixels at the border."""
    H, W = img.shape
    acc = np.zeros_like(img)
    cnt = np.zeros_like(img)
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            ys0, ys1 = max(0, dy), H + min(0, dy)
            xs0, xs1 = max(0, dx), W + min(0, dx)
            acc[ys0 - dy:ys1 - dy, xs0 - dx:xs1 - dx] += img[ys0:ys1, xs0:xs1]
            cnt[ys0 - dy:ys1 - dy, xs0 - dx:xs1 - dx] += 1.0
    return acc / cnt


@dataclass
class StereoPair:
    left: np.ndarray        # (H, W) float32
    right: np.ndarray       # (H, W) float32
    disparity: np.ndarray   # (H, W) int32, ground truth


def stereo_pair(W: int, H: int, L: int, n_regions: int, sigma: float, seed: int,
                planar: bool = False, background: int | None = 2) -> StereoPair:
    """Seeded synthetic rectified stereo pair (see the module docstring)."""
    rng = Rng(seed, 1)
    right = _box3(rng.uniform(H * W).reshape(H, W) * 255.0)
    ys, xs = np.mgrid[0:H, 0:W]
    if planar:
        a, b = rng.uniform(2) * 0.04 - 0.02
        c = rng.uniform(1)[0] * (L - 1)
        disp = np.clip(np.rint(a * xs + b * ys + c), 0, L - 1).astype(np.int64)
    else:
        disp = np.full((H, W), background if background is not None else 0, dtype=np.int64)
    for _ in range(n_regions):
        x0, x1 = np.sort(rng.integers(0, W - 1, 2))
        y0, y1 = np.sort(rng.integers(0, H - 1, 2))
        if planar:
            a, b = rng.uniform(2) * 0.04 - 0.02
            c = rng.uniform(1)[0] * (L - 1)
            sl = (slice(y0, y1 + 1), slice(x0, x1 + 1))
            disp[sl] = np.clip(np.rint(a * xs[sl] + b * ys[sl] + c), 0, L - 1).astype(np.int64)
        else:
            disp[y0:y1 + 1, x0:x1 + 1] = rng.integers(0, L - 1, 1)[0]
    src = np.maximum(xs - disp, 0)
    left = right[ys, src] + sigma * rng.normal(H * W).reshape(H, W)
    return StereoPair(left.astype(np.float32), right.astype(np.float32), disp.astype(np.int32))


def cost_volume(pair: StereoPair, L: int, coef: float, cap: float) -> np.ndarray:
    """Label-planar float32 data costs, shape (L, H, W): D[d, y, x]."""
    H, W = pair.left.shape
    coef32, cap32 = np.float32(coef), np.float32(cap)
    out = np.empty((L, H, W), dtype=np.float32)
    xs = np.arange(W)
    for d in range(L):
        shifted = pair.right[:, np.maximum(xs - d, 0)]
        out[d] = coef32 * np.minimum(np.abs(pair.left - shifted), cap32)
    return out


def sm_table(L: int, model: int, scale, d=None, dtype=np.float32) -> np.ndarray:
    """Smoothness table V, flat, index fp + L*fq, as the reference fills it
    (src/grid.cc:69-100): Potts lambda*(fp != fq), truncated linear
    min(scale*|fp-fq|, d), truncated quadratic min(scale*(fp-fq)^2, d)."""
    fp = np.arange(L)[None, :]
    fq = np.arange(L)[:, None]
    diff = np.abs(fp - fq).astype(dtype)
    s = dtype(scale)
    if model == POTTS:
        V = s * (fp != fq).astype(dtype)
    elif model == TRUNC_LINEAR:
        V = np.minimum(s * diff, dtype(d))
    elif model == TRUNC_QUAD:
        V = np.minimum(s * (diff * diff), dtype(d))
    else:
        raise ValueError("sm_table builds the Potts / linear / quadratic tables only")
    return np.ascontiguousarray(V.astype(dtype)).reshape(-1)


@dataclass
class Problem:
    """One grid MRF: label-planar costs D (L, H, W), flat table V, model id."""
    D: np.ndarray
    V: np.ndarray
    model: int
    scale: float
    trunc: float

    @property
    def shape(self):
        L, H, W = self.D.shape
        return W, H, L


def stereo_problem(W: int, H: int, L: int, *, seed: int, n_regions: int, sigma: float, planar: bool,
                   coef: float, cap: float, model: int, scale: float, trunc: float,
                   background: int | None = 2) -> Problem:
    pair = stereo_pair(W, H, L, n_regions, sigma, seed, planar=planar, background=background)
    D = cost_volume(pair, L, coef, cap)
    return Problem(D, sm_table(L, model, scale, trunc), model, scale, trunc)


# The benchmark workloads, as stated for the reference's headline metric.
def workload_plain_bp(seed: int = 0, W: int = 384, H: int = 288) -> Problem:
    """Plain loopy BP: 384x288, L=16, 12 constant rectangles on disparity 2,
    sigma 2, D = 0.07 min(|dI|, 15), V = min(|a-b|, 1.7); 50 iterations."""
    return stereo_problem(W, H, 16, seed=seed, n_regions=12, sigma=2.0, planar=False, coef=0.07, cap=15.0,
                          model=TRUNC_LINEAR, scale=1.0, trunc=1.7)


def workload_hbp(seed: int = 1, W: int = 1920, H: int = 1080) -> Problem:
    """Hierarchical BP: 1920x1080, L=64, 40 slanted planes, sigma 3,
    D = 0.07 min(|dI|, 15), V = min(|a-b|, 4); 5 levels x 10 iterations,
    then 5 ICM sweeps."""
    return stereo_problem(W, H, 64, seed=seed, n_regions=40, sigma=3.0, planar=True, coef=0.07, cap=15.0,
                          model=TRUNC_LINEAR, scale=1.0, trunc=4.0)


def workload_quad(seed: int = 3, W: int = 3840, H: int = 2160, L: int = 128) -> Problem:
    """Precision sweep: 3840x2160, L=128, 80 planes, D = 0.05 min(|dI|, 20),
    V = min((a-b)^2, 25); 40 iterations."""
    return stereo_problem(W, H, L, seed=seed, n_regions=80, sigma=3.0, planar=True, coef=0.05, cap=20.0,
                          model=TRUNC_QUAD, scale=1.0, trunc=25.0)


def batch_shapes(n: int = 64, seed: int = 2):
    """Sizes for the batched workload: W x H uniform in [200,1280] x [150,720],
    L drawn from {16, 32, 64}."""
    rng = Rng(seed, 7)
    Ws = rng.integers(200, 1280, n)
    Hs = rng.integers(150, 720, n)
    Ls = np.array([16, 32, 64])[rng.integers(0, 2, n)]
    return [(int(w), int(h), int(l)) for w, h, l in zip(Ws, Hs, Ls)]


def workload_batch_item(W: int, H: int, L: int, seed: int) -> Problem:
    return stereo_problem(W, H, L, seed=seed, n_regions=12, sigma=2.0, planar=False, coef=0.07, cap=15.0,
                          model=TRUNC_LINEAR, scale=1.0, trunc=1.7)


def random_problem(W: int, H: int, L: int, seed: int, model: int = TRUNC_LINEAR, scale: float = 1.0,
                   trunc: float = 1.7, dtype=np.float32, cost_max: float = 4.0) -> Problem:
    """Unstructured random costs (uniform in [0, cost_max)), for small parity cases."""
    rng = Rng(seed, 11)
    u = rng.uniform(L * H * W).reshape(L, H, W)
    if dtype == np.int32:
        D = np.floor(u * cost_max).astype(np.int32)
        V = sm_table(L, model, int(scale), int(trunc), dtype=np.int32) if model != EXPLICIT else None
    else:
        D = (u * cost_max).astype(np.float32)
        V = sm_table(L, model, scale, trunc) if model != EXPLICIT else None
    if V is None:
        v = Rng(seed, 12).uniform(L * L)
        V = (np.floor(v * 3) if dtype == np.int32 else v * 3).astype(dtype)
    return Problem(D, V, model, scale, trunc)
