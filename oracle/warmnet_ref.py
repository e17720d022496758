"""CPU restatement of the warm-start network (forward, loss, backward).

TEST INFRASTRUCTURE ONLY: the checker for the GPU kernels of
gridinfcuda_gb300/csrc/warmnet.cu.  Sums run in float64; with bf16=True the
values are rounded to BF16 (round to nearest even) exactly where the GPU
rounds them: the input x, the weights, the hidden activations, and every
gradient that feeds a tensor-core product.  With bf16=False the network is
plain float64, which tests/test_warmnet_cpu.py checks against finite
differences.

Network: conv3x3(L->h) ReLU, conv3x3(h->h) ReLU, conv3x3(h->h) ReLU,
conv3x3(h->L), zero padding, y = x + net(x); loss = mean((y - t)^2).
Parameters are flat, per layer the weights (cout, 3, 3, cin) then the bias.
"""
import numpy as np


def to_bf16(a):
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def shapes(L, hidden=32):
    ch = [L, hidden, hidden, hidden, L]
    return [(ch[i], ch[i + 1]) for i in range(4)]


def unpack(params, L, hidden=32):
    out, off = [], 0
    for cin, cout in shapes(L, hidden):
        n = cout * 9 * cin
        W = np.asarray(params[off:off + n], np.float64).reshape(cout, 3, 3, cin)
        off += n
        b = np.asarray(params[off:off + cout], np.float64)
        off += cout
        out.append((W, b))
    return out


def conv(x, W, b=None):
    """x (N, H, W, Cin), W (Cout, 3, 3, Cin) -> (N, H, W, Cout), zero padding."""
    N, H, Wd, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((N, H, Wd, W.shape[0]))
    for ky in range(3):
        for kx in range(3):
            out += np.einsum("nhwc,oc->nhwo", xp[:, ky:ky + H, kx:kx + Wd, :], W[:, ky, kx, :])
    return out if b is None else out + b


def forward(params, x, L, hidden=32, bf16=True):
    r = to_bf16 if bf16 else (lambda a: np.asarray(a, np.float64))
    layers = unpack(params, L, hidden)
    x64 = np.asarray(x, np.float64)
    acts = [r(x)]
    for l in range(3):
        W, b = layers[l]
        acts.append(r(np.maximum(conv(acts[-1], r(W), b), 0.0)))
    W, b = layers[3]
    y = x64 + conv(acts[3], r(W), b)
    return y, acts


def gradients(params, x, target, L, hidden=32, bf16=True):
    """(loss, flat gradient in the parameter order)."""
    r = to_bf16 if bf16 else (lambda a: np.asarray(a, np.float64))
    layers = unpack(params, L, hidden)
    y, acts = forward(params, x, L, hidden, bf16)
    d = y - np.asarray(target, np.float64)
    loss = float(np.mean(d * d))
    g = 2.0 * d / d.size
    grads = [None] * 4
    gb = r(g)
    for l in range(3, -1, -1):
        W, _ = layers[l]
        a = acts[l]
        H, Wd = a.shape[1], a.shape[2]
        ap = np.pad(a, ((0, 0), (1, 1), (1, 1), (0, 0)))
        dW = np.zeros_like(W)
        for ky in range(3):
            for kx in range(3):
                dW[:, ky, kx, :] = np.einsum("nhwo,nhwc->oc", gb, ap[:, ky:ky + H, kx:kx + Wd, :])
        db = g.sum(axis=(0, 1, 2))
        grads[l] = (dW, db)
        if l == 0:
            break
        Wf = r(W)[:, ::-1, ::-1, :].transpose(3, 1, 2, 0)  # (cin, 3, 3, cout), flipped
        da = conv(gb, Wf)
        g = da * (a > 0)
        gb = r(g)
    flat = np.concatenate([np.concatenate([dW.reshape(-1), db]) for dW, db in grads])
    return loss, flat


def init_params(L, hidden=32, seed=0):
    rng = np.random.default_rng(seed)
    parts = []
    for l, (cin, cout) in enumerate(shapes(L, hidden)):
        bound = np.sqrt(6.0 / (9 * cin)) * (0.1 if l == 3 else 1.0)
        parts.append(rng.uniform(-bound, bound, cout * 9 * cin))
        parts.append(rng.uniform(-0.05, 0.05, cout))
    return np.concatenate(parts).astype(np.float32)
