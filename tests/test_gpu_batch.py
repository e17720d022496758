"""Batched loopy BP (one persistent launch per group of half-sweeps, replayed
from a CUDA graph): every grid's labels must equal a single-grid solve of
the same grid, bit for bit, for every tile size and half-sweeps-per-launch."""
import os

import numpy as np
import pytest

from gridinfcuda_gb300 import synth

pytestmark = pytest.mark.gpu

# Every label bucket of the batch kernels: exact 16 / 32 / 64 and the
# non-exact ones below each (5, 24, 48).
SHAPES = [(37, 29, 16), (64, 40, 32), (23, 61, 64), (50, 50, 24), (3, 7, 16), (129, 17, 16), (8, 3, 32),
          (70, 45, 64), (33, 21, 5), (41, 30, 48)]


def _problems(seed0=0):
    import torch
    out = []
    for i, (W, H, L) in enumerate(SHAPES):
        model = synth.POTTS if i % 3 == 2 else synth.TRUNC_LINEAR
        P = synth.random_problem(W, H, L, seed0 + i, model=model, scale=0.7 if model == synth.POTTS else 1.0,
                                 trunc=2.5)
        out.append((torch.from_numpy(P.D).cuda(), torch.from_numpy(P.V).cuda(), P.model))
    return out


def _single(ginf, problems, iters):
    import torch
    res = []
    for D, V, m in problems:
        lab = torch.zeros(D.shape[1:], dtype=torch.int32, device="cuda")
        res.append(ginf.decode_hbp(D, V, m, 1, iters, labels=lab).cpu().numpy())
    return res


@pytest.mark.parametrize("tile,spl", [(8, 1), (16, 0), (32, 3), (16, 5), (8, 0)])
def test_batch_equals_single_grid_solves(ginf, tile, spl):
    import torch
    problems = _problems()
    iters = 11
    want = _single(ginf, problems, iters)
    labels = [torch.zeros(D.shape[1:], dtype=torch.int32, device="cuda") for D, _, _ in problems]
    with ginf.Batch(problems, labels, iters, tile_nodes=tile, sweeps_per_launch=spl) as b:
        assert b.config()["tuned_now"] is False
        for rep in range(2):
            b.run()
            for g, (lab, w) in enumerate(zip(labels, want)):
                assert np.array_equal(lab.cpu().numpy(), w), (tile, spl, rep, g)


@pytest.mark.parametrize("iters", [0, 1, 2])
def test_batch_short_runs(ginf, iters):
    import torch
    problems = _problems(50)
    want = _single(ginf, problems, iters)
    labels = [torch.zeros(D.shape[1:], dtype=torch.int32, device="cuda") for D, _, _ in problems]
    with ginf.Batch(problems, labels, iters, tile_nodes=16, sweeps_per_launch=0) as b:
        b.run()
    for lab, w in zip(labels, want):
        assert np.array_equal(lab.cpu().numpy(), w)


def test_batch_replay_sees_new_costs(ginf):
    import torch
    problems = _problems(7)
    labels = [torch.zeros(D.shape[1:], dtype=torch.int32, device="cuda") for D, _, _ in problems]
    with ginf.Batch(problems, labels, 9, tile_nodes=16, sweeps_per_launch=0) as b:
        b.run()
        fresh = _problems(99)
        for (D, V, _), (D2, V2, _) in zip(problems, fresh):
            D.copy_(D2)
            V.copy_(V2)
        b.run()
    want = _single(ginf, fresh, 9)
    for lab, w in zip(labels, want):
        assert np.array_equal(lab.cpu().numpy(), w)


def test_autotuner_measures_then_uses_its_cache(ginf, tmp_path, monkeypatch):
    import torch
    monkeypatch.setenv("GINF_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    problems = _problems(3)
    want = _single(ginf, problems, 8)
    labels = [torch.zeros(D.shape[1:], dtype=torch.int32, device="cuda") for D, _, _ in problems]
    with ginf.Batch(problems, labels, 8) as b:
        c1 = b.config()
        b.run()
    assert c1["tuned_now"] is True
    assert os.path.exists(tmp_path / "tune.json")
    assert '"tile_nodes"' in open(tmp_path / "tune.json").read()
    for lab, w in zip(labels, want):
        assert np.array_equal(lab.cpu().numpy(), w)
    with ginf.Batch(problems, labels, 8) as b:
        c2 = b.config()
    assert c2["tuned_now"] is False
    assert (c2["tile_nodes"], c2["sweeps_per_launch"]) == (c1["tile_nodes"], c1["sweeps_per_launch"])


def test_batch_rejects_unsupported_grids(ginf):
    import torch
    P = synth.random_problem(20, 20, 80, 1)
    D, V = torch.from_numpy(P.D).cuda(), torch.from_numpy(P.V).cuda()
    lab = torch.zeros((20, 20), dtype=torch.int32, device="cuda")
    with pytest.raises(ginf.GinfError) as e:
        ginf.Batch([(D, V, P.model)], [lab], 4)
    assert e.value.status == ginf.ERR_UNSUPPORTED


def test_stream_ordered_replays(ginf):
    """Two plans replayed stream-ordered on two streams, twice each: every
    replay equals the single-grid solves."""
    import torch
    iters = 7
    probs = [_problems(70), _problems(90)]
    want = [_single(ginf, p, iters) for p in probs]
    labels = [[torch.zeros(D.shape[1:], dtype=torch.int32, device="cuda") for D, _, _ in p] for p in probs]
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    plans = [ginf.Batch(p, l, iters, tile_nodes=16, sweeps_per_launch=1) for p, l in zip(probs, labels)]
    try:
        for rep in range(2):
            for k in range(2):
                plans[k].enqueue(streams[k].cuda_stream)
            for k in range(2):
                plans[k].sync()
                for g, (lab, w) in enumerate(zip(labels[k], want[k])):
                    assert np.array_equal(lab.cpu().numpy(), w), (rep, k, g)
                    lab.zero_()
            torch.cuda.synchronize()
    finally:
        for pl in plans:
            pl.close()


def test_batch_workload_scale_vs_oracle(ginf, orc, tmp_path, monkeypatch):
    """The seeded 64-grid batch workload (sizes 200x150 .. 1280x720, L in
    {16, 32, 64}, 30 half-sweeps, costs built on the GPU) plus two grids at
    the edges of its range -- the full 1280x720 x 64 and a non-exact label
    count (L = 48) -- solved by one autotuned plan.  Every grid must equal its
    single-grid solve, and the largest, the smallest, the first grid of each
    label count and the L = 48 grid must equal the CPU oracle's loopy BP
    (the reference's decodeBp, src/bp.cc:182-187) bit for bit."""
    import torch
    monkeypatch.setenv("GINF_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    iters = 30
    shapes = synth.batch_shapes(64, seed=2) + [(1280, 720, 64), (1001, 433, 48)]
    pairs, problems, labels = [], [], []
    for i, (W, H, L) in enumerate(shapes):
        pair = synth.stereo_pair(W, H, L, 12, 2.0, seed=100 + i)
        D = torch.empty((L, H, W), dtype=torch.float32, device="cuda")
        ginf.stereo_costs(torch.from_numpy(pair.left).cuda(), torch.from_numpy(pair.right).cuda(), L, 0.07, 15.0, D)
        V = torch.from_numpy(synth.sm_table(L, synth.TRUNC_LINEAR, 1.0, 1.7)).cuda()
        pairs.append(pair)
        problems.append((D, V, synth.TRUNC_LINEAR))
        labels.append(torch.zeros((H, W), dtype=torch.int32, device="cuda"))
    with ginf.Batch(problems, labels, iters, autotune=0) as b:
        assert b.config()["tuned_now"] is True
        b.run()
        got = [l.cpu().numpy() for l in labels]
    want = _single(ginf, problems, iters)
    for g, (a, w) in enumerate(zip(got, want)):
        assert np.array_equal(a, w), (g, shapes[g])
    size = [W * H * L for W, H, L in shapes]
    pick = {int(np.argmax(size)), int(np.argmin(size)), len(shapes) - 1}
    for L in (16, 32, 64):
        pick.add(next(i for i, s in enumerate(shapes) if s[2] == L))
    assert len(shapes) - 2 in pick   # 1280x720x64 is the largest
    for g in sorted(pick):
        W, H, L = shapes[g]
        D = synth.cost_volume(pairs[g], L, 0.07, 15.0)
        lab, _ = orc.hbp(D, synth.sm_table(L, synth.TRUNC_LINEAR, 1.0, 1.7), synth.TRUNC_LINEAR, 1, iters)
        assert np.array_equal(got[g], lab), (g, shapes[g])
