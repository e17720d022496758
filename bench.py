#!/usr/bin/env python3
"""Benchmark of the GB300 grid-MRF inference path.

Workload (default): hierarchical BP on the 1920x1080, L=64 synthetic stereo
problem -- 5 pyramid levels x 10 half-sweeps, then 5 Jacobi ICM sweeps and
the FP64 energy -- one "step" being one full solve.  Metric:
node-label-iterations per second, summed over the BP levels
(sum_t W_t*H_t*L*iterations per step).

  value     inputs resident in HBM; C-ABI ginf_solve on device buffers,
            timed with CUDA events on the stream the library runs on.
  e2e       the same solve with pinned HOST buffers, frames streamed
            through the stream-ordered ginf_solve (two workspaces on two
            streams): every frame's host->device copy of costs, table and
            labels and device->host copy of labels and energy are inside the
            timed region; one frame's copy overlaps the previous frame's
            sweeps.  The one-synchronous-call-per-frame times are reported
            beside it.
  roofline  the finest-level half-sweep kernel: algorithmic bytes (updated
            nodes x (L costs + 4L incoming + 4L outgoing) x 4 B) per launch
            over its mean launch duration, from CUDA events the library
            records around the finest-level sweeps of every timed step.

Multi-GPU: the path does not shard (one grid, one GPU); N ranks run N
independent replicas ("weak" scaling), value = all ranks' work / max time.
``--impl reference`` times the reference algorithm's CPU restatement (the
oracle, all host threads) on the same workload and prints its own line.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "hbp": dict(name="hbp_1920x1080_L64_5lvl_x10_icm5", W=1920, H=1080, L=64, levels=5, iters=10, icm=5),
    "plain": dict(name="lbp_384x288_L16_50it", W=384, H=288, L=16, levels=1, iters=50, icm=0),
    "quad": dict(name="lbp_quad_3840x2160_L128_40it", W=3840, H=2160, L=128, levels=1, iters=40, icm=0),
    "warm": dict(name="learned_warm_start_hbp_1920x1080_L64", W=1920, H=1080, L=64, levels=5, iters=0, icm=0),
    "batch": dict(name="batch64_lbp_200x150-1280x720_L16-64_30it", W=0, H=0, L=0, levels=1, iters=30, icm=0,
                  count=64),
    "alphabeta": dict(name="alpha_beta_384x288_L16_int_1pass", W=384, H=288, L=16, levels=1, iters=1, icm=0),
    "warmnet": dict(name="warmnet_forward_960x540_L64", W=960, H=540, L=64, levels=1, iters=0, icm=0),
}
METRIC = "node-label-iters/s (LBP)"
UNIT = "node*label*iter/s"


def make_problem(kind, cfg, seed_offset=0):
    from gridinfcuda_gb300 import synth
    if kind == "hbp":
        return synth.workload_hbp(seed=1 + seed_offset, W=cfg["W"], H=cfg["H"])
    if kind == "quad":
        return synth.workload_quad(seed=3 + seed_offset, W=cfg["W"], H=cfg["H"], L=cfg["L"])
    return synth.workload_plain_bp(seed=0 + seed_offset, W=cfg["W"], H=cfg["H"])


def bench_config(workload, cfg):
    """The workload's `config` dict, printed identically by both arms."""
    W, H, L = cfg["W"], cfg["H"], cfg["L"]
    if workload in ("hbp", "plain"):
        return {"workload": cfg["name"], "width": W, "height": H, "labels": L, "levels": cfg["levels"],
                "iters_per_level": cfg["iters"], "icm_sweeps": cfg["icm"],
                "smoothness": "min(|a-b|, 4)" if workload == "hbp" else "min(|a-b|, 1.7)",
                "node_label_iters_per_step": nli_per_step(cfg),
                "l2": (f"inputs larger than L2 (costs {W * H * L * 4 / 1e6:.0f} MB, "
                       f"records {W * H * L * 20 * 4 / 3 / 1e9:.2f} GB)") if workload == "hbp" else
                      "L2-resident (costs 7 MB, records 35 MB); no flush between steps"}
    return {"workload": cfg["name"]}


GOLDEN_CASE = {"hbp": ("hbp_1920x1080_L64", "icm5_sha", "icm5_energy_f64"),
               "plain": ("plain_bp_384x288_L16", "labels_sha", "energy_f64")}


def parity_vs_golden(workload, labels, energy):
    """Labels (SHA-256) and FP64 energy of the timed solve against the
    reference's own result for the same seeded input (tests/golden, written
    by the reference's CPU code)."""
    import hashlib
    import numpy as np
    name, sha_key, e_key = GOLDEN_CASE[workload]
    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        case = json.load(f)["cases"][name]
    got = hashlib.sha256(np.ascontiguousarray(labels).tobytes()).hexdigest()
    e_ref = case[e_key]
    rel = abs(energy - e_ref) / abs(e_ref) if energy is not None else None
    ok = got == case[sha_key] and rel is not None and rel <= 1e-12
    return {"ok": ok, "labels_sha_equal": got == case[sha_key], "energy": energy, "energy_reference": e_ref,
            "energy_rel_diff": rel, "against": f"tests/golden/golden.json:{name} (the reference's decodeHbp"
                                               f"{' + decodeIcmSync' if workload == 'hbp' else ''} on this input)"}


def nli_per_step(cfg):
    W, H, total = cfg["W"], cfg["H"], 0
    for _ in range(cfg["levels"]):
        total += W * H * cfg["L"] * cfg["iters"]
        W, H = (W + 1) // 2, (H + 1) // 2
    return total


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_traffic(cfg):
    """DRAM bytes per finest-level sweep launch from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "sweep_traffic.json")) as f:
            t = json.load(f)
        if t.get("workload") == cfg["name"]:
            return float(t["dram_bytes_per_launch"])
    except Exception:
        pass
    return None


# ---------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi clock / throttle samples every 200 ms during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id):
        self.gpu_id = gpu_id
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu_id), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def gpu_smi_id(local_rank):
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        ids = [v.strip() for v in vis.split(",") if v.strip()]
        if local_rank < len(ids):
            return ids[local_rank]
    return local_rank


# ---------------------------------------------------------------- distributed

def dist_setup(use_cuda):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl" if use_cuda else "gloo")
    return rank, local, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce_max(x, world, device=None):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(x, world, device=None):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------- CPU baseline

def cpu_port_step(P, cfg, nthreads):
    """One step of the reference algorithm on the host: the C restatement of
    decodeHbp + decodeIcmSync + getLabelingCost (oracle/ginf_oracle.c)."""
    import oracle
    lab, _ = oracle.hbp(P.D, P.V, P.model, cfg["levels"], cfg["iters"], nthreads=nthreads)
    if cfg["icm"]:
        lab = oracle.icm(P.D, P.V, lab, cfg["icm"], nthreads=nthreads)
    return oracle.energy(P.D, P.V, lab)


def host_description():
    """CPU model and core count of this host."""
    model = platform.processor() or platform.machine()
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    return {"cpu_model": model, "nproc": os.cpu_count()}


def cpu_baseline(P, cfg, nthreads):
    """The oracle (C restatement of the reference algorithm) on the host: one
    full step on all threads, and a single-core sample (the reference itself
    is single-threaded): two half-sweeps of the finest level alone."""
    import oracle
    oracle.build()
    t0 = time.perf_counter()
    cpu_port_step(P, cfg, nthreads)
    dt = time.perf_counter() - t0
    t0 = time.perf_counter()
    oracle.hbp(P.D, P.V, P.model, 1, 2, nthreads=1)
    dt1 = time.perf_counter() - t0
    nli1 = cfg["W"] * cfg["H"] * cfg["L"] * 2
    out = {"value": nli_per_step(cfg) / dt, "unit": UNIT, "cores": nthreads, "kind": "port",
           "sample": f"one full step ({cfg['name']}) of the oracle C restatement, {nthreads} OpenMP threads, "
                     f"{dt:.2f} s",
           "single_core": {"value": nli1 / dt1, "unit": UNIT, "cores": 1,
                           "sample": f"2 half-sweeps of the {cfg['W']}x{cfg['H']}x{cfg['L']} finest level, "
                                     f"1 thread, {dt1:.2f} s"}}
    out.update(host_description())
    return out


# ---------------------------------------------------------------- our arm

def run_ours(args, cfg):
    import numpy as np
    import torch
    from gridinfcuda_gb300 import capi

    rank, local, world = dist_setup(True)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    P = make_problem(args.workload, cfg, seed_offset=rank)
    D = torch.from_numpy(P.D).to(dev)
    V = torch.from_numpy(P.V).to(dev)
    lab = torch.zeros((cfg["H"], cfg["W"]), dtype=torch.int32, device=dev)
    ws = capi.Workspace()
    stream = torch.cuda.current_stream(dev)
    opt = dict(stream=stream.cuda_stream, tile_nodes=args.tile_nodes, sweeps_per_launch=args.sweeps_per_launch)

    def step():
        return capi.solve(D, V, P.model, cfg["levels"], cfg["iters"], cfg["icm"], labels=lab, workspace=ws,
                          want_stats=True, **opt)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(gpu_smi_id(local))
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    stats = []
    energy = None
    for _ in range(args.steps):
        _, energy, st = step()
        stats.append(st)
    ev1.record(stream)
    torch.cuda.synchronize()
    clock_info = clocks.stop()
    lab_timed = lab.cpu().numpy()
    barrier(world)
    ms = reduce_max(ev0.elapsed_time(ev1), world, dev)
    nli = stats[0]["node_label_iters"]
    value = world * args.steps * nli / (ms / 1e3)
    launches = reduce_sum(sum(s["kernel_launches"] for s in stats), world, dev)

    # Roofline of the finest level's half-sweeps (the dominant kernel): the
    # HBM bytes they must move (reported by the library: per updated node its
    # costs and four incoming messages in, four messages out) over their
    # CUDA-event time.
    l0_ms = sum(s["level0_sweep_ms"] for s in stats) / len(stats)
    l0_launches = stats[0]["level0_sweep_launches"]
    l0_bytes = stats[0]["level0_alg_bytes"]
    W, H, L = cfg["W"], cfg["H"], cfg["L"]
    per_launch_s = l0_ms / l0_launches / 1e3
    alg_bytes = l0_bytes / l0_launches
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / per_launch_s / 1e9
    traffic = load_traffic(cfg)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
                "kernel": f"sweep_kernel<float,float,{L},...> (finest level)",
                "algorithmic_bytes_per_launch": alg_bytes, "mean_launch_ms": round(per_launch_s * 1e3, 4),
                "launches_per_step": l0_launches}

    # End to end through the C ABI with pinned host buffers.
    Dh = torch.from_numpy(P.D).pin_memory()
    Vh = torch.from_numpy(P.V).pin_memory()
    labh = torch.zeros((cfg["H"], cfg["W"]), dtype=torch.int32).pin_memory()

    def step_host(access):
        return capi.solve(Dh, Vh, P.model, cfg["levels"], cfg["iters"], cfg["icm"], labels=labh, workspace=ws,
                          want_stats=True, host_access=access, **opt)

    def time_e2e(access):
        for _ in range(max(1, min(args.warmup, 2))):
            step_host(access)
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        est = None
        for _ in range(args.steps):
            _, _, est = step_host(access)
        torch.cuda.synchronize()
        return reduce_max(time.perf_counter() - t0, world, dev), est

    # One synchronous call per frame: the device reads the pinned costs in
    # place (the transfer fused into the layout transform), or they are
    # staged by one host-to-device copy first.
    sync_s, est = time_e2e(capi.HOST_AUTO)
    copy_s, _ = time_e2e(capi.HOST_COPY)

    # Frames streamed through the stream-ordered call: two workspaces on two
    # streams, so frame i+1's host-to-device copy (copy engine) runs under
    # frame i's sweeps.  Every frame still moves its costs in and its labels
    # and energy out inside the timed region.
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    wss = [ws, capi.Workspace()]
    labs = [labh, torch.zeros_like(labh).pin_memory()]
    energies = [ctypes.c_double(), ctypes.c_double()]

    frame_opt = {k: v for k, v in opt.items() if k != "stream"}

    def frames(n):
        for i in range(n):
            k = i % 2
            capi.solve_async(Dh, Vh, P.model, cfg["levels"], cfg["iters"], cfg["icm"], labs[k], energies[k], wss[k],
                             streams[k].cuda_stream, host_access=capi.HOST_COPY, **frame_opt)
        for w in wss:
            w.sync()

    frames(max(2, min(args.warmup, 4)))
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    frames(args.steps)
    torch.cuda.synchronize()
    pipe_s = reduce_max(time.perf_counter() - t0, world, dev)
    if abs(energies[0].value - energies[1].value) > 1e-9 * abs(energies[0].value):
        raise RuntimeError("stream-ordered frames disagree")

    # Where the end-to-end time goes: the host link alone (one pinned copy of
    # a frame's costs, CUDA events), and the same two-workspace pipeline with
    # the inputs already on the device (its overhead without any copy).
    h2d_bytes = int(est["h2d_bytes"])
    stage = torch.empty_like(D)
    c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    copy_stream = torch.cuda.Stream()
    with torch.cuda.stream(copy_stream):
        stage.copy_(Dh, non_blocking=True)
        c0.record(copy_stream)
        for _ in range(5):
            stage.copy_(Dh, non_blocking=True)
        c1.record(copy_stream)
    torch.cuda.synchronize()
    h2d_gbs = 5 * Dh.numel() * 4 / (c0.elapsed_time(c1) / 1e3) / 1e9
    del stage
    labd = [lab, torch.zeros_like(lab)]

    def frames_device(n):
        for i in range(n):
            k = i % 2
            capi.solve_async(D, V, P.model, cfg["levels"], cfg["iters"], cfg["icm"], labd[k], energies[k], wss[k],
                             streams[k].cuda_stream, **frame_opt)
        for w in wss:
            w.sync()

    frames_device(2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    frames_device(args.steps)
    torch.cuda.synchronize()
    pipe_dev_s = time.perf_counter() - t0
    wss[1].close()
    e2e_ms = pipe_s * 1e3 / args.steps
    dev_ms = ms / args.steps
    copy_ms = h2d_bytes / (h2d_gbs * 1e9) * 1e3
    e2e = {"value": world * args.steps * nli / pipe_s, "unit": UNIT, "h2d_bytes_per_step": h2d_bytes,
           "d2h_bytes_per_step": int(est["d2h_bytes"]), "ms_per_step": round(e2e_ms, 3),
           "mode": "stream-ordered ginf_solve, 2 workspaces / 2 streams, pinned host buffers",
           "sync_call_ms_per_step": round(sync_s * 1e3 / args.steps, 3),
           "sync_call_staged_copy_ms_per_step": round(copy_s * 1e3 / args.steps, 3),
           "attribution": {
               "pinned_h2d_gbs": round(h2d_gbs, 1),
               "h2d_ms_per_step_alone": round(copy_ms, 3),
               "device_ms_per_step": round(dev_ms, 3),
               "pipelined_device_inputs_ms_per_step": round(pipe_dev_s * 1e3 / args.steps, 3),
               "copy_hidden_frac": round(max(0.0, min(1.0, (dev_ms + copy_ms - e2e_ms) / copy_ms)), 3),
               "note": "e2e = max(device, copy) if the copy were fully hidden; pipelined_device_inputs is the "
                       "same two-stream loop without any host copy"}}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(P, cfg, os.cpu_count() or 1)

    parity = None
    if rank == 0 and not args.size:
        parity = parity_vs_golden(args.workload, lab_timed, energy)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded stereo pair, slanted planar regions; no dataset)",
                "config": bench_config(args.workload, cfg), "parallelism": f"replicas x{world}",
                "parity": parity, "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clock_info,
                "gpu_launches": int(launches), "energy": energy,
                "phases_ms": {k: round(stats[-1][k], 4) for k in ("upload_ms", "prepare_ms", "sweep_ms",
                                                                  "level0_sweep_ms", "icm_ms", "energy_ms",
                                                                  "download_ms", "total_ms")}}
        print(json.dumps(line), flush=True)
    ws.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# ---------------------------------------------------------------- precision sweep

def run_precision(args, cfg):
    """Truncated-quadratic LBP (standard message rule) with the FP32 and the
    FP16 message store, each timed, and each compared with an FP64 run of the
    same kernels on the same input: message error (both sides re-normalised to
    zero mean per message, max |a-b| / max |b|), label agreement on interior
    nodes, FP64 energy gap."""
    import torch
    from gridinfcuda_gb300 import capi

    torch.cuda.set_device(0)
    P = make_problem("quad", cfg)
    D = torch.from_numpy(P.D).cuda()
    V = torch.from_numpy(P.V).cuda()
    W, H, L, iters = cfg["W"], cfg["H"], cfg["L"], cfg["iters"]
    ws = capi.Workspace()
    stream = torch.cuda.current_stream()
    base = dict(rule=capi.RULE_STANDARD, stream=stream.cuda_stream, workspace=ws)
    nli = W * H * L * iters

    def solve(store, ctype, want_msgs):
        return capi.decode_hbp(D, V, P.model, 1, iters, want_msgs=want_msgs, want_stats=True, store=store,
                               compute_type=ctype, **base)

    def compare(msgs, lab, msgs64, lab64, e64):
        worst, scale = 0.0, 0.0
        for r0 in range(0, H, 64):
            a = msgs[r0:r0 + 64].double()
            b = msgs64[r0:r0 + 64]
            a = a - a.mean(dim=-1, keepdim=True)
            b = b - b.mean(dim=-1, keepdim=True)
            worst = max(worst, float((a - b).abs().max()))
            scale = max(scale, float(b.abs().max()))
            del a, b
        e = capi.energy(D, V, P.model, lab, workspace=ws)
        return {"msg_rel_err": worst / max(scale, 1e-30),
                "label_agreement": float((lab[1:-1, 1:-1] == lab64[1:-1, 1:-1]).double().mean()),
                "energy": e, "energy_rel_gap": abs(e - e64) / abs(e64)}

    out = {}
    # Error against the FP64 run after 8, 16 and the configured 40 half-sweeps:
    # loopy BP on this problem does not converge, and the gap between any two
    # precisions grows geometrically with the iteration count.
    curve = {"f32": {}, "f16": {}}
    for n_it in (8, 16, iters):
        t0 = time.perf_counter()
        lab64, msgs64, st64 = capi.decode_hbp(D, V, P.model, 1, n_it, want_msgs=True, want_stats=True,
                                              store=capi.STORE_NATIVE, compute_type=capi.F64, **base)
        t64 = time.perf_counter() - t0
        e64 = capi.energy(D, V, P.model, lab64, workspace=ws)
        if n_it == iters:
            out["fp64_oracle"] = {"seconds": round(t64, 2), "sweep_ms": round(st64["sweep_ms"], 2), "energy": e64}
        for name, store in (("f32", capi.STORE_NATIVE), ("f16", capi.STORE_F16)):
            lab, msgs, _ = capi.decode_hbp(D, V, P.model, 1, n_it, want_msgs=True, want_stats=True, store=store,
                                           **base)
            curve[name][n_it] = compare(msgs, lab, msgs64, lab64, e64)
            del msgs
        del msgs64
        torch.cuda.empty_cache()
    for name, store in (("f32", capi.STORE_NATIVE), ("f16", capi.STORE_F16)):
        for _ in range(args.warmup):
            solve(store, -1, False)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        sts = []
        for _ in range(args.steps):
            sts.append(solve(store, -1, False)[1])
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / args.steps
        per_launch = sum(x["level0_sweep_ms"] for x in sts) / len(sts) / iters
        store_b = 2 if name == "f16" else 4
        alg = (W - 2) * (H - 2) / 2 * (L * 4 + 8 * L * store_b)
        out[name] = dict(curve[name][iters])
        out[name].update({"value": nli / (ms / 1e3), "unit": UNIT, "ms_per_solve": round(ms, 3),
                          "sweep_launch_ms": round(per_launch, 4),
                          "sweep_hbm_gbs": round(alg / (per_launch / 1e3) / 1e9, 1),
                          "algorithmic_bytes_per_launch": alg,
                          "vs_fp64_by_iterations": {str(k): v for k, v in curve[name].items()}})
    peak, peak_kind = load_peaks()
    line = {"metric": METRIC, "value": out["f16"]["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": out["f16"]["ms_per_solve"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f16 store / f32 arithmetic",
            "data": "synthetic (seeded stereo pair, 80 slanted planar regions; no dataset)",
            "config": {"workload": cfg["name"], "width": W, "height": H, "labels": L, "iters": iters,
                       "smoothness": "min((a-b)^2, 25), standard message rule",
                       "costs": "0.05 * min(|dI|, 20)"},
            "precision": out, "peak_hbm_gbs": peak, "peak_source": peak_kind}
    print(json.dumps(line), flush=True)
    ws.close()


# ---------------------------------------------------------------- batched grids

def run_batch(args, cfg):
    """64 independent grids (sizes uniform in 200x150..1280x720, L in
    {16, 32, 64}), 30 half-sweeps each, solved by one captured batch plan
    (persistent launches replayed from a CUDA graph, autotuned).  The cost
    volumes are built on the GPU from seeded stereo pairs."""
    import torch
    from gridinfcuda_gb300 import capi, synth

    rank, local, world = dist_setup(True)
    torch.cuda.set_device(local)
    shapes = synth.batch_shapes(cfg["count"], seed=2)
    problems, labels, nli = [], [], 0
    for i, (W, H, L) in enumerate(shapes):
        pair = synth.stereo_pair(W, H, L, 12, 2.0, seed=100 + i + 1000 * rank)
        D = torch.empty((L, H, W), dtype=torch.float32, device="cuda")
        capi.stereo_costs(torch.from_numpy(pair.left).cuda(), torch.from_numpy(pair.right).cuda(), L, 0.07, 15.0, D)
        V = torch.from_numpy(synth.sm_table(L, synth.TRUNC_LINEAR, 1.0, 1.7)).cuda()
        problems.append((D, V, synth.TRUNC_LINEAR))
        labels.append(torch.zeros((H, W), dtype=torch.int32, device="cuda"))
        nli += W * H * L * cfg["iters"]
    t0 = time.perf_counter()
    plan = capi.Batch(problems, labels, cfg["iters"], autotune=1 if args.retune else 0,
                      tile_nodes=args.tile_nodes, sweeps_per_launch=args.sweeps_per_launch)
    plan_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        plan.run(stream.cuda_stream)
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(gpu_smi_id(local))
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    sts = [plan.run(stream.cuda_stream, want_stats=True) for _ in range(args.steps)]
    ev1.record(stream)
    torch.cuda.synchronize()
    clock_info = clocks.stop()
    ms = reduce_max(ev0.elapsed_time(ev1), world)
    value = world * args.steps * nli / (ms / 1e3)
    # End to end: every batch's costs uploaded from pinned host memory and its
    # labels read back inside the timed region.  First one synchronous replay
    # per batch; then batches streamed through two plans on two streams
    # (stream-ordered replays), so batch i+1's upload runs under batch i's
    # sweeps.
    hostD = [D.cpu().pin_memory() for D, _, _ in problems]
    hostL = [[torch.empty(l.shape, dtype=torch.int32).pin_memory() for l in labels] for _ in range(2)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for (D, _, _), h in zip(problems, hostD):
            D.copy_(h, non_blocking=True)
        plan.run(stream.cuda_stream)
        for l, h in zip(labels, hostL[0]):
            h.copy_(l, non_blocking=True)
        torch.cuda.synchronize()
    sync_s = reduce_max(time.perf_counter() - t0, world)
    pc = plan.config()
    problems2 = [(D.clone(), V, m) for D, V, m in problems]
    labels2 = [torch.zeros_like(l) for l in labels]
    plan2 = capi.Batch(problems2, labels2, cfg["iters"], tile_nodes=pc["tile_nodes"],
                       sweeps_per_launch=pc["sweeps_per_launch"])
    plans = [(plan, problems, labels), (plan2, problems2, labels2)]
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]

    def batches(n):
        for i in range(n):
            k = i % 2
            pl, probs, labs = plans[k]
            with torch.cuda.stream(streams[k]):
                for (D, _, _), h in zip(probs, hostD):
                    D.copy_(h, non_blocking=True)
            pl.enqueue(streams[k].cuda_stream)
            with torch.cuda.stream(streams[k]):
                for l, h in zip(labs, hostL[k]):
                    h.copy_(l, non_blocking=True)
        for pl, _, _ in plans:
            pl.sync()
        torch.cuda.synchronize()

    batches(2)
    barrier(world)
    t0 = time.perf_counter()
    batches(args.steps)
    e2e_s = reduce_max(time.perf_counter() - t0, world)
    plan2.close()
    h2d = sum(h.numel() * 4 for h in hostD)
    d2h = sum(h.numel() * 4 for h in hostL[0])
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (64 seeded stereo pairs, cost volumes built on the GPU)",
                "config": {"workload": cfg["name"], "grids": len(shapes), "iters": cfg["iters"],
                           "node_label_iters_per_step": nli, "plan": plan.config(),
                           "plan_create_s": round(plan_s, 2), "parallelism": f"replicas x{world}"},
                "e2e": {"value": world * args.steps * nli / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h, "ms_per_step": round(e2e_s * 1e3 / args.steps, 3),
                        "mode": "stream-ordered batch replays, 2 plans / 2 streams, pinned host buffers",
                        "sync_run_ms_per_step": round(sync_s * 1e3 / args.steps, 3)},
                "clocks": clock_info, "gpu_launches": int(sum(s["kernel_launches"] for s in sts))}
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = batch_cpu_baseline(problems, cfg["iters"])
        line["parity"] = batch_parity(problems, labels, cfg["iters"])
        print(json.dumps(line), flush=True)
    plan.close()


def batch_parity(problems, labels, iters):
    """Labels of the timed batch against the oracle's loopy BP (the
    reference's decodeBp semantics, src/bp.cc:182-187) on a sample of its
    grids: the largest, and the first grid of each label count."""
    import hashlib
    import numpy as np
    import oracle
    oracle.build()
    size = [D.numel() for D, _, _ in problems]
    pick = {int(np.argmax(size))}
    for L in sorted({D.shape[0] for D, _, _ in problems}):
        pick.add(next(i for i, (D, _, _) in enumerate(problems) if D.shape[0] == L))
    out = {"grids": [], "against": "oracle loopy BP (bit-identical to the reference's decodeBp)"}
    for g in sorted(pick):
        D, V, model = problems[g]
        want, _ = oracle.hbp(D.cpu().numpy(), V.cpu().numpy(), model, 1, iters, nthreads=os.cpu_count() or 1)
        got = labels[g].cpu().numpy()
        L, H, W = D.shape
        out["grids"].append({"index": g, "shape": f"{W}x{H}x{L}", "equal": bool(np.array_equal(got, want)),
                             "labels_sha": hashlib.sha256(np.ascontiguousarray(got).tobytes()).hexdigest()[:16]})
    out["ok"] = all(x["equal"] for x in out["grids"])
    return out


def batch_cpu_baseline(problems, iters, sample=8):
    """Independent grids on all host cores: the oracle's BP (reference
    semantics) on the first `sample` grids of the batch, OpenMP over rows."""
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    nli, dt = 0, 0.0
    for D, V, model in problems[:sample]:
        Dh, Vh = D.cpu().numpy(), V.cpu().numpy()
        L, H, W = Dh.shape
        t0 = time.perf_counter()
        oracle.hbp(Dh, Vh, model, 1, iters, nthreads=threads)
        dt += time.perf_counter() - t0
        nli += W * H * L * iters
    out = {"value": nli / dt, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"the first {sample} grids of the batch, {iters} half-sweeps each, {threads} OpenMP threads, "
                     f"{dt:.2f} s"}
    out.update(host_description())
    return out


# ---------------------------------------------------------------- learned warm start

def run_warm(args, cfg):
    """Train the warm-start network on converged BP messages of seeded
    512x384x64 grids with the library's own tensor-core kernels, then measure
    time to energy (within 0.5 % of converged plain HBP) warm vs cold on
    unseen 1920x1080x64 grids."""
    import torch
    from gridinfcuda_gb300 import capi, warmstart

    torch.cuda.set_device(0)
    log = (lambda m: print(m, file=sys.stderr, flush=True)) if args.verbose else None
    t0 = time.perf_counter()
    X, Y = warmstart.make_training_set(n=args.train_grids, level=args.warm_level)
    t_data = time.perf_counter() - t0
    net = capi.WarmNet(64, 32, seed=1)
    t0 = time.perf_counter()
    hist = warmstart.train(net, X, Y, epochs=args.epochs, batch=args.batch, lr=args.lr, log=log)
    t_train = time.perf_counter() - t0
    if args.save_net:
        net.save(args.save_net)
    base_loss = float(((X - Y) ** 2).mean())   # loss of the network-free guess y = x
    del X, Y
    torch.cuda.empty_cache()
    res = warmstart.evaluate(net, n=args.eval_grids, log=log, level=args.warm_level)
    summ = warmstart.summarize(res)
    line = {"metric": "ms to plain-BP energy +0.5%, warm-start vs plain", "value": summ["ms_warm_mean"],
            "unit": "ms", "n_gpus": 1, "higher_is_better": False, "vs_baseline": None, "dtype": "bf16 net / f32 BP",
            "data": "synthetic (seeded planar-region stereo; no dataset)",
            "config": {"workload": cfg["name"], "train_grids": args.train_grids, "train_size": "512x384x64",
                       "eval_grids": args.eval_grids, "epochs": args.epochs, "levels": 5,
                       "warm_level": args.warm_level, "batch": args.batch, "lr": args.lr},
            "warm_start": summ,
            "training": {"data_s": round(t_data, 1), "train_s": round(t_train, 1), "final_loss": hist[-1],
                         "first_epoch_loss": hist[0], "loss_without_network": base_loss}}
    print(json.dumps(line), flush=True)
    net.close()


# ---------------------------------------------------------------- alpha-beta swap

def run_alphabeta(args, cfg):
    """Alpha-beta swap (src/graphcut.cc:197-279) on the reference example's
    integer problem shape: 8-bit grey images of the seeded 384x288 stereo
    pair, costs min(|L(x) - R(x-k)|, 20) for x >= L-1 (ginf_stereo_costs_u8),
    TruncLinear(10, 20), 16 labels, from the 30-iteration loopy-BP labels,
    `iters` passes.  One step is one solve from device buffers; the oracle's
    C restatement (single-threaded, as the reference) is timed on the same
    input and its labels compared."""
    import hashlib
    import numpy as np
    import torch
    from gridinfcuda_gb300 import capi, synth
    torch.cuda.set_device(0)
    W, H, L, iters = cfg["W"], cfg["H"], cfg["L"], cfg["iters"]
    pair = synth.stereo_pair(W, H, L, 12, 2.0, seed=0)
    left = np.clip(np.rint(pair.left), 0, 255).astype(np.uint8)
    right = np.clip(np.rint(pair.right), 0, 255).astype(np.uint8)
    D = torch.empty((L, H, W), dtype=torch.int32, device="cuda")
    capi.stereo_costs_u8(torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda(), L, 20, D)
    V = torch.from_numpy(synth.sm_table(L, synth.TRUNC_LINEAR, 10, 20, dtype=np.int32)).cuda()
    init = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    capi.decode_hbp(D, V, synth.TRUNC_LINEAR, 1, 30, labels=init)
    ws = capi.Workspace()
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        capi.decode_alpha_beta(D, V, synth.TRUNC_LINEAR, init, iters, workspace=ws, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        out = capi.decode_alpha_beta(D, V, synth.TRUNC_LINEAR, init, iters, workspace=ws, stream=stream.cuda_stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    got = out.cpu().numpy()
    e0 = capi.energy(D, V, synth.TRUNC_LINEAR, init, workspace=ws)
    e1 = capi.energy(D, V, synth.TRUNC_LINEAR, out, workspace=ws)
    pairs = L * (L - 1) // 2
    line = {"metric": "alpha-beta swap node*pair/s", "value": W * H * pairs * iters / (ms / 1e3),
            "unit": "node*pair/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32", "data": "synthetic (seeded stereo pair as 8-bit grey images; no dataset)",
            "config": {"workload": cfg["name"], "width": W, "height": H, "labels": L, "passes": iters,
                       "costs": "min(|L(x)-R(x-k)|, 20) for x >= L-1", "smoothness": "min(10|a-b|, 20)",
                       "initial": "30-iteration loopy BP labels"},
            "energy_initial": e0, "energy": e1, "labels_changed": int((got != init.cpu().numpy()).sum()),
            "gpu_launches": 1}
    if not args.no_cpu_baseline:
        import oracle
        oracle.build()
        Dh, Vh, ih = D.cpu().numpy(), V.cpu().numpy(), init.cpu().numpy()
        t0 = time.perf_counter()
        want = oracle.alpha_beta(Dh, Vh, ih, iters)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": W * H * pairs * iters / dt, "unit": "node*pair/s", "cores": 1,
                                "kind": "port", "sample": f"one full solve, {dt:.2f} s (the reference is "
                                                          f"single-threaded)"}
        line["cpu_baseline"].update(host_description())
        line["parity"] = {"ok": bool(np.array_equal(got, want)),
                          "labels_sha": hashlib.sha256(got.tobytes()).hexdigest()[:16],
                          "against": "oracle C restatement of src/graphcut.cc (bit-identical to the reference)"}
    print(json.dumps(line), flush=True)
    ws.close()


# ---------------------------------------------------------------- warm-start network

def warmnet_bytes_flops(W, H, L, hidden=32):
    """Algorithmic HBM bytes and FLOPs of one forward pass over an n=1, HxW,
    L-label input: the FP32 -> BF16 conversion of x, four 3x3 convolutions
    (BF16 activations, each read once and written once), the last layer's
    FP32 residual read and FP32 output write."""
    pix = W * H
    ch = [L, hidden, hidden, hidden, L]
    nbytes = pix * L * (4 + 2)                      # x read as FP32, written as BF16
    for i in range(4):
        nbytes += pix * ch[i] * 2                   # layer input (BF16)
        nbytes += pix * ch[i + 1] * (4 if i == 3 else 2)
    nbytes += pix * L * 4                           # residual (x, FP32)
    flops = 2 * pix * 9 * sum(ch[i] * ch[i + 1] for i in range(4))
    return nbytes, flops


def run_warmnet(args, cfg):
    """The warm-start network's forward pass (x = level costs, y = x +
    net(x)) on a 960x540x64 input -- level 1 of a 1920x1080x64 grid -- through
    the C ABI (ginf_warmnet_forward, device buffers), its four 3x3
    convolutions on tcgen05 with tensor-memory accumulators; and one training
    step (forward, loss, data and weight gradients, Adam) on a batch of 16
    level-1 inputs of 512x384 grids.  Each call synchronises, so a step's
    time includes the host's return; the per-kernel split is the ncu launch
    list's."""
    import torch
    from gridinfcuda_gb300 import capi
    torch.cuda.set_device(0)
    W, H, L = cfg["W"], cfg["H"], cfg["L"]
    net = capi.WarmNet(num_labels=L, hidden=32, seed=1)
    gen = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand((1, H, W, L), device="cuda", generator=gen) * 4
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        y = net.forward(x, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for a, b in evs:
        a.record(stream)
        y = net.forward(x, stream=stream.cuda_stream)
        b.record(stream)
    torch.cuda.synchronize()
    ms = sorted(a.elapsed_time(b) for a, b in evs)[len(evs) // 2]
    nbytes, flops = warmnet_bytes_flops(W, H, L)
    xb = torch.rand((16, 192, 256, L), device="cuda", generator=gen) * 4
    tb = xb + 0.1 * torch.rand(xb.shape, device="cuda", generator=gen)
    for _ in range(args.warmup):
        net.train_step(xb, tb, lr=1e-4, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        net.train_step(xb, tb, lr=1e-4, stream=stream.cuda_stream)
    t1.record(stream)
    torch.cuda.synchronize()
    ms_train = t0.elapsed_time(t1) / args.steps
    hbm, hbm_src = load_peaks()
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            tfl = float(json.load(f)["bf16_tflops"])
    except Exception:
        tfl = 1900.0
    achieved = nbytes / (ms / 1e3) / 1e9
    line = {"metric": "warm-start network forward, 960x540x64 (ms per call)", "value": round(ms, 4), "unit": "ms",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (fp32 accumulate)",
            "data": "synthetic (uniform inputs, seeded random weights)",
            "config": {"workload": cfg["name"], "width": W, "height": H, "labels": L, "hidden": 32,
                       "layers": "conv3x3 L->32->32->32->L, ReLU, residual", "gflop": round(flops / 1e9, 2),
                       "algorithmic_mb": round(nbytes / 1e6, 1)},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                         "frac": round(achieved / hbm, 4), "traffic": None, "peak_source": hbm_src,
                         "note": "whole forward call (5 kernels, host return included) over its algorithmic bytes"},
            "tensor_tflops": round(flops / (ms / 1e3) / 1e12, 1), "tensor_peak_tflops": tfl,
            "train_step_ms": round(ms_train, 3),
            "train_step_batch": "16 x 192x256x64 (level 1 of 512x384 grids)",
            "gpu_launches": 5}
    print(json.dumps(line), flush=True)
    net.close()


# ---------------------------------------------------------------- reference arm

def run_reference(args, cfg):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    import oracle
    oracle.build()
    P = make_problem(args.workload, cfg)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_port_step(P, cfg, threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_port_step(P, cfg, threads)
    dt = time.perf_counter() - t0
    value = args.steps * nli_per_step(cfg) / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3 / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded stereo pair, slanted planar regions; no dataset)",
            "config": bench_config(args.workload, cfg), "parallelism": "host CPU, all threads",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"full steps of the oracle C restatement of src/bp.cc + src/icm.cc + "
                                       f"src/grid.cc (the reference sources are not on this host), "
                                       f"{threads} OpenMP threads"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="hbp")
    ap.add_argument("--tile-nodes", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--train-grids", type=int, default=2000, help="warm workload: training grids")
    ap.add_argument("--eval-grids", type=int, default=256, help="warm workload: evaluation grids")
    ap.add_argument("--epochs", type=int, default=30, help="warm workload: training epochs")
    ap.add_argument("--save-net", default=None, help="warm workload: write the trained network here")
    ap.add_argument("--warm-level", type=int, default=1, help="warm workload: pyramid level the network seeds")
    ap.add_argument("--batch", type=int, default=16, help="warm workload: training batch (images)")
    ap.add_argument("--lr", type=float, default=1e-3, help="warm workload: Adam learning rate")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--retune", action="store_true", help="batch workload: re-measure the autotuner's choice")
    ap.add_argument("--sweeps-per-launch", type=int, default=0,
                    help="batch workload: half-sweeps per persistent launch (0: autotuned, with --tile-nodes 0); "
                         "single grids: most half-sweeps per cluster launch (0: default, 1: one per launch)")
    ap.add_argument("--size", default=None, help="WxH override of the workload's grid size (profiling runs)")
    ap.add_argument("--grids", type=int, default=0,
                    help="batch workload: number of grids (profiling runs; default 64)")
    args = ap.parse_args()
    if args.warmup < 3:
        print("note: the timing rules ask for at least 3 warm-up steps", file=sys.stderr)
    cfg = dict(WORKLOADS[args.workload])
    if args.size:
        w, h = (int(v) for v in args.size.lower().split("x"))
        cfg.update(W=w, H=h, name=cfg["name"].replace(f"{cfg['W']}x{cfg['H']}", f"{w}x{h}"))
    if args.grids and args.workload == "batch":
        cfg.update(count=args.grids, name=cfg["name"].replace(f"batch{cfg['count']}", f"batch{args.grids}"))
    if args.impl == "reference":
        run_reference(args, cfg)
    elif args.workload == "warm":
        import gridinfcuda_gb300
        gridinfcuda_gb300.build()
        run_warm(args, cfg)
    elif args.workload == "batch":
        import gridinfcuda_gb300
        gridinfcuda_gb300.build()
        run_batch(args, cfg)
    elif args.workload == "alphabeta":
        import gridinfcuda_gb300
        gridinfcuda_gb300.build()
        run_alphabeta(args, cfg)
    elif args.workload == "warmnet":
        import gridinfcuda_gb300
        gridinfcuda_gb300.build()
        run_warmnet(args, cfg)
    elif args.workload == "quad":
        import gridinfcuda_gb300
        gridinfcuda_gb300.build()
        run_precision(args, cfg)
    else:
        import gridinfcuda_gb300
        gridinfcuda_gb300.build()
        run_ours(args, cfg)


if __name__ == "__main__":
    main()
