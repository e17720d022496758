#!/usr/bin/env python3
"""Benchmark of the GB300 grid-MRF inference path.

Workload (default): hierarchical BP on the 1920x1080, L=64 synthetic stereo
problem -- 5 pyramid levels x 10 half-sweeps, then 5 Jacobi ICM sweeps and
the FP64 energy -- one "step" being one full solve.  Metric:
node-label-iterations per second, summed over the BP levels
(sum_t W_t*H_t*L*iterations per step).

  value     inputs resident in HBM; C-ABI ginf_solve on device buffers,
            timed with CUDA events on the stream the library runs on.
  e2e       the same call with pinned HOST buffers: the host->device copy of
            the costs and labels and the device->host copy of labels and
            energy are inside the timed region.
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
import json
import os
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
}
METRIC = "node-label-iters/s (LBP)"
UNIT = "node*label*iter/s"


def make_problem(kind, cfg, seed_offset=0):
    from gridinfcuda_gb300 import synth
    if kind == "hbp":
        return synth.workload_hbp(seed=1 + seed_offset, W=cfg["W"], H=cfg["H"])
    return synth.workload_plain_bp(seed=0 + seed_offset, W=cfg["W"], H=cfg["H"])


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


def cpu_baseline(P, cfg, nthreads):
    import oracle
    oracle.build()
    t0 = time.perf_counter()
    cpu_port_step(P, cfg, nthreads)
    dt = time.perf_counter() - t0
    return {"value": nli_per_step(cfg) / dt, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"one full step ({cfg['name']}) of the oracle C restatement, {nthreads} OpenMP threads, "
                      f"{dt:.2f} s"}


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
    opt = dict(stream=stream.cuda_stream, tile_nodes=args.tile_nodes)

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
    barrier(world)
    ms = reduce_max(ev0.elapsed_time(ev1), world, dev)
    nli = stats[0]["node_label_iters"]
    value = world * args.steps * nli / (ms / 1e3)
    launches = reduce_sum(sum(s["kernel_launches"] for s in stats), world, dev)

    # Roofline of the finest-level half-sweep (the dominant kernel).
    l0_ms = sum(s["level0_sweep_ms"] for s in stats) / len(stats)
    l0_launches = stats[0]["level0_sweep_launches"]
    per_launch_s = l0_ms / l0_launches / 1e3
    W, H, L = cfg["W"], cfg["H"], cfg["L"]
    alg_bytes = (W - 2) * (H - 2) / 2 * 9 * L * 4   # updated nodes x 9L floats per launch
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / per_launch_s / 1e9
    traffic = load_traffic(cfg)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
                "kernel": "sweep_kernel<float,float,64,...> (finest level)",
                "algorithmic_bytes_per_launch": alg_bytes, "mean_launch_ms": round(per_launch_s * 1e3, 4)}

    # End to end through the C ABI with pinned host buffers.
    Dh = torch.from_numpy(P.D).pin_memory()
    Vh = torch.from_numpy(P.V).pin_memory()
    labh = torch.zeros((cfg["H"], cfg["W"]), dtype=torch.int32).pin_memory()

    def step_host():
        return capi.solve(Dh, Vh, P.model, cfg["levels"], cfg["iters"], cfg["icm"], labels=labh, workspace=ws,
                          want_stats=True, **opt)

    for _ in range(max(1, min(args.warmup, 2))):
        step_host()
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    est = None
    for _ in range(args.steps):
        _, _, est = step_host()
    torch.cuda.synchronize()
    e2e_s = reduce_max(time.perf_counter() - t0, world, dev)
    e2e = {"value": world * args.steps * nli / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(est["h2d_bytes"]),
           "d2h_bytes_per_step": int(est["d2h_bytes"]), "ms_per_step": round(e2e_s * 1e3 / args.steps, 3)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(P, cfg, os.cpu_count() or 1)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded stereo pair, slanted planar regions; no dataset)",
                "config": {"workload": cfg["name"], "width": W, "height": H, "labels": L,
                           "levels": cfg["levels"], "iters_per_level": cfg["iters"], "icm_sweeps": cfg["icm"],
                           "smoothness": "min(|a-b|, 4)" if args.workload == "hbp" else "min(|a-b|, 1.7)",
                           "node_label_iters_per_step": nli, "parallelism": f"replicas x{world}",
                           "l2": f"inputs larger than L2 (costs {W * H * L * 4 / 1e6:.0f} MB, "
                                 f"records {W * H * L * 20 * 4 / 3 / 1e9:.2f} GB)"},
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clock_info,
                "gpu_launches": int(launches), "energy": energy,
                "phases_ms": {k: round(stats[-1][k], 4) for k in ("upload_ms", "prepare_ms", "sweep_ms",
                                                                  "level0_sweep_ms", "icm_ms", "energy_ms",
                                                                  "download_ms", "total_ms")}}
        print(json.dumps(line), flush=True)
    ws.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


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
            "config": {"workload": cfg["name"], "width": cfg["W"], "height": cfg["H"], "labels": cfg["L"],
                       "levels": cfg["levels"], "iters_per_level": cfg["iters"], "icm_sweeps": cfg["icm"],
                       "parallelism": "host CPU, all threads"},
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
    ap.add_argument("--size", default=None, help="WxH override of the workload's grid size (profiling runs)")
    args = ap.parse_args()
    if args.warmup < 3:
        print("note: the timing rules ask for at least 3 warm-up steps", file=sys.stderr)
    cfg = dict(WORKLOADS[args.workload])
    if args.size:
        w, h = (int(v) for v in args.size.lower().split("x"))
        cfg.update(W=w, H=h, name=cfg["name"].replace(f"{cfg['W']}x{cfg['H']}", f"{w}x{h}"))
    if args.impl == "reference":
        run_reference(args, cfg)
    else:
        import gridinfcuda_gb300
        gridinfcuda_gb300.build()
        run_ours(args, cfg)


if __name__ == "__main__":
    main()
