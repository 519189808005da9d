"""Benchmark of the 3D DG advection hot path on one GB300 (or N replicas).

Workload: the periodic unit box, Ne = 32^3 hexahedra of order p = 7
(512 nodes each, 16.8M DOF), seeded Gaussian tracer (sigma 0.1) in a seeded
smooth velocity field, SSP-RK3 with dt at CFL 0.1, FP64 plain form.  One
"step" is one SSP-RK3 time step of the whole box (three fused stage kernels).

Metric: GDOF-updates/s = Np * Ne * 3 * steps / t / 1e9 (one DOF-update is one
DOF advanced through one RK stage).  `value` is timed with CUDA events on the
solver's stream with the state resident in HBM; `e2e` goes through the C ABI
with pinned host buffers (upload q,u,v,w, one step, download q, every step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With --impl reference the CPU oracle (a C + OpenMP restatement of the
reference's Fortran path; the Fortran reference cannot be built here) is timed
on the host cores on the same workload.  Under torchrun with N > 1 every rank
runs an independent replica (the spec path is single-GPU); rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "scale-dg-kernel-extraction_gb300")
sys.path.insert(0, PKG)

# algorithmic bytes per DOF-update: stage 1 reads q,u,v,w and writes q (40 B);
# stages 2 and 3 also read q0 (48 B).  FP32 form: velocity in FP32.
BYTES_PER_DOF_UPDATE = {"fp64": 136.0 / 3.0, "fp32": 100.0 / 3.0}


def flops_per_dof_update(p: int) -> float:
    """flux products 3, contractions 6 Nq, combine 6, lift 11, RK 5, and 21 per
    face node times 6/Nq face nodes per DOF."""
    nq = p + 1
    return 25.0 + 6.0 * nq + 126.0 / nq


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def make_workload(p: int, ne: int, seed: int):
    import sdg
    import workloads as W
    x, D, Dt, L = sdg.operator_generate(p)
    q, u, v, w = W.blob(ne, ne, ne, x, seed)
    dt = W.cfl_dt(ne, ne, ne, p, u, v, w)
    return dict(x=x, D=D, Dt=Dt, L=L, q=q, u=u, v=v, w=w, dt=dt)


def time_oracle(wl, p, ne, min_seconds: float, max_steps: int, warmup: int = 0):
    """Runs the oracle (C + OpenMP) step by step; returns (steps, seconds, threads)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    import workloads as W
    m = O.Mesh(ne, ne, ne, p, wl["x"])
    arrs = [W.with_halo(a, m.NeA, m.Np) for a in (wl["q"], wl["u"], wl["v"], wl["w"])]
    for a in arrs:
        m.update_halo(a)
    q = arrs[0]
    for _ in range(warmup):
        O.run(m, q, arrs[1], arrs[2], arrs[3], wl["D"], wl["Dt"], wl["L"], wl["dt"], 1, O.OPT1)
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps:
        O.run(m, q, arrs[1], arrs[2], arrs[3], wl["D"], wl["Dt"], wl["L"], wl["dt"], 1, O.OPT1)
        steps += 1
        if time.perf_counter() - t0 >= min_seconds:
            break
    return steps, time.perf_counter() - t0, O.num_threads()


def load_traffic(key: str):
    path = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    v = d.get(key)
    return float(v["bytes_per_launch"]) if isinstance(v, dict) else None


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    wl = make_workload(args.p, args.ne, args.seed)
    ndof = (args.p + 1) ** 3 * args.ne ** 3
    # warm-up steps, then K timed steps of the same workload
    steps, secs, threads = time_oracle(wl, args.p, args.ne, 0.0, args.steps, args.warmup)
    v = ndof * 3 * steps / secs / 1e9
    line = {
        "impl": "reference",
        "metric": metric_name(args), "value": v, "unit": "GDOF-updates/s", "n_gpus": ws,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Gaussian tracer, seeded smooth velocity)",
        "config": config(args),
        "cpu_baseline": {"value": v, "unit": "GDOF-updates/s", "cores": threads, "kind": "port",
                         "sample": f"{steps} SSP-RK3 steps of the full {args.ne}^3 p={args.p} box "
                                   "(C + OpenMP restatement of the Fortran reference; "
                                   "the reference itself has no compiler here)"},
        "e2e": {"value": v, "unit": "GDOF-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def metric_name(args) -> str:
    return f"GDOF-updates/s (p={args.p}, {args.ne}^3, {'FP64' if args.precision == 'fp64' else 'FP32-compute/FP64-state'})"


def config(args) -> dict:
    ndof = (args.p + 1) ** 3 * args.ne ** 3
    ws_bytes = ndof * (8 * 3 + (24 if args.precision == "fp64" else 12))
    return {"workload": f"3D DG advection, periodic unit box, Ne={args.ne}^3, p={args.p}, "
                        f"SSP-RK3, CFL 0.1, {args.precision} plain form",
            "p": args.p, "Ne": [args.ne] * 3, "dof": ndof, "opt": "OPT1",
            "precision": args.precision,
            "l2": f"inputs larger than L2 (state+velocity working set {ws_bytes / 1e6:.0f} MB "
                  "vs 129 MB L2)",
            "parallelism": "replicas (one independent box per GPU)"}


def run_ours(args, ws, rank, local):
    import sdg
    if sdg.device_count() < 1:
        raise SystemExit("bench.py: no CUDA device")
    sdg.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist  # plumbing for the barrier and the max only
        dist.init_process_group("gloo")

    def barrier():
        if dist is not None:
            dist.barrier()

    p, ne = args.p, args.ne
    prec = sdg.PREC_FP64 if args.precision == "fp64" else sdg.PREC_FP32
    wl = make_workload(p, ne, args.seed + rank)
    ndof = (p + 1) ** 3 * ne ** 3
    s = sdg.Solver(ne, ne, ne, p, wl["D"], wl["L"], opt=sdg.OPT_OPT1, precision=prec)
    s.upload(wl["q"], wl["u"], wl["v"], wl["w"])
    s.step(wl["dt"], args.warmup)
    sdg.synchronize()

    # ---- device-resident timing (CUDA events on the solver's stream) ----
    clocks = ClockSampler(local)
    barrier()
    sdg.synchronize()
    clocks.start()
    time.sleep(0.3)  # let the sampler start
    t_wall0 = time.perf_counter()
    ms = s.step_timed(wl["dt"], args.steps)
    sdg.synchronize()
    t_wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    barrier()
    t = ms / 1e3
    if dist is not None:
        import torch
        tt = torch.tensor([t], dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    value = ws * ndof * 3 * args.steps / t / 1e9
    per_gpu = ndof * 3 * args.steps / t / 1e9

    # ---- roofline of the fused stage kernel (the only kernel in a step) ----
    launches = 3 * args.steps
    avg_launch = t / launches
    bpd = BYTES_PER_DOF_UPDATE[args.precision]
    achieved = bpd * ndof / avg_launch / 1e9
    peak, peak_kind = measured_peaks()
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
            "algorithmic_bytes_per_dof_update": bpd,
            "traffic": load_traffic(f"stage_{args.precision}_p{p}_ne{ne}"),
            "kernel": f"stage_kernel<{p},{'double' if prec == 0 else 'float'}>",
            "avg_launch_ms": avg_launch * 1e3}
    fl = flops_per_dof_update(p)
    pk = sdg.microbench_peaks()
    pipe = "dfma_tflops" if args.precision == "fp64" else "ffma_tflops"
    roof["compute"] = {"pipe": "FP64 (DFMA)" if args.precision == "fp64" else "FP32 (FFMA)",
                       "flops_per_dof_update": fl, "achieved_tflops": fl * per_gpu / 1e3,
                       "peak_tflops_measured_live": pk[pipe],
                       "frac": fl * per_gpu / 1e3 / pk[pipe]}

    # ---- end to end through the C ABI with pinned host buffers ----
    e2e = None
    if not args.no_e2e:
        pins = [sdg.PinnedArray(ndof) for _ in range(5)]
        for pa, src in zip(pins, (wl["q"], wl["u"], wl["v"], wl["w"])):
            pa.array[:] = src
        k = max(1, min(args.steps, args.e2e_steps))
        # one untimed round trip
        s.upload_ptrs(*(pa.ptr for pa in pins[:4]))
        s.step(wl["dt"], 1)
        s.download_ptr(pins[4].ptr)
        barrier()
        t0 = time.perf_counter()
        for _ in range(k):
            s.upload_ptrs(*(pa.ptr for pa in pins[:4]))
            s.step(wl["dt"], 1)
            s.download_ptr(pins[4].ptr)  # synchronises the stream
        te = time.perf_counter() - t0
        if dist is not None:
            import torch
            tt = torch.tensor([te], dtype=torch.float64)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            te = float(tt.item())
        e2e = {"value": ws * ndof * 3 * k / te / 1e9, "unit": "GDOF-updates/s",
               "h2d_bytes_per_step": 4 * 8 * ndof, "d2h_bytes_per_step": 8 * ndof,
               "steps": k, "path": "sdg_solver_upload + sdg_solver_step + sdg_solver_download"}
        for pa in pins:
            pa.free()
    s.close()

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0

    cpu = None
    if ws == 1 and not args.no_cpu_baseline:
        steps, secs, threads = time_oracle(wl, p, ne, args.cpu_seconds, 10 ** 6)
        cpu = {"value": ndof * 3 * steps / secs / 1e9, "unit": "GDOF-updates/s", "cores": threads,
               "kind": "port",
               "sample": f"{steps} SSP-RK3 steps of the same {ne}^3 p={p} box in FP64 "
                         f"({secs:.1f} s; C + OpenMP restatement of the Fortran reference)"}
    line = {
        "metric": metric_name(args), "value": value, "unit": "GDOF-updates/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32-compute/f64-state",
        "data": "synthetic (seeded Gaussian tracer, seeded smooth velocity)",
        "config": config(args), "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": launches, "clocks": clk, "wall_s_timed_region": t_wall,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--p", type=int, default=7)
    ap.add_argument("--ne", type=int, default=32)
    ap.add_argument("--precision", choices=["fp64", "fp32"], default="fp64")
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    return run_ours(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
