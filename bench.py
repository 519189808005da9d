"""Benchmark of the 3D DG advection hot path on one GB300 (or N replicas).

Workload: the periodic unit box, Ne = 32^3 hexahedra of order p = 7
(512 nodes each, 16.8M DOF), the reference's own operators
(operator_data/p7.dat), seeded Gaussian tracer (sigma 0.1) in a seeded smooth
velocity field, SSP-RK3 with dt at CFL 0.1, FP64 plain form.  One "step" is
one SSP-RK3 time step of the whole box (three fused stage kernels).

Metric: GDOF-updates/s = Np * Ne * 3 * steps / t / 1e9 (one DOF-update is one
DOF advanced through one RK stage).  `value` is timed with CUDA events on the
solver's stream with the state resident in HBM; `e2e` goes through the C ABI
with pinned host buffers (upload q,u,v,w, one step, download q, every step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--results FILE]

Output: the secondary measurements (emulated FP64, the per-stage drop-in
path, standalone operators, the batched ensemble, serving, the order sweep)
are printed first, one JSON line each with a "section" key; the LAST line is
the compact headline (metric, value, e2e, roofline, cpu_baseline, clocks,
parity and a serving / ensemble summary).  --results also writes every line
to one JSON file.

With --impl reference the CPU oracle (a C + OpenMP restatement of the
reference's Fortran path, which has no Fortran compiler to build it with) is
timed on the host cores on the same workload, through its timing build
(-O3 -fopenmp, multiply-add contraction, -mcpu=native on aarch64); that arm
loads only the oracle.  Under torchrun with N > 1 every rank runs an
independent replica (the path is built for one GPU and exchanges nothing
between boxes); rank 0 prints.
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
BYTES_PER_DOF_UPDATE = {"fp64": 136.0 / 3.0, "fp64emu": 136.0 / 3.0, "fp32": 100.0 / 3.0}


def face_factor_bytes(precision: str, opt: str, p: int) -> float:
    """Bytes per DOF-update of the face-flux velocity factors the even-odd FP64
    and emulated-FP64 stages share within a step: stage 1 writes (tP, tM) for
    the 6 Nq^2 face nodes of each element (96/Nq B a DOF), stages 2 and 3 read
    them, so every launch moves 96/Nq B a DOF."""
    return 96.0 / (p + 1) if opt == "evenodd" and precision in ("fp64", "fp64emu") else 0.0
PRECISIONS = {"fp64": 0, "fp32": 1, "fp64emu": 2}


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
    """The bench box on the reference's own operators (operator_data/p{p}.dat,
    the committed bit-exact fixture); numpy only, so that the reference arm
    loads nothing of the product."""
    import workloads as W
    x, D, Dt, L = W.reference_operators(p)
    q, u, v, w = W.blob(ne, ne, ne, x, seed)
    dt = W.cfl_dt(ne, ne, ne, p, u, v, w)
    return dict(x=x, D=D, Dt=Dt, L=L, q=q, u=u, v=v, w=w, dt=dt)


class OracleBox:
    """The CPU oracle (C + OpenMP) set up on the bench workload: mesh arrays,
    fields with halos, the tendency of the initial state, and timed steps."""

    def __init__(self, wl, p, ne):
        # the reference's OpenMP settings for a timed CPU run: one thread per
        # core, bound close (read when the oracle library starts OpenMP)
        os.environ.setdefault("OMP_PROC_BIND", "close")
        os.environ.setdefault("OMP_PLACES", "cores")
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        import workloads as W
        self.O, self.wl = O, wl
        self.m = O.Mesh(ne, ne, ne, p, wl["x"])
        self.arrs = [W.with_halo(a, self.m.NeA, self.m.Np)
                     for a in (wl["q"], wl["u"], wl["v"], wl["w"])]
        for a in self.arrs:
            self.m.update_halo(a)
        self.threads = O.num_threads()

    def tendency(self):
        m = self.m
        return self.O.cal_tend(m, *self.arrs, self.wl["D"], self.wl["Dt"], self.wl["L"],
                               self.O.OPT1)[: m.Np * m.Ne]

    def time_steps(self, min_seconds: float, max_steps: int, warmup: int = 0):
        """Steps a copy of the state in the reference's OPT1 order through the
        oracle's timing build (contraction allowed, -mcpu=native on aarch64,
        all host cores); returns (steps, seconds)."""
        O, wl, m = self.O, self.wl, self.m
        q = self.arrs[0].copy()
        args = (self.arrs[1], self.arrs[2], self.arrs[3], wl["D"], wl["Dt"], wl["L"], wl["dt"])
        for _ in range(warmup):
            O.run(m, q, *args[:3], *args[3:6], args[6], 1, O.OPT1, fast=True)
        steps, t0 = 0, time.perf_counter()
        while steps < max_steps:
            O.run(m, q, *args[:3], *args[3:6], args[6], 1, O.OPT1, fast=True)
            steps += 1
            if time.perf_counter() - t0 >= min_seconds:
                break
        return steps, time.perf_counter() - t0


def load_traffic(key: str, field: str = "bytes_per_launch"):
    """A figure of one kernel's ncu capture (profiles/dram_traffic.json)."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    v = d.get(key)
    return float(v[field]) if isinstance(v, dict) and field in v else None


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    wl = make_workload(args.p, args.ne, args.seed)
    ndof = (args.p + 1) ** 3 * args.ne ** 3
    # warm-up steps, then K timed steps of the same workload
    ob = OracleBox(wl, args.p, args.ne)
    steps, secs = ob.time_steps(float("inf"), args.steps, args.warmup)
    threads = ob.threads
    v = ndof * 3 * steps / secs / 1e9
    line = {
        "impl": "reference",
        "metric": metric_name(args), "value": v, "unit": "GDOF-updates/s", "n_gpus": ws,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Gaussian tracer, seeded smooth velocity)",
        "config": config(args, reference=True),
        "cpu_baseline": {"value": v, "unit": "GDOF-updates/s", "cores": threads, "kind": "port",
                         "sample": f"{steps} SSP-RK3 steps of the full {args.ne}^3 p={args.p} box, "
                                   "OPT1 order (C + OpenMP restatement of the Fortran reference, "
                                   "timing build; no Fortran compiler for the reference itself)"},
        "e2e": {"value": v, "unit": "GDOF-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


PREC_LABEL = {"fp64": "FP64", "fp64emu": "FP64 state, double-float arithmetic",
              "fp32": "FP32-compute/FP64-state"}


def metric_name(args) -> str:
    return f"GDOF-updates/s (p={args.p}, {args.ne}^3, {PREC_LABEL[args.precision]})"


def config(args, reference: bool = False) -> dict:
    """The workload's description.  The reference arm times the reference's
    OPT1 order; ours names the order its stage kernel sums in."""
    ndof = (args.p + 1) ** 3 * args.ne ** 3
    ws_bytes = ndof * (8 * 3 + (12 if args.precision == "fp32" else 24))
    return {"workload": f"3D DG advection, periodic unit box, Ne={args.ne}^3, p={args.p}, "
                        f"SSP-RK3, CFL 0.1, {args.precision} plain form",
            "p": args.p, "Ne": [args.ne] * 3, "dof": ndof,
            "opt": "OPT1" if reference else args.opt.upper(),
            "precision": "fp64" if reference else args.precision,
            "operators": f"reference operator_data/p{args.p}.dat",
            "l2": f"inputs > L2 ({ws_bytes / 1e6:.0f} MB working set, 129 MB L2)",
            "parallelism": "replicas"}


OPTS = {"general": 1, "opt1": 2, "evenodd": 3}


def time_solver(sdg, wl, p, ne, prec, steps, warmup, local, barrier, sample_clocks,
                opt=OPTS["opt1"]):
    """Uploads the workload, warms up, and times `steps` steps with CUDA events
    on the solver's stream.  Returns (solver, seconds, clocks)."""
    s = sdg.Solver(ne, ne, ne, p, wl["D"], wl["L"], opt=opt, precision=prec)
    s.upload(wl["q"], wl["u"], wl["v"], wl["w"])
    s.step(wl["dt"], warmup)
    sdg.synchronize()
    clocks = ClockSampler(local) if sample_clocks else None
    barrier()
    if clocks:
        clocks.start()
        time.sleep(0.3)  # let the sampler start
    ms = s.step_timed(wl["dt"], steps)
    sdg.synchronize()
    clk = clocks.stop() if clocks else None
    barrier()
    return s, ms / 1e3, clk


def roofline(precision, p, ne, ndof, t, steps, peaks, opt="opt1"):
    """The stage kernel against its roofs.

    HBM: achieved = the algorithmic bytes per DOF-update (45.33 B FP64 and
    emulated, 33.33 B FP32: state, velocity and the RK buffers) x the DOF of
    one launch / the average launch time (3 launches a step, nothing else in
    the step).  The face-flux velocity factors the even-odd FP64 and emulated
    stages share within a step are implementation bytes, reported beside it
    (`implementation_bytes_per_dof_update`) and not counted.  `traffic` is
    the ncu DRAM bytes per launch of the same kernel.

    Compute: the FP64 pipe binds the FP64 forms (1.2 TFLOP/s DFMA against
    88.75 flops a DOF-update at p = 7).  `compute.frac` is that pipe's busy
    share from the kernel's ncu capture (sm__pipe_fp64_cycles_active);
    `achieved_tflops` counts the reference's formulas (25 + 6 Nq + 126 / Nq
    flops a DOF-update) against the DFMA peak measured live.  The FP32 and
    emulated forms report those flops against the live FFMA peak, and the
    emulated form its FP64 pipe's busy share apart (`fp64_pipe_busy`)."""
    launches = 3 * steps
    avg_launch = t / launches
    bpd = BYTES_PER_DOF_UPDATE[precision]
    impl = face_factor_bytes(precision, opt, p)
    achieved = bpd * ndof / avg_launch / 1e9
    peak, peak_kind = measured_peaks()
    per_gpu = ndof * 3 * steps / t / 1e9
    fl = flops_per_dof_update(p)
    pipe = "dfma_tflops" if precision == "fp64" else "ffma_tflops"
    kernel = {"fp64": f"stage_kernel<{p},double>", "fp32": f"stage_kernel<{p},float>",
              "fp64emu": f"stage_emu_kernel<{p}>"}[precision]
    tkey = f"stage_{precision}_p{p}_ne{ne}"
    if precision == "fp64" and opt == "evenodd":
        kernel, tkey = f"stage_eo_kernel<{p},double>", f"stage_fp64eo_p{p}_ne{ne}"
    elif precision == "fp64emu" and opt == "evenodd":
        kernel, tkey = f"stage_emu_eo_kernel<{p}>", f"stage_fp64emueo_p{p}_ne{ne}"
    elif precision == "fp32" and opt == "evenodd":
        # the single box's own kernels at the lowest orders (same arithmetic)
        k32 = {1: "stage_p1_kernel", 2: "stage_col_kernel<2>", 3: "stage_p3_kernel"}
        kernel = k32.get(p, f"stage_eo_kernel<{p},float>")
        tkey = f"stage_fp32eo_p{p}_ne{ne}"
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak,
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
            "algorithmic_bytes_per_dof_update": bpd,
            "implementation_bytes_per_dof_update": impl,
            "traffic": load_traffic(tkey),
            "kernel": kernel, "avg_launch_ms": avg_launch * 1e3}
    if peaks is not None:
        comp = {"pipe": "FP64 (DFMA)" if precision == "fp64" else "FP32 (FFMA)",
                "flops_per_dof_update": fl,
                "achieved_tflops": fl * per_gpu / 1e3,
                "peak_tflops_measured_live": peaks[pipe]}
        busy = load_traffic(tkey, "fp64_pipe_active")
        if busy is not None and precision == "fp64":
            comp["frac"] = busy
            comp["frac_source"] = "sm__pipe_fp64_cycles_active, ncu capture of this kernel"
        else:
            comp["frac"] = fl * per_gpu / 1e3 / peaks[pipe]
            comp["frac_source"] = "reference-formula flops / live peak"
            if busy is not None:
                # the emulated form's FP64 work (face flux, RK combine) on
                # the 1/64-rate pipe, beside its FP32 contraction
                comp["fp64_pipe_busy"] = busy
                comp["fp64_pipe_busy_source"] = ("sm__pipe_fp64_cycles_active, ncu capture "
                                                 "of this kernel")
        roof["compute"] = comp
        if precision == "fp64":
            # the FP64 pipe binds when it is busier than HBM
            roof["binding_roof"] = "fp64_pipe" if comp["frac"] > roof["frac"] else "hbm"
    return roof


def ensemble_workload(n, seed):
    """The batched-ensemble config: n instances, Ne per axis uniform in 4..24
    independently per axis, p in {3,5,7}, Gaussian width uniform in
    [0.05, 0.2], constant velocity of magnitude uniform in [0, 1] in a uniform
    random direction, dt at CFL 0.1; drawn with splitmix64."""
    import math
    import workloads as W
    members = []
    for i in range(n):
        r = W.SplitMix64(seed + i)
        dims = tuple(r.randint(4, 24) for _ in range(3))
        p = (3, 5, 7)[r.randint(0, 2)]
        sigma = 0.05 + 0.15 * r.uniform()
        centre = [r.uniform() for _ in range(3)]
        ct = 2.0 * r.uniform() - 1.0
        ph = 2.0 * math.pi * r.uniform()
        st = math.sqrt(max(0.0, 1.0 - ct * ct))
        mag = r.uniform()
        vel = (mag * st * math.cos(ph), mag * st * math.sin(ph), mag * ct)
        vsum = max(sum(abs(x) for x in vel), 1e-3)
        dt = 0.1 * min(1.0 / d for d in dims) / ((2 * p + 1) * vsum)
        members.append(dict(dims=dims, p=p, sigma=sigma, centre=centre, vel=vel, dt=dt))
    return members


def bench_ensemble(sdg, args):
    import workloads as W
    members = ensemble_workload(args.ens_n, args.seed + 1000)
    ops = {p: W.reference_operators(p) for p in (3, 5, 7)}
    t0 = time.perf_counter()
    ens = sdg.Ensemble([m["dims"] for m in members], [m["p"] for m in members],
                       [m["dt"] for m in members], ops)
    if args.batch_opt != "auto":
        ens.set_opt(OPTS[args.batch_opt])
    ens.set_parallel_groups(args.parallel_groups)
    for i, m in enumerate(members):
        ens.init_blob(i, m["centre"], m["sigma"], m["vel"])
    sdg.synchronize()
    # initial states of a few members, for the FP64 comparison below
    sample = list(range(0, args.ens_n, max(1, args.ens_n // 6)))[:6]
    q0 = {i: ens.download(i) for i in sample}
    cfg = ens.tune()
    ens.step(args.warmup)
    sdg.synchronize()
    nst = args.ens_steps - args.warmup
    ms = ens.step_timed(nst)
    t = ms / 1e3
    dof = ens.total_dofs
    # the plain FP64 path on the same members (sequential solves), measured
    # on the sample and scaled by DOF count
    plain_t, plain_dof, errs, drift = 0.0, 0, [], []
    for i in sample:
        m = members[i]
        x, D, Dt, L = ops[m["p"]]
        s = sdg.Solver(*m["dims"], m["p"], D, L, opt=OPTS[args.opt], precision=sdg.PREC_FP64)
        n = q0[i].size
        s.upload(q0[i], np.full(n, m["vel"][0]), np.full(n, m["vel"][1]), np.full(n, m["vel"][2]))
        plain_t += s.step_timed(m["dt"], args.ens_steps) / 1e3
        plain_dof += n
        ref = s.download()
        s.close()
        got = ens.download(i)
        # members ran warmup + timed = ens_steps steps
        errs.append(float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
        m0 = W.mass(q0[i], x, *m["dims"])
        drift.append(abs(W.mass(got, x, *m["dims"]) - m0) / abs(m0))
    launches = ens.launches_per_step()
    # the same members with ONE persistent launch per RK stage over every order
    ens.set_single_launch(True)
    ens.step(args.warmup)
    sdg.synchronize()
    t1 = ens.step_timed(nst) / 1e3
    launches1 = ens.launches_per_step()
    ens.close()
    per_solve = t / nst * args.ens_steps
    plain_per_solve = plain_t / plain_dof * dof  # all members, sequentially
    return {
        "workload": f"{args.ens_n} instances, Ne per axis U{{4..24}}, p in {{3,5,7}}, "
                    f"sigma U[0.05,0.2], constant |u|<=1, {args.ens_steps} steps, "
                    "FP32 compute / FP64 RK state, one launch per order and stage, "
                    "CUDA graph",
        "total_dof": dof,
        "solves_per_s": args.ens_n / per_solve,
        "gdof_updates_per_s": dof * 3 * nst / t / 1e9,
        "hbm_frac": dof * 3 * nst * BYTES_PER_DOF_UPDATE["fp32"] / t / 1e9 / measured_peaks()[0],
        "plain_fp64_solves_per_s": args.ens_n / plain_per_solve,
        "ratio_vs_plain": plain_per_solve / per_solve,
        "rel_l2_vs_fp64_max": max(errs), "mass_drift_max": max(drift),
        "autotuned": cfg, "launches_per_step": launches,
        "single_launch_per_stage": {"solves_per_s": args.ens_n / (t1 / nst * args.ens_steps),
                                    "launches_per_step": launches1,
                                    "ratio_to_per_order_launches": t / t1},
        "setup_s": time.perf_counter() - t0,
    }


def bench_order_sweep(sdg, args):
    """Orders 1..15 at about 16.8M DOF (Ne per axis = round(256/(p+1))), the
    seeded blob workload, nstep steps: throughput of the FP64 (OPT1 order and
    even-odd body), emulated-FP64 and FP32 (node and even-odd body) forms, and the relative L2 error and mass drift of the latter two
    against the FP64 form (which matches the CPU oracle to 1e-12 per
    tendency, tested)."""
    import workloads as W
    out = []
    for p in range(1, 16):
        ne = int(round(256.0 / (p + 1)))
        x, D, Dt, L = W.reference_operators(p)
        q, u, v, w = W.blob(ne, ne, ne, x, args.seed + p)
        dt = W.cfl_dt(ne, ne, ne, p, u, v, w)
        ndof = q.size
        m0 = W.mass(q, x, ne, ne, ne)
        row = {"p": p, "Ne": ne, "dof": ndof, "nstep": args.sweep_steps}
        res = {}
        for name, prec, opt in (("fp64", sdg.PREC_FP64, sdg.OPT_OPT1),
                                ("fp64eo", sdg.PREC_FP64, sdg.OPT_EVENODD),
                                ("fp64emu", sdg.PREC_FP64_EMU, sdg.OPT_OPT1),
                                ("fp64emueo", sdg.PREC_FP64_EMU, sdg.OPT_EVENODD),
                                ("fp32", sdg.PREC_FP32, sdg.OPT_OPT1),
                                ("fp32eo", sdg.PREC_FP32, sdg.OPT_EVENODD)):
            s = sdg.Solver(ne, ne, ne, p, D, L, opt=opt, precision=prec)
            s.upload(q, u, v, w)
            ms = s.step_timed(dt, args.sweep_steps)
            res[name] = s.download()
            s.close()
            row[f"{name}_gdof_updates_per_s"] = ndof * 3 * args.sweep_steps / (ms / 1e3) / 1e9
            row[f"{name}_mass_drift"] = abs(W.mass(res[name], x, ne, ne, ne) - m0) / abs(m0)
        ref = res["fp64"]
        for name in ("fp64eo", "fp64emu", "fp64emueo", "fp32", "fp32eo"):
            row[f"{name}_rel_l2_vs_fp64"] = float(np.linalg.norm(res[name] - ref) /
                                                  np.linalg.norm(ref))
        out.append(row)
    return out


def bench_operators(sdg, args, peaks, reps=30):
    """The reference's standalone operator entry points on device arrays over
    the bench box's elements (Ne^3 blocks of Nq^3 values, inputs larger than
    L2): tensorprod_divlike_dirXYZ (OPT1 and GENERAL orders), gradlike,
    divlike_var5 (5 variables a node), element matvec, Lift_hexahedral,
    update_halo and the device mesh build.  Each is queued `reps` times on one
    stream and timed on the host with a synchronize on both sides (calls of
    0.1-3 ms, so the launch cost is a few per cent at most).  Bytes are the
    arrays each call must read and write once (FP64), flops its
    multiply-adds x 2."""
    lib, A = sdg.lib, sdg.DeviceArray
    p, ne = args.p, args.ne
    nq, np_ = p + 1, (p + 1) ** 3
    ne3 = ne ** 3
    n = np_ * ne3
    ntf = 6 * nq * nq
    nhalo = 6 * ne * ne
    nhn = nq * nq * nhalo
    rng = np.random.default_rng(args.seed + 5)
    import workloads as W
    x1, D, Dt, L = W.reference_operators(p)
    Dd, Dtd, Ld = A(D), A(Dt), A(L)
    hbm = measured_peaks()[0]
    dfma = peaks["dfma_tflops"] if peaks else None

    def timed(fn, k=reps):
        fn()
        sdg.synchronize()
        t0 = time.perf_counter()
        for _ in range(k):
            fn()
        sdg.synchronize()
        return (time.perf_counter() - t0) / k

    out = {"workload": f"{ne}^3 elements of order {p} ({n} nodes a field), device arrays, "
                       f"{reps} queued calls each, host-timed with a synchronize on both sides",
           "operators": {}}

    def record(name, fn, nbytes, flops, ref):
        t = timed(fn)
        row = {"ms_per_call": t * 1e3, "gbs": nbytes / t / 1e9, "hbm_frac": nbytes / t / 1e9 / hbm,
               "bytes_per_call": nbytes, "ref": ref}
        if flops:
            row["gflops"] = flops / t / 1e9
            if dfma:
                row["fp64_pipe_frac"] = flops / t / 1e12 / dfma
        out["operators"][name] = row

    fin = [A(rng.standard_normal(n)) for _ in range(3)]
    fout = [A(n=n) for _ in range(3)]
    chk = sdg._check
    for opt, oname in ((sdg.OPT_OPT1, "OPT1"), (sdg.OPT_GENERAL, "GENERAL")):
        record(f"tensorprod_divlike_dirXYZ ({oname})",
               lambda opt=opt: chk(lib.sdg_tensorprod_divlike_dirXYZ_dev(
                   fout[0].ptr, fout[1].ptr, fout[2].ptr, Dd.ptr, Dtd.ptr, fin[0].ptr,
                   fin[1].ptr, fin[2].ptr, nq, ne3, opt, None), "divlike"),
               48 * n, 6 * nq * n, "mod_dg_optr_kernel.f90:62-136")
    record("tensorprod_gradlike_dirXYZ",
           lambda: chk(lib.sdg_tensorprod_gradlike_dirXYZ_dev(
               fout[0].ptr, fout[1].ptr, fout[2].ptr, Dd.ptr, Dtd.ptr, fin[0].ptr, nq, ne3,
               None), "gradlike"),
           32 * n, 6 * nq * n, "opt1 erb:166-219")
    record("element_matvec_dir (z)",
           lambda: chk(lib.sdg_element_matvec_dir_dev(3, fout[0].ptr, Dtd.ptr, fin[0].ptr, nq,
                                                      ne3, None), "matvec"),
           16 * n, 2 * nq * n, "opt1 erb:51-129")
    lin = A(rng.standard_normal(ntf * ne3))
    record("tensorprod_Lift_hexahedral",
           lambda: chk(lib.sdg_tensorprod_Lift_hexahedral_dev(fout[0].ptr, Ld.ptr, lin.ptr, nq,
                                                              ne3, None), "lift"),
           8 * (n + ntf * ne3), 12 * n, "mod_dg_optr_kernel.f90:139-190")
    del fin, fout, lin
    # five variables a node: 3 inputs and 3 outputs of 5 n values
    ne5 = max(1, ne3 // 5)
    n5 = 5 * np_ * ne5
    vin = [A(rng.standard_normal(n5)) for _ in range(3)]
    vout = [A(n=n5) for _ in range(3)]
    record("tensorprod_divlike_dirXYZ_var5",
           lambda: chk(lib.sdg_tensorprod_divlike_dirXYZ_var5_dev(
               vout[0].ptr, vout[1].ptr, vout[2].ptr, Dd.ptr, Dtd.ptr, vin[0].ptr, vin[1].ptr,
               vin[2].ptr, nq, ne5, None), "var5"),
           48 * n5, 6 * nq * n5, "opt1 erb:347-465")
    out["operators"]["tensorprod_divlike_dirXYZ_var5"]["elements"] = ne5
    del vin, vout
    vm, vp = A(n=ntf * ne3, dtype=np.int32), A(n=ntf * ne3, dtype=np.int32)
    nf, fs = A(n=3 * ntf * ne3), A(n=ntf * ne3)
    es, hm = A(n=3 * n), A(n=nhn, dtype=np.int32)
    record("mesh_setup (device)",
           lambda: chk(lib.sdg_mesh_setup_dev(ne, ne, ne, p, 1.0, 1.0, 1.0, None, vm.ptr, vp.ptr,
                                              nf.ptr, es.ptr, fs.ptr, None, hm.ptr, None),
                       "mesh_setup"),
           # VMapM, VMapP (4 B), normal_fn (24 B), Fscale (8 B) a face node, Escale 24 B a
           # node, the halo map 4 B a halo node: written once
           40 * ntf * ne3 + 24 * n + 4 * nhn, 0, "mod_mesh.f90:74-193")
    f = A(n=np_ * (ne3 + nhalo))
    record("update_halo",
           lambda: chk(lib.sdg_update_halo_dev(f.ptr, hm.ptr, np_, ne3, nhn, None), "halo"),
           20 * nhn, 0, "mod_mesh.f90:209-221")
    out["operators"]["update_halo"]["halo_nodes"] = nhn
    return out


def bench_dropin(sdg, args, wl, fused_rate, opt=None):
    """The reference-shaped per-stage path on the bench workload, all on device
    arrays: mesh arrays built on the device (sdg_mesh_setup_dev), then per step
    q0 = q and three times update_halo(q), advect3d_eq_cal_tend(...) and the RK
    stage, as main.f90:51-80 calls them.  Timed on the host around K steps
    (queued asynchronously on one stream, launch cost included).  opt: the
    tendency's type (OPT1, the reference's order, by default; EVENODD the
    even-odd tendency kernel)."""
    opt = sdg.OPT_OPT1 if opt is None else opt
    import ctypes as C
    p, ne = args.p, args.ne
    nq, np_ = p + 1, (p + 1) ** 3
    ntf = 6 * nq * nq
    ne3 = ne ** 3
    nhalo = 6 * ne * ne
    nea = ne3 + nhalo
    nhn = nq * nq * nhalo
    lib = sdg.lib
    A = sdg.DeviceArray
    vm, vp = A(n=ntf * ne3, dtype=np.int32), A(n=ntf * ne3, dtype=np.int32)
    nf, fs = A(n=3 * ntf * ne3), A(n=ntf * ne3)
    es, hm = A(n=3 * np_ * ne3), A(n=nhn, dtype=np.int32)
    sdg._check(lib.sdg_mesh_setup_dev(ne, ne, ne, p, 1.0, 1.0, 1.0, None, vm.ptr, vp.ptr, nf.ptr,
                                      es.ptr, fs.ptr, None, hm.ptr, None), "sdg_mesh_setup_dev")
    fields = []
    for key in ("q", "u", "v", "w"):
        h = np.zeros(np_ * nea)
        h[: np_ * ne3] = wl[key]
        d = A(h)
        sdg._check(lib.sdg_update_halo_dev(d.ptr, hm.ptr, np_, ne3, nhn, None), "update_halo")
        fields.append(d)
    q, u, v, w = fields
    D, Dt, L = A(wl["D"]), A(wl["Dt"]), A(wl["L"])
    dqdt, q0 = A(n=np_ * nea), A(n=np_ * ne3)
    flux, err = A(n=ntf * ne3), A(np.zeros(1, dtype=np.int32))
    dt = wl["dt"]

    def step():
        sdg._check(lib.sdg_memcpy_d2d_async(q0.ptr, q.ptr, 8 * np_ * ne3, None), "q0 = q")
        for stage in range(3):
            lib.sdg_update_halo_dev(q.ptr, hm.ptr, np_, ne3, nhn, None)
            lib.sdg_advect3d_eq_cal_tend_dev(dqdt.ptr, q.ptr, u.ptr, v.ptr, w.ptr, D.ptr, Dt.ptr,
                                             L.ptr, vm.ptr, vp.ptr, nf.ptr, es.ptr, fs.ptr, nq,
                                             np_, ntf, ne3, nea, opt, flux.ptr, err.ptr,
                                             None)
            lib.sdg_rk_stage_dev(q.ptr, q0.ptr, dqdt.ptr, np_, ne3, stage, dt, None)

    for _ in range(args.warmup):
        step()
    sdg.synchronize()
    k = max(2, min(args.steps, 20))
    t0 = time.perf_counter()
    for _ in range(k):
        step()
    sdg.synchronize()
    t = time.perf_counter() - t0
    assert err.numpy()[0] == 0
    rate = np_ * ne3 * 3 * k / t / 1e9
    # the essential bytes plus the reference's geometry arrays, which this path
    # streams: Escale 24 B per DOF, VMapM/VMapP/normal_fn/Fscale 40 B per face
    # node (6/Nq face nodes per DOF)
    bpd = BYTES_PER_DOF_UPDATE["fp64"] + 24.0 + 40.0 * 6.0 / nq
    oname = {sdg.OPT_OPT1: "OPT1 order", sdg.OPT_GENERAL: "GENERAL order",
             sdg.OPT_EVENODD: "even-odd tendency kernel"}[opt]
    return {"workload": f"same {ne}^3 p={p} box through the per-stage device entry points "
                        "(update_halo, advect3d_eq_cal_tend_dev with VMapM/VMapP gathers, "
                        f"rk_stage_dev, {oname}) as the reference's loop calls them",
            "gdof_updates_per_s": rate, "ms_per_step": 1e3 * t / k, "steps": k,
            "launches_per_step": 13, "fused_over_dropin": fused_rate / rate,
            "bytes_per_dof_update_with_geometry": bpd,
            "achieved_gbs_with_geometry": bpd * rate}


def bench_dropin_step(sdg, args, wl, fused_rate, opt=None):
    """The time loop on the reference's arrays in one call
    (sdg_advect3d_eq_step_dev): mesh arrays built on the device, then K
    SSP-RK3 steps; EVENODD runs one fused launch a stage (face flux from
    VMapM/VMapP, normal_fn and Fscale, per-node Escale, lift, RK update),
    OPT1 the reference's per-stage sequence.  Timed on the host around the
    call with a synchronize on both sides."""
    opt = sdg.OPT_EVENODD if opt is None else opt
    p, ne = args.p, args.ne
    nq, np_ = p + 1, (p + 1) ** 3
    ntf = 6 * nq * nq
    ne3 = ne ** 3
    nhalo = 6 * ne * ne
    nea = ne3 + nhalo
    nhn = nq * nq * nhalo
    lib = sdg.lib
    A = sdg.DeviceArray
    vm, vp = A(n=ntf * ne3, dtype=np.int32), A(n=ntf * ne3, dtype=np.int32)
    nf, fs = A(n=3 * ntf * ne3), A(n=ntf * ne3)
    es, hm = A(n=3 * np_ * ne3), A(n=nhn, dtype=np.int32)
    sdg._check(lib.sdg_mesh_setup_dev(ne, ne, ne, p, 1.0, 1.0, 1.0, None, vm.ptr, vp.ptr, nf.ptr,
                                      es.ptr, fs.ptr, None, hm.ptr, None), "sdg_mesh_setup_dev")
    fields = []
    for key in ("q", "u", "v", "w"):
        h = np.zeros(np_ * nea)
        h[: np_ * ne3] = wl[key]
        d = A(h)
        sdg._check(lib.sdg_update_halo_dev(d.ptr, hm.ptr, np_, ne3, nhn, None), "update_halo")
        fields.append(d)
    q, u, v, w = fields
    D, Dt, L = A(wl["D"]), A(wl["Dt"]), A(wl["L"])
    nbytes = int(lib.sdg_advect3d_eq_step_scratch_bytes(nq, ne3))
    scratch = A(n=nbytes, dtype=np.uint8)
    err = A(np.zeros(1, dtype=np.int32))

    def run(k):
        sdg._check(lib.sdg_advect3d_eq_step_dev(
            q.ptr, u.ptr, v.ptr, w.ptr, D.ptr, Dt.ptr, L.ptr, vm.ptr, vp.ptr, nf.ptr, es.ptr,
            fs.ptr, hm.ptr, nq, np_, ntf, ne3, nea, nhn, wl["dt"], k, opt, scratch.ptr, nbytes,
            err.ptr, None), "sdg_advect3d_eq_step_dev")

    run(args.warmup)
    sdg.synchronize()
    k = max(2, min(args.steps, 20))
    t0 = time.perf_counter()
    run(k)
    sdg.synchronize()
    t = time.perf_counter() - t0
    assert err.numpy()[0] == 0
    rate = np_ * ne3 * 3 * k / t / 1e9
    oname = {sdg.OPT_OPT1: "OPT1 order, the reference's per-stage sequence",
             sdg.OPT_EVENODD: "one fused even-odd launch a stage"}[opt]
    return {"workload": f"same {ne}^3 p={p} box, sdg_advect3d_eq_step_dev on the reference's "
                        f"arrays (VMapM/VMapP, halo_src_map, normal_fn, Escale, Fscale), {oname}",
            "gdof_updates_per_s": rate, "ms_per_step": 1e3 * t / k, "steps": k,
            "launches_per_step": 3 if opt == sdg.OPT_EVENODD else 13,
            "ratio_to_fused_structured_stage": rate / fused_rate,
            "scratch_bytes": nbytes}


def bench_slabs(sdg, args, wl, fused_rate, nparts=4):
    """The bench box split into z-slab partitions that exchange their face
    planes before every stage (sdg_slabs_*): all partitions on this GPU, so
    the rate shows the exchange's cost on one device (pack, one copy per
    message, unpack), not multi-GPU scaling."""
    p, ne = args.p, args.ne
    s = sdg.Slabs(ne, ne, ne, p, wl["D"], wl["L"], nparts, opt=OPTS[args.opt],
                  precision=PRECISIONS[args.precision])
    s.upload(wl["q"], wl["u"], wl["v"], wl["w"])
    s.step(wl["dt"], args.warmup)
    sdg.synchronize()
    k = max(2, min(args.steps, 20))
    t0 = time.perf_counter()
    s.step(wl["dt"], k)
    sdg.synchronize()
    t = time.perf_counter() - t0
    rate = (p + 1) ** 3 * ne ** 3 * 3 * k / t / 1e9
    out = {"workload": f"same {ne}^3 p={p} box as {nparts} z-slab partitions on one GPU, "
                       "face planes exchanged before every stage",
           "nparts": nparts, "gdof_updates_per_s": rate, "ms_per_step": 1e3 * t / k,
           "steps": k, "exchange_bytes_per_stage": s.exchange_bytes(),
           "ratio_to_single_box": rate / fused_rate}
    s.close()
    return out


def bench_tensor_cores(sdg, args, reps=20):
    """The FP32 contraction of tensorprod_divlike_dirXYZ (three directions)
    at p = 15 on 16^3 elements (16.8M nodes, 201 MB of FP32 input and 201 MB
    of output): on the tensor cores (tcgen05 kind::tf32, 3xTF32 pairs) and on
    the CUDA cores, each queued `reps` times and timed on the host with a
    synchronize on both sides, beside one FP32 even-odd stage of the same box
    (the contractions are its dominant arithmetic)."""
    import workloads as W
    p, ne = 15, 16
    nq = p + 1
    ne3 = ne ** 3
    n = nq ** 3 * ne3
    x, D, Dt, L = W.reference_operators(p)
    lib, A = sdg.lib, sdg.DeviceArray
    rng = np.random.default_rng(args.seed + 9)
    ins = [A(rng.standard_normal(n).astype(np.float32)) for _ in range(3)]
    outs = [A(n=n, dtype=np.float32) for _ in range(3)]
    Dd = A(np.asarray(D, dtype=np.float32))
    err = A(np.zeros(1, dtype=np.int32))
    res = {"workload": f"{ne}^3 elements at p = {p}, FP32 arrays, three directions, "
                       f"{reps} queued calls each"}
    for name, tc in (("tensor_cores", 1), ("cuda_cores", 0)):
        def call():
            sdg._check(lib.sdg_tensorprod_divlike_dirXYZ_f32_dev(
                outs[0].ptr, outs[1].ptr, outs[2].ptr, Dd.ptr, ins[0].ptr, ins[1].ptr,
                ins[2].ptr, nq, ne3, tc, err.ptr, None), "divlike_f32")
        call()
        sdg.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            call()
        sdg.synchronize()
        t = (time.perf_counter() - t0) / reps
        res[name] = {"ms_per_call": 1e3 * t, "gbs": 24.0 * n / t / 1e9,
                     "tflops": 2.0 * 3 * nq * n / t / 1e12}
    assert int(err.numpy()[0]) == 0
    q, u, v, w = W.blob(ne, ne, ne, x, args.seed + 15)
    s = sdg.Solver(ne, ne, ne, p, D, L, opt=sdg.OPT_EVENODD, precision=sdg.PREC_FP32)
    s.upload(q, u, v, w)
    dt = W.cfl_dt(ne, ne, ne, p, u, v, w)
    s.step(dt, 2)
    ms = s.step_timed(dt, 10)
    s.close()
    res["fp32_evenodd_stage_ms"] = ms / 30.0
    res["tensor_over_cuda_cores"] = (res["cuda_cores"]["ms_per_call"] /
                                     res["tensor_cores"]["ms_per_call"])
    return res


def bench_serving(sdg, args, rate=None, plain_cache=None):
    """Poisson arrivals of solves (Ne per axis U{4..32}, p U{2..11}, nstep
    U{10..500}, Gaussian tracer in a constant velocity, FP32 compute / FP64
    state) into the continuous-batching server.  The request stream is the
    same at every rate (only the arrival times scale), so plain_cache keeps
    the plain-path time of its sample across calls."""
    import math
    import workloads as W
    ops = {p: W.reference_operators(p) for p in range(2, 12)}
    rng = W.SplitMix64(args.seed + 5000)
    reqs, arrivals, t = [], [], 0.0
    for i in range(args.serve_n):
        dims = tuple(rng.randint(4, args.serve_max_ne) for _ in range(3))
        p = rng.randint(2, 11)
        nstep = rng.randint(10, 500)
        vel = (2 * rng.uniform() - 1, 2 * rng.uniform() - 1, 2 * rng.uniform() - 1)
        dt = 0.1 * min(1.0 / d for d in dims) / ((2 * p + 1) * max(sum(abs(v) for v in vel), 1e-3))
        reqs.append(dict(NeX=dims[0], NeY=dims[1], NeZ=dims[2], p=p, nstep=nstep, dt=dt,
                         centre=[rng.uniform() for _ in range(3)],
                         sigma=0.05 + 0.15 * rng.uniform(), velocity=vel))
        t += -math.log(1.0 - rng.uniform()) / (rate or args.serve_rate)
        arrivals.append(t)
    srv = sdg.Server(ops, hbm_budget_bytes=int(args.serve_budget_gb * (1 << 30)),
                     opt=0 if args.batch_opt == "auto" else OPTS[args.batch_opt],
                     parallel_groups=args.parallel_groups)
    # warm the batched kernel and the pool
    srv.wait(srv.submit(**reqs[0]))
    srv.reset_stats()
    tickets = []
    t0 = time.perf_counter()
    for r, ta in zip(reqs, arrivals):
        now = time.perf_counter() - t0
        if ta > now:
            time.sleep(ta - now)
        tickets.append(srv.submit(**r))
    lat = [srv.wait(tk)[0]["latency_s"] for tk in tickets]
    span = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    dofs = sum((r["p"] + 1) ** 3 * r["NeX"] * r["NeY"] * r["NeZ"] * 3 * r["nstep"] for r in reqs)
    # the plain FP64 path on the first requests, one after the other
    k = min(args.serve_plain_sample, len(reqs))
    pt = 0.0
    cached = plain_cache.get("t") if plain_cache is not None else None
    for r in (reqs[:k] if cached is None else []):
        x, D, Dt, L = ops[r["p"]]
        s = sdg.Solver(r["NeX"], r["NeY"], r["NeZ"], r["p"], D, L, opt=OPTS[args.opt],
                       precision=sdg.PREC_FP64)
        n = (r["p"] + 1) ** 3 * r["NeX"] * r["NeY"] * r["NeZ"]
        # the work per step does not depend on the values: a zero tracer
        s.upload(np.zeros(n), np.full(n, r["velocity"][0]), np.full(n, r["velocity"][1]),
                 np.full(n, r["velocity"][2]))
        sdg.synchronize()
        tt = time.perf_counter()
        s.step(r["dt"], r["nstep"])
        sdg.synchronize()
        pt += time.perf_counter() - tt
        s.close()
    if cached is not None:
        pt = cached
    elif plain_cache is not None:
        plain_cache["t"] = pt
    sample_dofs = sum((r["p"] + 1) ** 3 * r["NeX"] * r["NeY"] * r["NeZ"] * 3 * r["nstep"]
                      for r in reqs[:k])
    plain_solves = len(reqs) / (pt * dofs / sample_dofs)
    return {
        "workload": f"{args.serve_n} requests, Poisson arrivals at {rate or args.serve_rate} req/s, "
                    f"Ne per axis U{{4..{args.serve_max_ne}}}, p U{{2..11}}, nstep U{{10..500}}, "
                    "FP32 compute / FP64 state, admission by HBM budget",
        "offered_rate_req_s": rate or args.serve_rate,
        "solves_per_s": len(reqs) / span,
        "p50_latency_s": float(np.percentile(lat, 50)),
        "p99_latency_s": float(np.percentile(lat, 99)),
        "gdof_updates_per_s": dofs / span / 1e9,
        "plain_fp64_solves_per_s_same_requests": plain_solves,
        "ratio_vs_plain": (len(reqs) / span) / plain_solves,
        "server": {k2: st[k2] for k2 in ("completed", "steps_run", "launches", "fatal_status")},
    }


class Replicas:
    """Replica plumbing under torchrun: a gloo process group used only for the
    barrier around the timed region and the max of the per-rank times.  The
    path exchanges no data between GPUs: each rank advances its own box."""

    def __init__(self, ws: int):
        self.ws = ws
        self.dist = None
        if ws > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self) -> None:
        if self.dist is not None:
            self.dist.barrier()

    def tmax(self, t: float) -> float:
        if self.dist is None:
            return t
        import torch
        tt = torch.tensor([t], dtype=torch.float64)
        self.dist.all_reduce(tt, op=self.dist.ReduceOp.MAX)
        return float(tt.item())

    def close(self) -> None:
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


def whole_job_rate(ws: int, ndof: int, steps: int, t_max: float) -> float:
    """GDOF-updates/s of all replicas: every rank advanced ndof DOFs through
    3*steps stages, and the job took the slowest rank's time."""
    return ws * ndof * 3 * steps / t_max / 1e9


def _round(x, sig=4):
    """Rounds every float of a JSON-able structure to `sig` significant digits."""
    if isinstance(x, float):
        return float(f"{x:.{sig}g}")
    if isinstance(x, dict):
        return {k: _round(v, sig) for k, v in x.items()}
    if isinstance(x, list):
        return [_round(v, sig) for v in x]
    return x


def headline_line(args, ws, value, t, roof, cpu, e2e, clk, parity, sections) -> dict:
    """The compact last line (kept well under 2 KB): the contract's keys, the
    roofline, the CPU baseline, e2e, clocks and parity, plus one-line
    summaries of serving (solves/s and p99 against the plain GPU path) and of
    the batched ensemble.  Everything else is in the earlier section lines."""
    line = {
        "metric": metric_name(args), "value": value, "unit": "GDOF-updates/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp64": "f64", "fp64emu": "f64-state/double-float",
                  "fp32": "f32-compute/f64-state"}[args.precision],
        "data": "synthetic (seeded Gaussian tracer, seeded smooth velocity)",
        "config": config(args),
        "roofline": {k: roof[k] for k in ("bound", "achieved", "peak", "unit", "frac", "traffic",
                                          "algorithmic_bytes_per_dof_update",
                                          "implementation_bytes_per_dof_update", "kernel",
                                          "binding_roof") if k in roof},
        "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": 3 * args.steps, "clocks": clk,
        "parity": parity,
    }
    if "compute" in roof:
        c = roof["compute"]
        line["roofline"]["compute"] = {k: c[k] for k in ("pipe", "frac", "frac_source",
                                                         "achieved_tflops",
                                                         "peak_tflops_measured_live")}
    if e2e is not None:
        line["e2e"] = {k: e2e[k] for k in ("value", "unit", "h2d_bytes_per_step",
                                           "d2h_bytes_per_step", "steps")}
    srv = sections.get("serving_saturated") or sections.get("serving")
    if srv:
        line["serving"] = {k: srv[k] for k in ("offered_rate_req_s", "solves_per_s",
                                               "p50_latency_s", "p99_latency_s",
                                               "ratio_vs_plain")}
    ens = sections.get("ensemble")
    if ens:
        line["ensemble"] = {k: ens[k] for k in ("solves_per_s", "ratio_vs_plain",
                                                "rel_l2_vs_fp64_max", "hbm_frac")}
    return _round(line)


def emit_section(name: str, body, out: dict) -> None:
    """Prints one secondary measurement as its own JSON line and keeps it."""
    out[name] = body
    print(json.dumps({"section": name, "result": body}), flush=True)


def run_ours(args, ws, rank, local):
    import sdg
    if sdg.device_count() < 1:
        raise SystemExit("bench.py: no CUDA device")
    sdg.set_device(local)
    rep = Replicas(ws)
    barrier, tmax = rep.barrier, rep.tmax

    p, ne = args.p, args.ne
    wl = make_workload(p, ne, args.seed + rank)
    ndof = (p + 1) ** 3 * ne ** 3

    # ---- headline: the requested precision, device-resident ----
    s, t, clk = time_solver(sdg, wl, p, ne, PRECISIONS[args.precision], args.steps,
                            args.warmup, local, barrier, True, OPTS[args.opt])
    t = tmax(t)
    value = whole_job_rate(ws, ndof, args.steps, t)
    peaks = None if args.no_microbench else sdg.microbench_peaks()
    roof = roofline(args.precision, p, ne, ndof, t, args.steps, peaks, args.opt)

    # ---- end to end through the C ABI with pinned host buffers ----
    # every step uploads q, u, v, w from page-locked host memory and downloads
    # q; the pipelined entry point overlaps step r+1's upload and step r-1's
    # download with step r's kernels
    e2e = None
    if not args.no_e2e:
        pins = [sdg.PinnedArray(ndof) for _ in range(5)]
        for pa, src in zip(pins, (wl["q"], wl["u"], wl["v"], wl["w"])):
            pa.array[:] = src
        k = max(2, min(args.steps, args.e2e_steps))
        ins = [[pins[c].ptr] * k for c in range(4)]
        outs = [pins[4].ptr] * k
        s.solve_host_pipelined(*[x[:2] for x in ins], outs[:2], wl["dt"], 1)  # warm-up
        barrier()
        t0 = time.perf_counter()
        s.solve_host_pipelined(*ins, outs, wl["dt"], 1)
        te = tmax(time.perf_counter() - t0)
        e2e = {"value": ws * ndof * 3 * k / te / 1e9, "unit": "GDOF-updates/s",
               "h2d_bytes_per_step": 4 * 8 * ndof, "d2h_bytes_per_step": 8 * ndof,
               "steps": k, "path": "sdg_solver_solve_host_pipelined: per step, upload "
                                   "q,u,v,w + one SSP-RK3 step + download q, overlapped "
                                   "across steps on two buffer sets"}
        for pa in pins:
            pa.free()
    tend_main = None
    if rank == 0 and not args.no_cpu_baseline:
        s.upload(wl["q"], wl["u"], wl["v"], wl["w"])  # the initial state again
        tend_main = s.tendency()
    s.close()

    # ---- the other FP64-state path on the same workload ----
    other = None
    tend_emu = None
    if args.precision == "fp64" and not args.no_emu:
        se, te_, _ = time_solver(sdg, wl, p, ne, PRECISIONS["fp64emu"], args.steps,
                                 args.warmup, local, barrier, False, OPTS[args.opt])
        te_ = tmax(te_)
        other = {"precision": "fp64emu",
                 "description": "FP64 state and RK combine; flux, divergence and lift in "
                                "double-float (two FP32 numbers) on the FP32 pipes",
                 "value": ws * ndof * 3 * args.steps / te_ / 1e9, "unit": "GDOF-updates/s",
                 "ms_per_step": 1e3 * te_ / args.steps,
                 "roofline": roofline("fp64emu", p, ne, ndof, te_, args.steps, peaks, args.opt)}
        if rank == 0 and not args.no_cpu_baseline:
            se.upload(wl["q"], wl["u"], wl["v"], wl["w"])
            tend_emu = se.tendency()
        se.close()

    if rank != 0:
        rep.close()
        return 0

    sections: dict = {}
    if e2e is not None:
        emit_section("e2e_detail", e2e, sections)
    emit_section("roofline_detail", roof, sections)
    cpu = None
    parity = None
    if not args.no_cpu_baseline:
        ob = OracleBox(wl, p, ne)
        ref = ob.tendency()

        def rl2(x):
            return float(np.linalg.norm(x - ref) / np.linalg.norm(ref))

        parity = {"tendency_rel_l2_vs_oracle": rl2(tend_main),
                  "tolerance": 1e-12 if args.precision != "fp32" else 1e-5,
                  "state": "initial state, reference operators p%d.dat" % p}
        if other is not None:
            other["tendency_rel_l2_vs_fp64_oracle"] = rl2(tend_emu)
        if ws == 1:
            steps, secs = ob.time_steps(args.cpu_seconds, 10 ** 6)
            cpu = {"value": ndof * 3 * steps / secs / 1e9, "unit": "GDOF-updates/s",
                   "cores": ob.threads, "kind": "port",
                   "sample": f"{steps} SSP-RK3 steps of the same box, OPT1 order, "
                             f"{secs:.1f} s (C+OpenMP restatement of the reference)"}
    if other is not None:
        emit_section("fp64_emulated", other, sections)
    if ws == 1 and not args.no_dropin:
        emit_section("dropin", bench_dropin(sdg, args, wl, value), sections)
        emit_section("dropin_evenodd", bench_dropin(sdg, args, wl, value, sdg.OPT_EVENODD),
                     sections)
        emit_section("dropin_step", bench_dropin_step(sdg, args, wl, value), sections)
        emit_section("dropin_step_opt1", bench_dropin_step(sdg, args, wl, value, sdg.OPT_OPT1),
                     sections)
    if ws == 1 and not args.no_slabs:
        emit_section("slabs", bench_slabs(sdg, args, wl, value), sections)
    if ws == 1 and not args.no_operators:
        emit_section("operators", bench_operators(sdg, args, peaks), sections)
        emit_section("tensor_core_contraction", bench_tensor_cores(sdg, args), sections)
    if ws == 1 and not args.no_ensemble:
        emit_section("ensemble", bench_ensemble(sdg, args), sections)
    if ws == 1 and not args.no_serving:
        plain_cache = {}
        emit_section("serving", bench_serving(sdg, args, plain_cache=plain_cache), sections)
        # the same request stream offered faster than the GPU can serve it:
        # throughput and tail latency of the saturated server
        emit_section("serving_saturated",
                     bench_serving(sdg, args, args.serve_rate_saturated, plain_cache), sections)
        # the offered rate swept across the 10-2000 req/s range
        sweep = []
        for r in (float(x) for x in args.serve_sweep.split(",") if x):
            res = bench_serving(sdg, args, r, plain_cache)
            sweep.append({k: res[k] for k in ("offered_rate_req_s", "solves_per_s",
                                              "p50_latency_s", "p99_latency_s",
                                              "gdof_updates_per_s", "ratio_vs_plain")})
        emit_section("serving_rate_sweep", sweep, sections)
    if ws == 1 and not args.no_sweep:
        emit_section("order_sweep", bench_order_sweep(sdg, args), sections)
    line = headline_line(args, ws, value, t, roof, cpu, e2e, clk, parity, sections)
    if args.results:
        with open(args.results, "w") as f:
            json.dump({"headline": line, "sections": sections}, f, indent=1)
    print(json.dumps(line), flush=True)
    rep.close()
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--p", type=int, default=7)
    ap.add_argument("--ne", type=int, default=32)
    ap.add_argument("--precision", choices=["fp64", "fp64emu", "fp32"], default="fp64")
    ap.add_argument("--opt", choices=["general", "opt1", "evenodd"], default="evenodd",
                    help="summation order of the FP64 stage: the reference's GENERAL or "
                         "OPT1 order, or the even-odd factorised body")
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-emu", action="store_true",
                    help="skip the emulated-FP64 measurement beside the FP64 headline")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-dropin", action="store_true",
                    help="skip the per-stage drop-in path measurement")
    ap.add_argument("--no-slabs", action="store_true",
                    help="skip the z-slab partition measurement")
    ap.add_argument("--no-operators", action="store_true",
                    help="skip the standalone operator entry points (divlike, gradlike, "
                         "var5, matvec, Lift, update_halo, mesh build)")
    ap.add_argument("--batch-opt", choices=["auto", "general", "evenodd"], default="auto",
                    help="stage body of the batched kernels (ensemble and serving): auto = "
                         "chosen per order (the ensemble's tuner, the server's measured "
                         "defaults), else fixed for every order")
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--sweep-steps", type=int, default=100)
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--ens-n", type=int, default=256)
    ap.add_argument("--ens-steps", type=int, default=100)
    ap.add_argument("--serve-n", type=int, default=60)
    ap.add_argument("--serve-rate", type=float, default=20.0)
    ap.add_argument("--serve-rate-saturated", type=float, default=200.0)
    ap.add_argument("--parallel-groups", action="store_true",
                    help="run the batched forms' order groups on parallel streams instead of "
                         "one after the other")
    ap.add_argument("--serve-sweep", default="10,50,100,500,2000",
                    help="offered rates (req/s) of the serving sweep, comma separated")
    ap.add_argument("--serve-max-ne", type=int, default=32)
    ap.add_argument("--serve-budget-gb", type=float, default=64.0)
    ap.add_argument("--serve-plain-sample", type=int, default=8)
    ap.add_argument("--no-microbench", action="store_true",
                    help="skip the live DFMA/FFMA peak measurement")
    ap.add_argument("--results", default=None,
                    help="also write the headline and every section to this JSON file")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    return run_ours(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
