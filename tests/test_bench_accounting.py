"""bench.py's byte and flop accounting on CPU: the roofline's algorithmic bytes
per DOF-update and the standalone-operator section, driven through a stand-in
library that records the calls instead of launching anything."""
import sys
import types

import numpy as np
import pytest

from helpers import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_bytes_per_dof_update():
    # stage 1: q, u, v, w in, q out (40 B); stages 2-3 also q0 (48 B)
    assert bench.BYTES_PER_DOF_UPDATE["fp64"] == pytest.approx((40 + 48 + 48) / 3)
    assert bench.BYTES_PER_DOF_UPDATE["fp32"] == pytest.approx((28 + 36 + 36) / 3)
    # the even-odd FP64 and emulated stages move (tP, tM) of 6 Nq^2 face nodes
    # per element: 16 * 6 Nq^2 / Nq^3 = 96 / Nq bytes a DOF in every launch
    for p in range(1, 16):
        for prec in ("fp64", "fp64emu"):
            assert bench.face_factor_bytes(prec, "evenodd", p) == pytest.approx(96 / (p + 1))
            assert bench.face_factor_bytes(prec, "opt1", p) == 0
        assert bench.face_factor_bytes("fp32", "evenodd", p) == 0
    assert bench.BYTES_PER_DOF_UPDATE["fp64"] + bench.face_factor_bytes(
        "fp64", "evenodd", 7) == pytest.approx(57 + 1 / 3)


class _Lib:
    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        def call(*args):
            self.calls.append((name, args))
            return 0
        return call


class _Dev:
    def __init__(self, src=None, n=0, dtype=np.float64):
        self.n = np.asarray(src).size if src is not None else n
        self.ptr = 1


def test_operator_section_counts_each_array_once(monkeypatch):
    lib = _Lib()
    fake = types.SimpleNamespace(
        lib=lib, DeviceArray=_Dev, synchronize=lambda: None, _check=lambda r, w: None,
        operator_generate=lambda p: (np.zeros(p + 1), np.zeros((p + 1) ** 2),
                                     np.zeros((p + 1) ** 2), np.zeros(6 * (p + 1) ** 3)),
        OPT_OPT1=2, OPT_GENERAL=1)
    monkeypatch.setattr(bench, "measured_peaks", lambda: (1000.0, "measured"))
    p, ne = 3, 5
    out = bench.bench_operators(fake, types.SimpleNamespace(p=p, ne=ne, seed=1),
                                {"dfma_tflops": 1.0}, reps=2)
    ops = out["operators"]
    nq, n = p + 1, (p + 1) ** 3 * ne ** 3
    ntf = 6 * nq * nq
    assert ops["tensorprod_divlike_dirXYZ (OPT1)"]["bytes_per_call"] == 48 * n
    assert ops["tensorprod_divlike_dirXYZ (GENERAL)"]["bytes_per_call"] == 48 * n
    assert ops["tensorprod_gradlike_dirXYZ"]["bytes_per_call"] == 32 * n
    assert ops["element_matvec_dir (z)"]["bytes_per_call"] == 16 * n
    assert ops["tensorprod_Lift_hexahedral"]["bytes_per_call"] == 8 * (n + ntf * ne ** 3)
    ne5 = ne ** 3 // 5
    assert ops["tensorprod_divlike_dirXYZ_var5"]["bytes_per_call"] == 48 * 5 * nq ** 3 * ne5
    nhn = nq * nq * 6 * ne * ne
    assert ops["update_halo"]["bytes_per_call"] == 20 * nhn
    for row in ops.values():
        assert row["hbm_frac"] == pytest.approx(row["gbs"] / 1000.0)
    # each operator: one untimed call and `reps` timed ones, OPT1 and GENERAL both
    names = [c[0] for c in lib.calls]
    assert names.count("sdg_tensorprod_divlike_dirXYZ_dev") == 6
    assert {c[1][10] for c in lib.calls if c[0] == "sdg_tensorprod_divlike_dirXYZ_dev"} == {1, 2}
    assert names.count("sdg_tensorprod_divlike_dirXYZ_var5_dev") == 3
    assert names.count("sdg_mesh_setup_dev") == 3


def test_roofline_counts_algorithmic_bytes_only(monkeypatch):
    """roofline.frac uses the algorithmic bytes (45.33 B a DOF-update for
    FP64); the even-odd stage's shared face factors are reported apart."""
    monkeypatch.setattr(bench, "measured_peaks", lambda: (6000.0, "measured"))
    p, ne, steps = 7, 32, 10
    ndof = (p + 1) ** 3 * ne ** 3
    t = 0.026  # seconds for 10 steps = 30 launches
    peaks = {"dfma_tflops": 1.25, "ffma_tflops": 75.0}
    r = bench.roofline("fp64", p, ne, ndof, t, steps, peaks, "evenodd")
    assert r["algorithmic_bytes_per_dof_update"] == pytest.approx(136 / 3)
    assert r["implementation_bytes_per_dof_update"] == pytest.approx(12.0)
    achieved = 136 / 3 * ndof / (t / 30) / 1e9
    assert r["achieved"] == pytest.approx(achieved)
    assert r["frac"] == pytest.approx(achieved / 6000.0)
    assert r["binding_roof"] == "fp64_pipe"
    assert 0 < r["compute"]["frac"] <= 1.0
    r32 = bench.roofline("fp32", p, ne, ndof, t, steps, peaks, "evenodd")
    assert r32["algorithmic_bytes_per_dof_update"] == pytest.approx(100 / 3)
    assert r32["implementation_bytes_per_dof_update"] == 0


def test_headline_line_is_compact(monkeypatch):
    """The last line the benchmark prints stays under 2 KB with every
    section present, and carries the contract's keys."""
    import json
    monkeypatch.setattr(bench, "measured_peaks", lambda: (6775.3, "measured"))
    args = types.SimpleNamespace(p=7, ne=32, steps=50, warmup=3, precision="fp64",
                                 opt="evenodd")
    ndof = 8 ** 3 * 32 ** 3
    peaks = {"dfma_tflops": 1.2612345, "ffma_tflops": 75.123456}
    roof = bench.roofline("fp64", 7, 32, ndof, 0.1303, 50, peaks, "evenodd")
    cpu = {"value": 0.4234567, "unit": "GDOF-updates/s", "cores": 16, "kind": "port",
           "sample": "40 SSP-RK3 steps of the same 32^3 p=7 box, OPT1 order (10.1 s; C + "
                     "OpenMP restatement of the Fortran reference, timing build)"}
    e2e = {"value": 18.123456, "unit": "GDOF-updates/s", "h2d_bytes_per_step": 536870912,
           "d2h_bytes_per_step": 134217728, "steps": 50, "path": "x" * 200}
    clk = {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "samples": 37, "reasons": []}
    parity = {"tendency_rel_l2_vs_oracle": 1.123456e-14, "tolerance": 1e-12,
              "state": "initial state, reference operators p7.dat"}
    srv = {"offered_rate_req_s": 200.0, "solves_per_s": 33.2123, "p50_latency_s": 1.3123,
           "p99_latency_s": 1.73123, "ratio_vs_plain": 5.2123, "workload": "y" * 300}
    ens = {"solves_per_s": 443.123, "ratio_vs_plain": 6.7123, "rel_l2_vs_fp64_max": 8.1e-8,
           "hbm_frac": 0.51234, "autotuned": {"z": "z" * 500}}
    line = bench.headline_line(args, 1, 19.31234, 0.1303, roof, cpu, e2e, clk, parity,
                               {"serving_saturated": srv, "ensemble": ens})
    text = json.dumps(line)
    assert len(text) <= 2048, len(text)
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "dtype", "config", "roofline", "cpu_baseline", "e2e",
                "clocks", "parity", "gpu_launches"):
        assert key in line
    assert line["gpu_launches"] == 150
    assert line["config"]["opt"] == "EVENODD"
    assert bench.config(args, reference=True)["opt"] == "OPT1"


def test_emulated_roofline_reports_its_fp64_pipe_apart(monkeypatch):
    """The emulated form's compute fraction is its FP32 flops against the
    FFMA peak; the FP64 pipe's busy share from the capture sits beside it."""
    monkeypatch.setattr(bench, "measured_peaks", lambda: (6000.0, "measured"))
    p, ne, steps = 7, 32, 10
    ndof = (p + 1) ** 3 * ne ** 3
    t = 0.01
    peaks = {"dfma_tflops": 1.25, "ffma_tflops": 75.0}
    r = bench.roofline("fp64emu", p, ne, ndof, t, steps, peaks, "evenodd")
    c = r["compute"]
    assert c["pipe"] == "FP32 (FFMA)"
    assert c["frac"] == pytest.approx(c["achieved_tflops"] / 75.0)
    assert c["fp64_pipe_busy"] == pytest.approx(0.597)
    assert "binding_roof" not in r
