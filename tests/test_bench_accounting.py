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
