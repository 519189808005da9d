"""Shared helpers for the tests: building cases and comparing results."""
from __future__ import annotations

import glob
import os

import numpy as np

import oracle as O
import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
# the golden cases (inputs and oracle outputs); operator_data.npz holds operators only
GOLDEN_CASES = sorted(f for f in glob.glob(os.path.join(GOLDEN, "*.npz"))
                      if os.path.basename(f) != "operator_data.npz")

# tolerances stated by the parity contract
TOL_TEND = 1e-12     # relative L2 per tendency (plain FP64 form)
TOL_RUN = 1e-10      # relative L2 of q after nstep (plain FP64 form)
TOL_FP32 = 1e-5      # relative L2 of the FP32-compute form against FP64


def rel_l2(x, ref) -> float:
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    den = np.linalg.norm(ref)
    return float(np.linalg.norm(x - ref) / (den if den > 0 else 1.0))


def operators(p: int, source: str = "file"):
    """(x1D, D1D, D1D_tr, Lift) of order p.

    source "file": the reference's own operator_data/p{p}.dat, bit for bit
    (the committed fixture tests/golden/operator_data.npz); "generated": the
    product's GLL generator (sdg_operator_generate), which agrees with the
    files to <= 5e-14."""
    if source == "file":
        return W.reference_operators(p)
    if source == "generated":
        import sdg
        return sdg.operator_generate(p)
    raise ValueError(source)


class Case:
    """A periodic box with fields, built by the oracle like main.f90's init."""

    def __init__(self, NeX, NeY, NeZ, p, ic="blob", seed=W.BASE_SEED, vel=(1.0, 0.5, 0.25),
                 ops=None):
        self.NeX, self.NeY, self.NeZ, self.p = NeX, NeY, NeZ, p
        self.x1D, self.D, self.Dt, self.Lift = ops if ops is not None else operators(p)
        self.mesh = O.Mesh(NeX, NeY, NeZ, p, self.x1D)
        m = self.mesh
        if ic == "sine":
            q, u, v, w = W.sine(NeX, NeY, NeZ, self.x1D, vel)
        else:
            q, u, v, w = W.blob(NeX, NeY, NeZ, self.x1D, seed)
        self.q, self.u, self.v, self.w = (W.with_halo(a, m.NeA, m.Np) for a in (q, u, v, w))
        for f in (self.q, self.u, self.v, self.w):
            m.update_halo(f)
        self.dt = W.cfl_dt(NeX, NeY, NeZ, p, u, v, w)

    def term_scale(self) -> float:
        """Size of the terms the tendency sums (Escale |D| |q| |u| over the
        owned nodes): the floor of a relative error whose exact result
        vanishes, as at p = 1 on a one-element periodic box, where all eight
        nodes are the same point and the tendency is rounding noise."""
        n = self.nown
        vmax = max(np.abs(a[:n]).max() for a in (self.u, self.v, self.w))
        es = max(self.NeX, self.NeY, self.NeZ) * 2.0
        return float(es * np.abs(self.D).max() * vmax * np.linalg.norm(self.q[:n]))

    @property
    def nown(self) -> int:
        return self.mesh.Np * self.mesh.Ne

    def oracle_tend(self, opt=O.OPT1):
        return O.cal_tend(self.mesh, self.q, self.u, self.v, self.w, self.D, self.Dt, self.Lift,
                          opt)[: self.nown]

    def oracle_run(self, nstep, opt=O.OPT1):
        q = self.q.copy()
        O.run(self.mesh, q, self.u, self.v, self.w, self.D, self.Dt, self.Lift, self.dt, nstep,
              opt)
        return q[: self.nown]
