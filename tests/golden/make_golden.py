"""Generates the golden fixtures tests/golden/p*_*.npz with the CPU oracle.

Each fixture is self-contained: it stores the operators (the reference's own
operator_data/p{p}.dat, from tests/golden/operator_data.npz), the owned
initial fields and the oracle's outputs (tendency in OPT1 and GENERAL order,
and q after nstep SSP-RK3 steps), so that the GPU path and the oracle can be
checked against it on any machine.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "scale-dg-kernel-extraction_gb300"))

import oracle as O  # noqa: E402
import workloads as W  # noqa: E402

CASES = [
    # name, (NeX, NeY, NeZ), p, ic, nstep
    ("p1_sine_4x4x4", (4, 4, 4), 1, "sine", 20),
    ("p3_sine_3x2x4", (3, 2, 4), 3, "sine", 10),
    ("p7_blob_2x2x2", (2, 2, 2), 7, "blob", 5),
    ("p8_blob_2x1x2", (2, 1, 2), 8, "blob", 4),
]


def make(name, dims, p, ic, nstep):
    NeX, NeY, NeZ = dims
    x, D, Dt, L = W.reference_operators(p)
    m = O.Mesh(NeX, NeY, NeZ, p, x)
    if ic == "sine":
        q, u, v, w = W.sine(NeX, NeY, NeZ, x, (1.0, 0.5, 0.25))
    else:
        q, u, v, w = W.blob(NeX, NeY, NeZ, x, W.BASE_SEED + 7)
    dt = W.cfl_dt(NeX, NeY, NeZ, p, u, v, w)
    qa, ua, va, wa = (W.with_halo(a, m.NeA, m.Np) for a in (q, u, v, w))
    for f in (qa, ua, va, wa):
        m.update_halo(f)
    n = m.Np * m.Ne
    d1 = O.cal_tend(m, qa, ua, va, wa, D, Dt, L, O.OPT1)[:n]
    d2 = O.cal_tend(m, qa, ua, va, wa, D, Dt, L, O.GENERAL)[:n]
    qq = qa.copy()
    O.run(m, qq, ua, va, wa, D, Dt, L, dt, nstep, O.OPT1)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), dims=np.array([NeX, NeY, NeZ, p, nstep]),
                        x1D=x, D=D, Lift=L, q=q, u=u, v=v, w=w, dt=np.array(dt),
                        dqdt_opt1=d1, dqdt_general=d2, q_final=qq[:n])


if __name__ == "__main__":
    for c in CASES:
        make(*c)
        print("wrote", c[0])
