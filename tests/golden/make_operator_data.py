"""Captures the reference's operator files as a binary fixture.

The reference reads its element operators from operator_data/p{p}.dat
(element_init, mod_mesh.f90:253-263: three list-directed reads of x1D,
D1D(Nq,Nq) and Lift_mat(Nq,Nq,Nq,6), then D1D_tr = transpose(D1D)).  The GPU
parity tests, the golden fixtures, smoke() and both bench arms run on exactly
those numbers.  The reference tree is not present where the GPU tests run, so
this script reads every file p1..p15 once, through the oracle's reader (the
same list-directed parsing), and stores the parsed doubles bit for bit in
tests/golden/operator_data.npz:

    x1D_p{p} (Nq), D1D_p{p} (Nq*Nq), D1D_tr_p{p} (Nq*Nq), Lift_p{p} (6*Nq^3),
    sha256_p{p} (hex digest of the source file, to tie the arrays to it)

Run from the repository root where the reference is mounted:

    python tests/golden/make_operator_data.py
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# where the reference tree is mounted when the fixture is made
REFERENCE_OPERATOR_DIR = os.environ.get("SDG_REFERENCE_OPERATOR_DIR",
                                        "/root/reference/operator_data")
OUT = os.path.join(HERE, "operator_data.npz")
ORDERS = range(1, 16)


def source_path(p: int) -> str:
    return os.path.join(REFERENCE_OPERATOR_DIR, f"p{p}.dat")


def main() -> int:
    import oracle as O
    arrays = {}
    for p in ORDERS:
        path = source_path(p)
        x, D, Dt, L = O.read_operator_file(path, p)
        with open(path, "rb") as f:
            digest = hashlib.sha256(f.read()).hexdigest()
        arrays[f"x1D_p{p}"] = x
        arrays[f"D1D_p{p}"] = D
        arrays[f"D1D_tr_p{p}"] = Dt
        arrays[f"Lift_p{p}"] = L
        arrays[f"sha256_p{p}"] = np.array(digest)
    np.savez_compressed(OUT, **arrays)
    print("wrote", OUT)
    return 0


if __name__ == "__main__":
    sys.exit(main())
