"""Seeded synthetic inputs for the advection workloads.

There is no dataset: each workload is generated from a seed.  The recipe:

* node coordinates as mesh_setup places them (mod_mesh.f90:141-145, :332-353):
  x = (i_e - 0.5) dx + 0.5 dx x1D(i) on the periodic unit box;
* "sine": q = sin(2 pi x) sin(2 pi y) sin(2 pi z) with a constant velocity, the
  reference's own initial condition (main.f90:144-157);
* "blob": velocity U0 + 0.2 sum_{m=1..4} a_m sin(2 pi k_m.x + phi_m) with
  U0 = (1, 0.5, 0.25), integer k_m with 1 <= |k_m| <= 3, a_m a random unit
  vector and phi_m uniform in [0, 2 pi); tracer exp(-d^2 / (2 sigma^2)) with d
  the periodic minimum-image distance to a centre uniform in [0,1)^3;
* time step dt = CFL min(dx,dy,dz) / ((2p+1) max_nodes(|u|+|v|+|w|)), CFL 0.1
  (the reference takes dt from its namelist and has no CFL rule).

Random numbers come from splitmix64 (uniform double = top 53 bits / 2^53),
seeded with base seed + instance index.  Arrays are flat, column-major
(Np, Ne): node index fastest, element index e = ex + ey NeX + ez NeX NeY.
"""
from __future__ import annotations

import math
import os

import numpy as np

BASE_SEED = 20261203
U0 = (1.0, 0.5, 0.25)
_M64 = (1 << 64) - 1

# The reference's operator files operator_data/p1..p15.dat, parsed as
# element_init reads them (mod_mesh.f90:253-263) and stored bit for bit
# (made by tests/golden/make_operator_data.py).
OPERATOR_FIXTURE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "tests", "golden", "operator_data.npz")
_opcache: dict = {}


def reference_operators(p: int):
    """(x1D, D1D, D1D_tr, Lift_mat) of the reference's operator_data/p{p}.dat,
    flat column-major float64 arrays, exactly the doubles the reference's
    list-directed reads produce."""
    if not 1 <= p <= 15:
        raise ValueError(f"no operator file for order {p} (the reference ships p1..p15)")
    if p not in _opcache:
        with np.load(OPERATOR_FIXTURE) as z:
            _opcache[p] = tuple(np.ascontiguousarray(z[f"{k}_p{p}"], dtype=np.float64)
                                for k in ("x1D", "D1D", "D1D_tr", "Lift"))
    return tuple(a.copy() for a in _opcache[p])


def operator_source_digest(p: int) -> str:
    """sha256 of the operator file the arrays of reference_operators(p) came from."""
    with np.load(OPERATOR_FIXTURE) as z:
        return str(z[f"sha256_p{p}"])


class SplitMix64:
    def __init__(self, seed: int):
        self.state = seed & _M64

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & _M64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def uniform(self) -> float:
        return (self.next_u64() >> 11) * (1.0 / 9007199254740992.0)

    def randint(self, lo: int, hi: int) -> int:
        """Uniform integer in [lo, hi]."""
        return lo + int(self.uniform() * (hi - lo + 1))


def node_coords(NeX: int, NeY: int, NeZ: int, x1D: np.ndarray, L=(1.0, 1.0, 1.0)):
    """pos_en(:,:,1..3) as mesh_setup computes them, each flat (Np*Ne)."""
    Nq = len(x1D)
    dx, dy, dz = L[0] / NeX, L[1] / NeY, L[2] / NeZ
    x1D = np.asarray(x1D, dtype=np.float64)
    ex = np.arange(1, NeX + 1, dtype=np.float64)
    ey = np.arange(1, NeY + 1, dtype=np.float64)
    ez = np.arange(1, NeZ + 1, dtype=np.float64)
    # centre + 0.5*dx*x1D(i), evaluated as (xc) + ((0.5*dx)*x1D(i))
    px = ((ex - 0.5) * dx)[None, :] + (0.5 * dx) * x1D[:, None]  # (Nq, NeX)
    py = ((ey - 0.5) * dy)[None, :] + (0.5 * dy) * x1D[:, None]
    pz = ((ez - 0.5) * dz)[None, :] + (0.5 * dz) * x1D[:, None]
    # layout (i, j, k, ex, ey, ez) in Fortran order -> flat index
    # n + Np*e with n = i + Nq j + Nq^2 k and e = ex + NeX ey + NeX NeY ez
    shape = (Nq, Nq, Nq, NeX, NeY, NeZ)
    X = np.broadcast_to(px[:, None, None, :, None, None], shape)
    Y = np.broadcast_to(py[None, :, None, None, :, None], shape)
    Z = np.broadcast_to(pz[None, None, :, None, None, :], shape)
    return (np.ascontiguousarray(X.transpose(5, 4, 3, 2, 1, 0)).reshape(-1),
            np.ascontiguousarray(Y.transpose(5, 4, 3, 2, 1, 0)).reshape(-1),
            np.ascontiguousarray(Z.transpose(5, 4, 3, 2, 1, 0)).reshape(-1))


def sine(NeX, NeY, NeZ, x1D, vel=(1.0, 0.5, 0.25)):
    """(q, u, v, w) of main.f90:144-157 (PI = 4 atan(1))."""
    X, Y, Z = node_coords(NeX, NeY, NeZ, x1D)
    pi = 4.0 * math.atan(1.0)
    q = np.sin(2.0 * pi * X) * np.sin(2.0 * pi * Y) * np.sin(2.0 * pi * Z)
    n = q.size
    return q, np.full(n, vel[0]), np.full(n, vel[1]), np.full(n, vel[2])


def blob_params(seed: int, sigma: float = 0.1):
    """Draws the velocity modes and the tracer centre of one instance."""
    rng = SplitMix64(seed)
    modes = []
    while len(modes) < 4:
        k = [rng.randint(-3, 3) for _ in range(3)]
        kn = math.sqrt(sum(c * c for c in k))
        if not (1.0 <= kn <= 3.0):
            continue
        a = [2.0 * rng.uniform() - 1.0 for _ in range(3)]
        an = math.sqrt(sum(c * c for c in a))
        if an < 1e-3:
            continue
        a = [c / an for c in a]
        phi = 2.0 * math.pi * rng.uniform()
        modes.append((k, a, phi))
    centre = [rng.uniform() for _ in range(3)]
    return {"modes": modes, "centre": centre, "sigma": sigma}


def blob(NeX, NeY, NeZ, x1D, seed: int = BASE_SEED, sigma: float = 0.1):
    """(q, u, v, w): Gaussian tracer in a smooth seeded velocity field."""
    prm = blob_params(seed, sigma)
    X, Y, Z = node_coords(NeX, NeY, NeZ, x1D)
    u = np.full(X.size, U0[0])
    v = np.full(X.size, U0[1])
    w = np.full(X.size, U0[2])
    for k, a, phi in prm["modes"]:
        s = 0.2 * np.sin(2.0 * math.pi * (k[0] * X + k[1] * Y + k[2] * Z) + phi)
        u += a[0] * s
        v += a[1] * s
        w += a[2] * s
    c = prm["centre"]

    def mi(d):  # periodic minimum image on the unit box
        return d - np.round(d)

    d2 = mi(X - c[0]) ** 2 + mi(Y - c[1]) ** 2 + mi(Z - c[2]) ** 2
    q = np.exp(-d2 / (2.0 * sigma * sigma))
    return q, u, v, w


def cfl_dt(NeX, NeY, NeZ, p, u, v, w, cfl: float = 0.1, L=(1.0, 1.0, 1.0)) -> float:
    h = min(L[0] / NeX, L[1] / NeY, L[2] / NeZ)
    vmax = float(np.max(np.abs(u) + np.abs(v) + np.abs(w)))
    return cfl * h / ((2 * p + 1) * vmax)


def with_halo(a: np.ndarray, NeA: int, Np: int) -> np.ndarray:
    """Copies an owned (Np*Ne) field into a zeroed (Np*NeA) array."""
    out = np.zeros(Np * NeA)
    out[: a.size] = a
    return out


def gll_weights(x1D: np.ndarray) -> np.ndarray:
    """GLL quadrature weights w_i = 2 / (N (N+1) P_N(x_i)^2)."""
    N = len(x1D) - 1
    P = np.polynomial.legendre.legval(x1D, [0] * N + [1])
    return 2.0 / (N * (N + 1) * P * P)


def mass(q: np.ndarray, x1D: np.ndarray, NeX, NeY, NeZ, L=(1.0, 1.0, 1.0)) -> float:
    """sum_e sum_n w_i w_j w_k J_e q with J_e = dx dy dz / 8."""
    Nq = len(x1D)
    w1 = gll_weights(np.asarray(x1D))
    w3 = (w1[:, None, None] * w1[None, :, None] * w1[None, None, :]).transpose(2, 1, 0).reshape(-1)
    Ne = NeX * NeY * NeZ
    J = (L[0] / NeX) * (L[1] / NeY) * (L[2] / NeZ) / 8.0
    return float(J * np.sum(q[: Nq ** 3 * Ne].reshape(Ne, Nq ** 3) * w3[None, :]))
