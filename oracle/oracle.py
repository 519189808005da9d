"""ctypes wrapper of the CPU oracle (sdg_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check of
__graft_entry__.py and by the cpu_baseline / reference arm of bench.py, as the
oracle the parity tests compare against or the timed CPU baseline.  The product library never imports
it.  Arrays follow the reference's Fortran column-major layout and are passed
as flat numpy arrays (order='F' views are used for readability in tests).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsdg_oracle.so")
# the same source built for timing (multiply-add contraction, -mcpu=native on
# aarch64); only the timed CPU baseline loads it, never a parity check
FAST_LIB_PATH = os.path.join(HERE, "_build", "libsdg_oracle_fast.so")

GENERAL = 1
OPT1 = 2

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lib = None
_fast_lib = None


def build(force: bool = False) -> str:
    """Compile both oracle builds with the Makefile (gcc, a few seconds)."""
    src = max(os.path.getmtime(os.path.join(HERE, f)) for f in
              ("sdg_oracle.c", "sdg_oracle.h", "Makefile"))
    if force or any(not os.path.exists(p) or os.path.getmtime(p) < src
                    for p in (LIB_PATH, FAST_LIB_PATH)):
        subprocess.run(["make", "-s", "-C", HERE] + (["-B"] if force else []), check=True)
    return LIB_PATH


def lib():
    """The parity build (no multiply-add contraction)."""
    global _lib
    if _lib is None:
        build()
        _lib = _declare(C.CDLL(LIB_PATH))
    return _lib


def fast_lib():
    """The timing build (contraction allowed): for the timed CPU baseline only."""
    global _fast_lib
    if _fast_lib is None:
        build()
        _fast_lib = _declare(C.CDLL(FAST_LIB_PATH))
    return _fast_lib


def _declare(L):
    """Declares the argument types of the exported functions on a loaded build."""
    i = C.c_int
    d = C.c_double
    L.sdgo_read_operator_file.argtypes = [C.c_char_p, i, _dp, _dp, _dp, _dp]
    L.sdgo_read_operator_file.restype = i
    L.sdgo_fmask.argtypes = [i, _ip]
    L.sdgo_nhalo.argtypes = [i, i, i]
    L.sdgo_nhalo.restype = i
    L.sdgo_mesh_setup.argtypes = [i, i, i, i, d, d, d, _dp, _ip, _ip, _dp, _dp, _dp, _dp, _ip]
    L.sdgo_update_halo.argtypes = [_dp, _ip, i, i, i]
    L.sdgo_cal_elembnd_flux.argtypes = [_dp, _dp, _dp, _dp, _dp, _ip, _ip, _dp, _dp, i, i, i, i]
    L.sdgo_divlike.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, i, i]
    L.sdgo_lift.argtypes = [_dp, _dp, _dp, i]
    L.sdgo_gradlike.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp, i]
    L.sdgo_divlike_var5.argtypes = [_dp] * 8 + [i]
    L.sdgo_cal_dqdt.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                i, i, i, i, i, i]
    L.sdgo_cal_tend.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _ip,
                                _dp, _dp, _dp, i, i, i, i, i, i]
    L.sdgo_cal_tend.restype = i
    L.sdgo_rk_stage.argtypes = [_dp, _dp, _dp, i, i, i, d]
    L.sdgo_run.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _ip, _dp,
                           _dp, _dp, _ip, i, i, i, i, d, i, i, C.c_void_p]
    L.sdgo_run.restype = i
    L.sdgo_ic_sine.argtypes = [_dp, _dp, _dp, _dp, _dp, i, i, d, d, d]
    L.sdgo_num_threads.restype = i
    return L


def num_threads() -> int:
    return lib().sdgo_num_threads()


def read_operator_file(path: str, p: int):
    """(x1D, D1D, D1D_tr, Lift) read as element_init does (mod_mesh.f90:253-263)."""
    Nq = p + 1
    x = np.zeros(Nq)
    D = np.zeros(Nq * Nq)
    Dt = np.zeros(Nq * Nq)
    L = np.zeros(6 * Nq ** 3)
    st = lib().sdgo_read_operator_file(path.encode(), p, x, D, Dt, L)
    if st != 0:
        raise IOError(f"operator file {path}: status {st}")
    return x, D, Dt, L


def fmask(p: int) -> np.ndarray:
    Nq = p + 1
    out = np.zeros(6 * Nq * Nq, dtype=np.int32)
    lib().sdgo_fmask(p, out)
    return out


class Mesh:
    """mesh_setup outputs (mod_mesh.f90:74-193) for the periodic unit box."""

    def __init__(self, NeX, NeY, NeZ, p, x1D, L=(1.0, 1.0, 1.0)):
        self.NeX, self.NeY, self.NeZ, self.p = NeX, NeY, NeZ, p
        self.Nq = Nq = p + 1
        self.Np = Np = Nq ** 3
        self.Nfp = Nq * Nq
        self.NfpTot = NfpTot = 6 * Nq * Nq
        self.Ne = Ne = NeX * NeY * NeZ
        self.Nhalo = lib().sdgo_nhalo(NeX, NeY, NeZ)
        self.NeA = Ne + self.Nhalo
        self.NhaloNode = self.Nfp * self.Nhalo
        self.VMapM = np.zeros(NfpTot * Ne, dtype=np.int32)
        self.VMapP = np.zeros(NfpTot * Ne, dtype=np.int32)
        self.normal_fn = np.zeros(NfpTot * Ne * 3)
        self.Escale = np.zeros(Np * Ne * 3)
        self.Fscale = np.zeros(NfpTot * Ne)
        self.pos_en = np.zeros(Np * Ne * 3)
        self.halo_src_map = np.zeros(self.NhaloNode, dtype=np.int32)
        lib().sdgo_mesh_setup(NeX, NeY, NeZ, p, float(L[0]), float(L[1]), float(L[2]),
                              np.ascontiguousarray(x1D, dtype=np.float64), self.VMapM, self.VMapP,
                              self.normal_fn, self.Escale, self.Fscale, self.pos_en,
                              self.halo_src_map)

    def field(self) -> np.ndarray:
        """A zeroed (Np, NeA) field, flat."""
        return np.zeros(self.Np * self.NeA)

    def update_halo(self, f: np.ndarray) -> None:
        lib().sdgo_update_halo(f, self.halo_src_map, self.Np, self.Ne, self.NhaloNode)


def cal_tend(mesh: Mesh, q, u, v, w, D, Dt, Lift, opt=OPT1) -> np.ndarray:
    """advect3d_eq_cal_tend (mod_advect3d_eq.f90:41-85); q,u,v,w are (Np,NeA)
    with halos filled.  Returns dqdt (Np,NeA), owned part written."""
    m = mesh
    dqdt = np.zeros(m.Np * m.NeA)
    st = lib().sdgo_cal_tend(dqdt, q, u, v, w, D, Dt, Lift, m.VMapM, m.VMapP, m.normal_fn,
                             m.Escale, m.Fscale, m.Nq, m.Np, m.NfpTot, m.Ne, m.NeA, opt)
    if st:
        raise RuntimeError(f"oracle cal_tend status {st}")
    return dqdt


def elembnd_flux(mesh: Mesh, q, u, v, w) -> np.ndarray:
    m = mesh
    flux = np.zeros(m.NfpTot * m.Ne)
    lib().sdgo_cal_elembnd_flux(flux, q, u, v, w, m.VMapM, m.VMapP, m.normal_fn, m.Fscale,
                                m.Np, m.NfpTot, m.Ne, m.NeA)
    return flux


def divlike(D, Dt, fx, fy, fz, Nq, opt=OPT1):
    Np = Nq ** 3
    ox, oy, oz = np.zeros(Np), np.zeros(Np), np.zeros(Np)
    lib().sdgo_divlike(ox, oy, oz, D, Dt, np.ascontiguousarray(fx), np.ascontiguousarray(fy),
                       np.ascontiguousarray(fz), Nq, opt)
    return ox, oy, oz


def gradlike(D, Dt, f, Nq):
    """gradlike_dirXYZ of one element's field (erb:166-219, z along k)."""
    Np = Nq ** 3
    ox, oy, oz = np.zeros(Np), np.zeros(Np), np.zeros(Np)
    lib().sdgo_gradlike(ox, oy, oz, D, Dt, np.ascontiguousarray(f, dtype=np.float64), Nq)
    return ox, oy, oz


def divlike_var5(D, Dt, fx, fy, fz, Nq):
    """divlike_dirXYZ_var5 of one element, (Nq,Nq,Nq,5) arrays (erb:347-465)."""
    n = 5 * Nq ** 3
    ox, oy, oz = np.zeros(n), np.zeros(n), np.zeros(n)
    lib().sdgo_divlike_var5(ox, oy, oz, D, Dt, *[np.ascontiguousarray(a, dtype=np.float64)
                                                 for a in (fx, fy, fz)], Nq)
    return ox, oy, oz


def lift(Lift, flux_e, Nq):
    out = np.zeros(Nq ** 3)
    lib().sdgo_lift(out, Lift, np.ascontiguousarray(flux_e), Nq)
    return out


def run(mesh: Mesh, q, u, v, w, D, Dt, Lift, dt, nstep, opt=OPT1, minmax=False, fast=False):
    """Time loop of main.f90:51-80.  q is updated in place ((Np,NeA), owned
    part meaningful).  Returns the per-step (min, max) array when asked.
    fast=True runs the timing build (for the timed CPU baseline only)."""
    m = mesh
    q0 = np.zeros_like(q)
    dqdt = np.zeros_like(q)
    mm = np.zeros(2 * max(nstep, 1)) if minmax else None
    st = (fast_lib() if fast else lib()).sdgo_run(q, q0, dqdt, u, v, w, D, Dt, Lift, m.VMapM, m.VMapP, m.normal_fn,
                        m.Escale, m.Fscale, m.halo_src_map, m.Nq, m.Ne, m.NeA, m.NhaloNode,
                        float(dt), int(nstep), opt,
                        mm.ctypes.data_as(C.c_void_p) if mm is not None else None)
    if st:
        raise RuntimeError(f"oracle run status {st}")
    return mm.reshape(-1, 2) if mm is not None else None


def rk_stage(q, q0, dqdt, Np, Ne, stage, dt):
    lib().sdgo_rk_stage(q, q0, dqdt, Np, Ne, stage, float(dt))


def ic_sine(mesh: Mesh, vel=(1.0, 1.0, 1.0)):
    """main.f90:144-162: returns (q,u,v,w) as (Np,NeA) with halos filled."""
    m = mesh
    q, u, v, w = m.field(), m.field(), m.field(), m.field()
    lib().sdgo_ic_sine(q, u, v, w, m.pos_en, m.Np, m.Ne, float(vel[0]), float(vel[1]),
                       float(vel[2]))
    for f in (q, u, v, w):
        m.update_halo(f)
    return q, u, v, w
