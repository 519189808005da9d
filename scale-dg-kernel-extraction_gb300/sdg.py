"""Python binding of libsdg_gb300 (the C ABI declared in include/sdg_advect.h).

The names mirror the reference's Fortran interface -- dg_optr_kernel_setup,
advect3d_eq_cal_tend, tensorprod_divlike_dirXYZ, tensorprod_Lift_hexahedral,
update_halo -- with the same argument meaning, so a test reads like the
reference's driver (main.f90).  Arrays are flat numpy arrays in the reference's
column-major layout.  A nonzero status raises SdgError carrying the status and
the library's message.

The compute path is the CUDA library only: importing this module loads
libsdg_gb300.so and raises if it has not been built; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsdg_gb300.so")

OK = 0
ERR_INVALID_ARG = -1
ERR_UNSUPPORTED_ORDER = -2
ERR_BAD_OPTTYPE = -3
ERR_CUDA = -4
ERR_OUT_OF_MEMORY = -5
ERR_FILE = -6
ERR_MESH = -7
ERR_TIMEOUT = -8
ERR_NO_DEVICE = -9

OPT_GENERAL = 1
OPT_OPT1 = 2
PREC_FP64 = 0
PREC_FP32 = 1
PREC_FP64_EMU = 2

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_vp = C.c_void_p
_i = C.c_int
_d = C.c_double


class SdgError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        self.status = status
        super().__init__(f"{where}: status {status}: {message}")


def _load() -> C.CDLL:
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is not built; run `python build.py` in {HERE} "
            "(there is no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    sig = {
        "sdg_status_string": ([_i], C.c_char_p),
        "sdg_last_error": ([], C.c_char_p),
        "sdg_version": ([], C.c_char_p),
        "sdg_device_count": ([], _i),
        "sdg_device_synchronize": ([], _i),
        "sdg_set_device": ([_i], _i),
        "sdg_operator_read": ([C.c_char_p, _i, _dp, _dp, _vp, _dp], _i),
        "sdg_operator_generate": ([_i, _dp, _dp, _vp, _dp], _i),
        "sdg_dg_optr_kernel_setup": ([C.c_char_p], _i),
        "sdg_dg_optr_kernel_type": ([], _i),
        "sdg_advect3d_eq_cal_tend": ([_dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _ip,
                                      _dp, _dp, _dp, _i, _i, _i, _i, _i], _i),
        "sdg_advect3d_eq_cal_tend_dev": ([_vp] * 13 + [_i] * 6 + [_vp, _vp, _vp], _i),
        "sdg_tensorprod_divlike_dirXYZ": ([_dp] * 8 + [_i, _i], _i),
        "sdg_tensorprod_divlike_dirXYZ_dev": ([_vp] * 8 + [_i, _i, _i, _vp], _i),
        "sdg_tensorprod_Lift_hexahedral": ([_dp, _dp, _dp, _i, _i], _i),
        "sdg_tensorprod_Lift_hexahedral_dev": ([_vp, _vp, _vp, _i, _i, _vp], _i),
        "sdg_update_halo_dev": ([_vp, _vp, _i, _i, _i, _vp], _i),
        "sdg_rk_stage_dev": ([_vp, _vp, _vp, _i, _i, _i, _d, _vp], _i),
        "sdg_solver_create": ([C.POINTER(_vp), _i, _i, _i, _i, _d, _d, _d, _dp, _dp, _i, _i,
                               _vp], _i),
        "sdg_solver_check_mesh": ([_vp, _ip, _ip, _dp, _dp, _dp], _i),
        "sdg_solver_upload": ([_vp, _vp, _vp, _vp, _vp], _i),
        "sdg_solver_upload_dev": ([_vp, _vp, _vp, _vp, _vp], _i),
        "sdg_solver_step": ([_vp, _d, _i], _i),
        "sdg_solver_step_timed": ([_vp, _d, _i, C.POINTER(_d)], _i),
        "sdg_solver_download": ([_vp, _vp], _i),
        "sdg_solver_state_dev": ([_vp], _vp),
        "sdg_solver_tendency": ([_vp, _dp], _i),
        "sdg_solver_launches_per_step": ([_vp], _i),
        "sdg_solver_stream": ([_vp], _vp),
        "sdg_solver_destroy": ([_vp], _i),
        "sdg_dev_alloc": ([C.c_size_t, C.POINTER(_vp)], _i),
        "sdg_dev_free": ([_vp], _i),
        "sdg_memcpy_h2d": ([_vp, _vp, C.c_size_t], _i),
        "sdg_memcpy_d2h": ([_vp, _vp, C.c_size_t], _i),
        "sdg_memset_dev": ([_vp, _i, C.c_size_t], _i),
        "sdg_pinned_alloc": ([C.c_size_t, C.POINTER(_vp)], _i),
        "sdg_pinned_free": ([_vp], _i),
        "sdg_microbench_peaks": ([C.POINTER(_d)] * 4, _i),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    return L


lib = _load()


def _check(st: int, where: str) -> None:
    if st != OK:
        raise SdgError(st, where, lib.sdg_last_error().decode(errors="replace"))


def status_string(st: int) -> str:
    return lib.sdg_status_string(st).decode()


def device_count() -> int:
    return lib.sdg_device_count()


def set_device(device: int) -> None:
    _check(lib.sdg_set_device(device), "sdg_set_device")


def synchronize() -> None:
    _check(lib.sdg_device_synchronize(), "sdg_device_synchronize")


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64).reshape(-1)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32).reshape(-1)


# ---- operator data (mod_mesh.f90:226-327) ---------------------------------

def operator_read(path: str, p: int):
    """(x1D, D1D, D1D_tr, Lift_mat) from operator_data/p<p>.dat."""
    Nq = p + 1
    x, D, Dt, L = np.zeros(Nq), np.zeros(Nq * Nq), np.zeros(Nq * Nq), np.zeros(6 * Nq ** 3)
    _check(lib.sdg_operator_read(path.encode(), p, x, D, Dt.ctypes.data, L), "sdg_operator_read")
    return x, D, Dt, L


def operator_generate(p: int):
    """(x1D, D1D, D1D_tr, Lift_mat) computed from the GLL mathematics."""
    Nq = p + 1
    x, D, Dt, L = np.zeros(Nq), np.zeros(Nq * Nq), np.zeros(Nq * Nq), np.zeros(6 * Nq ** 3)
    _check(lib.sdg_operator_generate(p, x, D, Dt.ctypes.data, L), "sdg_operator_generate")
    return x, D, Dt, L


# ---- the reference's entry points ------------------------------------------

def dg_optr_kernel_setup(dgoptr_evaltype: str) -> None:
    """mod_dg_optr_kernel.f90:45-58; raises on an unsupported type."""
    _check(lib.sdg_dg_optr_kernel_setup(dgoptr_evaltype.encode()), "dg_optr_kernel_setup")


def dg_optr_kernel_type() -> int:
    return lib.sdg_dg_optr_kernel_type()


def advect3d_eq_cal_tend(dqdt, q, u, v, w, D1D, D1D_tr, Lift_mat, VMapM, VMapP, normal_fn,
                         Escale, Fscale, Nq, Np, NfpTot, Ne, NeA) -> None:
    """mod_advect3d_eq.f90:41-85 on host arrays; dqdt(:,1:Ne) is written in place."""
    if not (isinstance(dqdt, np.ndarray) and dqdt.dtype == np.float64 and dqdt.flags.c_contiguous):
        raise TypeError("dqdt must be a contiguous float64 array")
    _check(lib.sdg_advect3d_eq_cal_tend(
        dqdt.reshape(-1), _f64(q), _f64(u), _f64(v), _f64(w), _f64(D1D), _f64(D1D_tr),
        _f64(Lift_mat), _i32(VMapM), _i32(VMapP), _f64(normal_fn), _f64(Escale), _f64(Fscale),
        Nq, Np, NfpTot, Ne, NeA), "advect3d_eq_cal_tend")


def tensorprod_divlike_dirXYZ(Mat, Mat_tr, vec_in_x, vec_in_y, vec_in_z, Nq):
    """mod_dg_optr_kernel.f90:62-136 over len(vec_in_x)//Nq^3 elements."""
    ix, iy, iz = _f64(vec_in_x), _f64(vec_in_y), _f64(vec_in_z)
    nelem = ix.size // Nq ** 3
    ox, oy, oz = np.zeros_like(ix), np.zeros_like(iy), np.zeros_like(iz)
    _check(lib.sdg_tensorprod_divlike_dirXYZ(ox, oy, oz, _f64(Mat), _f64(Mat_tr), ix, iy, iz,
                                             Nq, nelem), "tensorprod_divlike_dirXYZ")
    return ox, oy, oz


def tensorprod_Lift_hexahedral(Lift, vec_in, Nq):
    """mod_dg_optr_kernel.f90:139-190 over len(vec_in)//(6 Nq^2) elements."""
    vi = _f64(vec_in)
    nelem = vi.size // (6 * Nq * Nq)
    out = np.zeros(nelem * Nq ** 3)
    _check(lib.sdg_tensorprod_Lift_hexahedral(out, _f64(Lift), vi, Nq, nelem),
           "tensorprod_Lift_hexahedral")
    return out


# ---- device memory for the *_dev entry points ------------------------------

class DeviceArray:
    """Device memory holding a copy of a numpy array (for the *_dev calls)."""

    def __init__(self, src=None, n: int = 0, dtype=np.float64):
        if src is not None:
            src = np.ascontiguousarray(src)
            dtype, n = src.dtype, src.size
        self.dtype = np.dtype(dtype)
        self.n = int(n)
        self._ptr = _vp()
        _check(lib.sdg_dev_alloc(self.n * self.dtype.itemsize, C.byref(self._ptr)),
               "sdg_dev_alloc")
        if src is not None:
            self.upload(src)

    @property
    def ptr(self) -> int:
        return self._ptr.value

    def upload(self, src) -> None:
        src = np.ascontiguousarray(src, dtype=self.dtype)
        _check(lib.sdg_memcpy_h2d(self.ptr, src.ctypes.data, src.nbytes), "sdg_memcpy_h2d")

    def zero(self) -> None:
        _check(lib.sdg_memset_dev(self.ptr, 0, self.n * self.dtype.itemsize), "sdg_memset_dev")

    def numpy(self) -> np.ndarray:
        out = np.empty(self.n, dtype=self.dtype)
        _check(lib.sdg_memcpy_d2h(out.ctypes.data, self.ptr, out.nbytes), "sdg_memcpy_d2h")
        return out

    def free(self) -> None:
        if self._ptr is not None and self._ptr.value:
            lib.sdg_dev_free(self._ptr)
        self._ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class PinnedArray:
    """A numpy view of page-locked host memory (freed with .free() or GC)."""

    def __init__(self, n: int, dtype=np.float64):
        dtype = np.dtype(dtype)
        self._ptr = _vp()
        _check(lib.sdg_pinned_alloc(n * dtype.itemsize, C.byref(self._ptr)), "sdg_pinned_alloc")
        buf = (C.c_char * (n * dtype.itemsize)).from_address(self._ptr.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=n)

    @property
    def ptr(self) -> int:
        return self._ptr.value

    def free(self) -> None:
        if self._ptr is not None and self._ptr.value:
            lib.sdg_pinned_free(self._ptr)
        self._ptr = None
        self.array = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Solver:
    """Device-resident periodic-box solver (sdg_solver_* in include/sdg_advect.h)."""

    def __init__(self, NeX, NeY, NeZ, p, D1D, Lift_mat, opt=OPT_OPT1, precision=PREC_FP64,
                 L=(1.0, 1.0, 1.0), stream=None):
        self._h = _vp()
        self.NeX, self.NeY, self.NeZ, self.p = NeX, NeY, NeZ, p
        self.Np = (p + 1) ** 3
        self.Ne = NeX * NeY * NeZ
        self.ndof = self.Np * self.Ne
        _check(lib.sdg_solver_create(C.byref(self._h), NeX, NeY, NeZ, p, float(L[0]),
                                     float(L[1]), float(L[2]), _f64(D1D), _f64(Lift_mat), opt,
                                     precision, stream), "sdg_solver_create")

    @property
    def handle(self):
        return self._h

    def check_mesh(self, VMapM, VMapP, normal_fn, Escale, Fscale) -> None:
        _check(lib.sdg_solver_check_mesh(self._h, _i32(VMapM), _i32(VMapP), _f64(normal_fn),
                                         _f64(Escale), _f64(Fscale)), "sdg_solver_check_mesh")

    def _owned(self, a) -> np.ndarray:
        a = _f64(a)
        if a.size < self.ndof:
            raise ValueError("field smaller than Np*Ne")
        return a

    def upload(self, q, u, v, w) -> None:
        arrs = [self._owned(x) for x in (q, u, v, w)]
        _check(lib.sdg_solver_upload(self._h, *[x.ctypes.data for x in arrs]),
               "sdg_solver_upload")
        self._keep = arrs  # keep alive until the asynchronous copy has run

    def upload_ptrs(self, q, u, v, w) -> None:
        """Host pointers (e.g. PinnedArray.ptr) of Np*Ne doubles each."""
        _check(lib.sdg_solver_upload(self._h, q, u, v, w), "sdg_solver_upload")

    def step(self, dt: float, nstep: int) -> None:
        _check(lib.sdg_solver_step(self._h, float(dt), int(nstep)), "sdg_solver_step")

    def step_timed(self, dt: float, nstep: int) -> float:
        """Steps and returns the device time in milliseconds (CUDA events)."""
        ms = _d()
        _check(lib.sdg_solver_step_timed(self._h, float(dt), int(nstep), C.byref(ms)),
               "sdg_solver_step_timed")
        return ms.value

    def download(self, out=None) -> np.ndarray:
        out = np.zeros(self.ndof) if out is None else out
        _check(lib.sdg_solver_download(self._h, out.ctypes.data), "sdg_solver_download")
        return out

    def download_ptr(self, ptr: int) -> None:
        _check(lib.sdg_solver_download(self._h, ptr), "sdg_solver_download")

    def tendency(self) -> np.ndarray:
        out = np.zeros(self.ndof)
        _check(lib.sdg_solver_tendency(self._h, out), "sdg_solver_tendency")
        return out

    @property
    def launches_per_step(self) -> int:
        return lib.sdg_solver_launches_per_step(self._h)

    @property
    def stream(self):
        return lib.sdg_solver_stream(self._h)

    def close(self) -> None:
        if self._h is not None and self._h.value:
            lib.sdg_solver_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def microbench_peaks() -> dict:
    v = [_d() for _ in range(4)]
    _check(lib.sdg_microbench_peaks(*[C.byref(x) for x in v]), "sdg_microbench_peaks")
    return {"dfma_tflops": v[0].value, "ffma_tflops": v[1].value,
            "cvt_roundtrip_tops": v[2].value}
