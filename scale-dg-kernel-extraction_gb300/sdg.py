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
OPT_EVENODD = 3  # solver only: even-odd FP64 stage
PREC_FP64 = 0
PREC_FP32 = 1
PREC_FP64_EMU = 2

class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("hbm_budget_bytes", C.c_size_t), ("max_active", C.c_int),
                ("max_window_steps", C.c_int), ("threads", C.c_int),
                ("epb_by_order", C.c_int * 16), ("opt", C.c_int),
                ("threads_by_order", C.c_int * 16), ("parallel_groups", C.c_int)]


class Request(C.Structure):
    _fields_ = [("NeX", C.c_int), ("NeY", C.c_int), ("NeZ", C.c_int), ("p", C.c_int),
                ("nstep", C.c_int), ("dt", C.c_double), ("centre", C.c_double * 3),
                ("sigma", C.c_double), ("velocity", C.c_double * 3)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int), ("latency_s", C.c_double), ("queue_s", C.c_double),
                ("dofs", C.c_longlong)]


class ServerStats(C.Structure):
    _fields_ = [("completed", C.c_longlong), ("steps_run", C.c_longlong),
                ("launches", C.c_longlong), ("dof_updates", C.c_double),
                ("bytes_in_use", C.c_size_t), ("active", C.c_int), ("pending", C.c_int),
                ("p50_latency_s", C.c_double), ("p99_latency_s", C.c_double),
                ("span_s", C.c_double), ("fatal_status", C.c_int)]


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
        "sdg_struct_size": ([C.c_char_p], C.c_size_t),
        "sdg_device_count": ([], _i),
        "sdg_device_synchronize": ([], _i),
        "sdg_set_device": ([_i], _i),
        "sdg_operator_read": ([C.c_char_p, _i, _dp, _dp, _vp, _dp], _i),
        "sdg_operator_generate": ([_i, _dp, _dp, _vp, _dp], _i),
        "sdg_evenodd_tables": ([_i, _dp, _dp, _dp], _i),
        "sdg_dg_optr_kernel_setup": ([C.c_char_p], _i),
        "sdg_dg_optr_kernel_type": ([], _i),
        "sdg_advect3d_eq_cal_tend": ([_dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _ip,
                                      _dp, _dp, _dp, _i, _i, _i, _i, _i], _i),
        "sdg_advect3d_eq_cal_tend_dev": ([_vp] * 13 + [_i] * 6 + [_vp, _vp, _vp], _i),
        "sdg_tensorprod_divlike_dirXYZ": ([_dp] * 8 + [_i, _i], _i),
        "sdg_tensorprod_divlike_dirXYZ_dev": ([_vp] * 8 + [_i, _i, _i, _vp], _i),
        "sdg_element_matvec_dir": ([_i, _dp, _dp, _dp, _i, _i], _i),
        "sdg_element_matvec_dir_dev": ([_i, _vp, _vp, _vp, _i, _i, _vp], _i),
        "sdg_tensorprod_gradlike_dirXYZ": ([_dp] * 6 + [_i, _i], _i),
        "sdg_tensorprod_gradlike_dirXYZ_dev": ([_vp] * 6 + [_i, _i, _vp], _i),
        "sdg_tensorprod_divlike_dirXYZ_var5": ([_dp] * 8 + [_i, _i], _i),
        "sdg_tensorprod_divlike_dirXYZ_var5_dev": ([_vp] * 8 + [_i, _i, _vp], _i),
        "sdg_tensorprod_Lift_hexahedral": ([_dp, _dp, _dp, _i, _i], _i),
        "sdg_tensorprod_Lift_hexahedral_dev": ([_vp, _vp, _vp, _i, _i, _vp], _i),
        "sdg_update_halo_dev": ([_vp, _vp, _i, _i, _i, _vp], _i),
        "sdg_minmax_dev": ([_vp, C.c_longlong, _vp, _vp, _vp], _i),
        "sdg_solver_minmax": ([_vp, _vp, _vp], _i),
        "sdg_solver_run": ([_vp, _d, _i, _i, _vp], _i),
        "sdg_mesh_setup_dev": ([_i, _i, _i, _i, _d, _d, _d, _vp] + [_vp] * 7 + [_vp], _i),
        "sdg_rk_stage_dev": ([_vp, _vp, _vp, _i, _i, _i, _d, _vp], _i),
        "sdg_advect3d_eq_step_scratch_bytes": ([_i, _i], C.c_size_t),
        "sdg_slab_plan": ([_i, _i, _ip, _ip, _ip], _i),
        "sdg_tensorprod_divlike_dirXYZ_f32_dev": ([_vp] * 7 + [_i, _i, _i, _vp, _vp], _i),
        "sdg_slabs_create": ([C.POINTER(_vp), _i, _i, _i, _i, _d, _d, _d, _dp, _dp, _i, _i, _i,
                              _vp], _i),
        "sdg_slabs_upload": ([_vp, _vp, _vp, _vp, _vp], _i),
        "sdg_slabs_step": ([_vp, _d, _i], _i),
        "sdg_slabs_download": ([_vp, _vp], _i),
        "sdg_slabs_exchange_bytes": ([_vp], C.c_longlong),
        "sdg_slabs_destroy": ([_vp], _i),
        "sdg_advect3d_eq_step_dev": ([_vp] * 13 + [_i] * 6 + [_d, _i, _i, _vp, C.c_size_t,
                                                          _vp, _vp], _i),
        "sdg_solver_create": ([C.POINTER(_vp), _i, _i, _i, _i, _d, _d, _d, _dp, _dp, _i, _i,
                               _vp], _i),
        "sdg_solver_check_mesh": ([_vp, _ip, _ip, _dp, _dp, _dp], _i),
        "sdg_solver_upload": ([_vp, _vp, _vp, _vp, _vp], _i),
        "sdg_solver_upload_dev": ([_vp, _vp, _vp, _vp, _vp], _i),
        "sdg_solver_step": ([_vp, _d, _i], _i),
        "sdg_solver_step_timed": ([_vp, _d, _i, C.POINTER(_d)], _i),
        "sdg_solver_download": ([_vp, _vp], _i),
        "sdg_solver_solve_host_pipelined": ([_vp, _i, C.POINTER(_vp), C.POINTER(_vp),
                                             C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), _d,
                                             _i], _i),
        "sdg_solver_state_dev": ([_vp], _vp),
        "sdg_solver_tendency": ([_vp, _dp], _i),
        "sdg_solver_launches_per_step": ([_vp], _i),
        "sdg_solver_stream": ([_vp], _vp),
        "sdg_solver_destroy": ([_vp], _i),
        "sdg_dev_alloc": ([C.c_size_t, C.POINTER(_vp)], _i),
        "sdg_dev_free": ([_vp], _i),
        "sdg_memcpy_h2d": ([_vp, _vp, C.c_size_t], _i),
        "sdg_memcpy_d2h": ([_vp, _vp, C.c_size_t], _i),
        "sdg_memcpy_d2d_async": ([_vp, _vp, C.c_size_t, _vp], _i),
        "sdg_memset_dev": ([_vp, _i, C.c_size_t], _i),
        "sdg_pinned_alloc": ([C.c_size_t, C.POINTER(_vp)], _i),
        "sdg_pinned_free": ([_vp], _i),
        "sdg_microbench_peaks": ([C.POINTER(_d)] * 4, _i),
        "sdg_ensemble_create": ([C.POINTER(_vp), _i, _ip, _ip, _dp, C.POINTER(_vp),
                                 C.POINTER(_vp), C.POINTER(_vp), _vp], _i),
        "sdg_ensemble_upload": ([_vp, _i, _dp, _dp, _dp, _dp], _i),
        "sdg_ensemble_init_blob": ([_vp, _i, _dp, _d, _dp], _i),
        "sdg_ensemble_tune": ([_vp], _i),
        "sdg_ensemble_set_epb": ([_vp, _i, _i], _i),
        "sdg_ensemble_set_opt": ([_vp, _i], _i),
        "sdg_ensemble_set_threads": ([_vp, _i], _i),
        "sdg_ensemble_set_order_threads": ([_vp, _i, _i], _i),
        "sdg_ensemble_get_threads": ([_vp, _ip], _i),
        "sdg_ensemble_set_parallel_groups": ([_vp, _i], _i),
        "sdg_ensemble_set_single_launch": ([_vp, _i], _i),
        "sdg_ensemble_get_config": ([_vp, _ip, C.POINTER(_i), C.POINTER(_i)], _i),
        "sdg_ensemble_get_bodies": ([_vp, _ip], _i),
        "sdg_ensemble_step": ([_vp, _i], _i),
        "sdg_ensemble_step_timed": ([_vp, _i, C.POINTER(_d)], _i),
        "sdg_ensemble_download": ([_vp, _i, _dp], _i),
        "sdg_ensemble_total_dofs": ([_vp], C.c_longlong),
        "sdg_ensemble_launches_per_step": ([_vp], _i),
        "sdg_ensemble_destroy": ([_vp], _i),
        "sdg_server_create": ([C.POINTER(_vp), C.POINTER(ServerConfig), C.POINTER(_vp),
                               C.POINTER(_vp), C.POINTER(_vp)], _i),
        "sdg_server_submit": ([_vp, C.POINTER(Request), _vp, C.POINTER(C.c_uint64)], _i),
        "sdg_server_wait": ([_vp, C.c_uint64, _d, C.POINTER(Result)], _i),
        "sdg_server_get_stats": ([_vp, C.POINTER(ServerStats)], _i),
        "sdg_server_reset_stats": ([_vp], _i),
        "sdg_server_inject_rebuild_failure": ([_vp], _i),
        "sdg_server_destroy": ([_vp], _i),
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


def evenodd_tables(Nq: int, D1D, Lift_mat) -> np.ndarray:
    """The even-odd tables of an order (3 x TE values; see sdg_advect.h)."""
    N = Nq
    H, HR, odd = N // 2, (N + 1) // 2, N & 1
    te = H * H + HR * H + odd * H + HR + H
    out = np.zeros(3 * te)
    _check(lib.sdg_evenodd_tables(Nq, _f64(D1D), _f64(Lift_mat), out), "sdg_evenodd_tables")
    return out


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


def element_matvec_dir(dir: int, Mat, vec_in, Nq):
    """matvec_dirX/Y/Z (opt1 erb:51-129), dir 1..3, over len(vec_in)//Nq^3
    elements; Mat is Mat_x, Mat_y_tr or Mat_z_tr."""
    vi = _f64(vec_in)
    out = np.zeros_like(vi)
    _check(lib.sdg_element_matvec_dir(int(dir), out, _f64(Mat), vi, Nq, vi.size // Nq ** 3),
           "element_matvec_dir")
    return out


def tensorprod_gradlike_dirXYZ(Mat, Mat_tr, vec_in, Nq):
    """gradlike_dirXYZ (opt1 erb:166-219) over len(vec_in)//Nq^3 elements."""
    vi = _f64(vec_in)
    nelem = vi.size // Nq ** 3
    ox, oy, oz = np.zeros_like(vi), np.zeros_like(vi), np.zeros_like(vi)
    _check(lib.sdg_tensorprod_gradlike_dirXYZ(ox, oy, oz, _f64(Mat), _f64(Mat_tr), vi, Nq,
                                              nelem), "tensorprod_gradlike_dirXYZ")
    return ox, oy, oz


def tensorprod_divlike_dirXYZ_var5(Mat, Mat_tr, vec_in_x, vec_in_y, vec_in_z, Nq):
    """divlike_dirXYZ_var5 (opt1 erb:347-465) over len(vec_in_x)//(5 Nq^3)
    elements, each (Nq,Nq,Nq,5)."""
    ix, iy, iz = _f64(vec_in_x), _f64(vec_in_y), _f64(vec_in_z)
    nelem = ix.size // (5 * Nq ** 3)
    ox, oy, oz = np.zeros_like(ix), np.zeros_like(iy), np.zeros_like(iz)
    _check(lib.sdg_tensorprod_divlike_dirXYZ_var5(ox, oy, oz, _f64(Mat), _f64(Mat_tr), ix, iy,
                                                  iz, Nq, nelem),
           "tensorprod_divlike_dirXYZ_var5")
    return ox, oy, oz


def tensorprod_Lift_hexahedral(Lift, vec_in, Nq):
    """mod_dg_optr_kernel.f90:139-190 over len(vec_in)//(6 Nq^2) elements."""
    vi = _f64(vec_in)
    nelem = vi.size // (6 * Nq * Nq)
    out = np.zeros(nelem * Nq ** 3)
    _check(lib.sdg_tensorprod_Lift_hexahedral(out, _f64(Lift), vi, Nq, nelem),
           "tensorprod_Lift_hexahedral")
    return out


def tensorprod_divlike_dirXYZ_f32(D1D, in_x, in_y, in_z, Nq, tensor_cores=True):
    """FP32 divlike of len(in_x) // Nq^3 elements through
    sdg_tensorprod_divlike_dirXYZ_f32_dev (tensor cores at Nq = 16, else the
    CUDA-core form).  Returns (out_x, out_y, out_z) as float32 arrays."""
    ins = [DeviceArray(np.ascontiguousarray(a, dtype=np.float32)) for a in (in_x, in_y, in_z)]
    n = ins[0].n
    nelem = n // Nq ** 3
    outs = [DeviceArray(n=n, dtype=np.float32) for _ in range(3)]
    Dd = DeviceArray(np.ascontiguousarray(D1D, dtype=np.float32))
    err = DeviceArray(np.zeros(1, dtype=np.int32))
    _check(lib.sdg_tensorprod_divlike_dirXYZ_f32_dev(
        outs[0].ptr, outs[1].ptr, outs[2].ptr, Dd.ptr, ins[0].ptr, ins[1].ptr, ins[2].ptr, Nq,
        nelem, 1 if tensor_cores else 0, err.ptr, None), "tensorprod_divlike_dirXYZ_f32")
    if int(err.numpy()[0]):
        raise SdgError(ERR_TIMEOUT, "tensorprod_divlike_dirXYZ_f32",
                       "the tensor-core wait ran out")
    return tuple(o.numpy() for o in outs)


def advect3d_eq_step(q, u, v, w, D1D, D1D_tr, Lift_mat, VMapM, VMapP, normal_fn, Escale,
                     Fscale, halo_src_map, Nq, Np, NfpTot, Ne, NeA, NhaloNode, dt, nstep,
                     opt=OPT_EVENODD):
    """nstep SSP-RK3 steps of the time loop of main.f90:51-80 on the
    reference's arrays through sdg_advect3d_eq_step_dev: uploads every array,
    runs, and returns q (Np*NeA, halo slots refreshed).  Raises SdgError with
    status ERR_MESH / ERR_INVALID_ARG when the device reports a bad map entry
    or operators without the even-odd symmetries."""
    arrs = [DeviceArray(_f64(a)) for a in (q, u, v, w, D1D, D1D_tr, Lift_mat)]
    maps = [DeviceArray(np.ascontiguousarray(a, dtype=np.int32)) for a in (VMapM, VMapP)]
    geo = [DeviceArray(_f64(a)) for a in (normal_fn, Escale, Fscale)]
    hm = DeviceArray(np.ascontiguousarray(halo_src_map, dtype=np.int32)) if NhaloNode > 0 \
        else None
    nbytes = int(lib.sdg_advect3d_eq_step_scratch_bytes(Nq, Ne))
    scratch = DeviceArray(n=max(nbytes, 1), dtype=np.uint8)
    err = DeviceArray(np.zeros(1, dtype=np.int32))
    _check(lib.sdg_advect3d_eq_step_dev(
        arrs[0].ptr, arrs[1].ptr, arrs[2].ptr, arrs[3].ptr, arrs[4].ptr, arrs[5].ptr, arrs[6].ptr,
        maps[0].ptr, maps[1].ptr, geo[0].ptr, geo[1].ptr, geo[2].ptr,
        hm.ptr if hm is not None else None, Nq, Np, NfpTot, Ne, NeA, NhaloNode, float(dt),
        int(nstep), int(opt), scratch.ptr, nbytes, err.ptr, None), "sdg_advect3d_eq_step_dev")
    flag = int(err.numpy()[0])
    if flag == 2:
        raise SdgError(ERR_INVALID_ARG, "advect3d_eq_step",
                       "operators lack the even-odd symmetries")
    if flag:
        raise SdgError(ERR_MESH, "advect3d_eq_step", "a map entry is out of range")
    return arrs[0].numpy()


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


def slab_plan(NeZ: int, nparts: int):
    """(z_begin, lo_src, hi_src) of the z-slab split (sdg_slab_plan, host only)."""
    zb = np.zeros(nparts + 1, dtype=np.int32)
    lo = np.zeros(max(nparts, 1), dtype=np.int32)
    hi = np.zeros(max(nparts, 1), dtype=np.int32)
    _check(lib.sdg_slab_plan(NeZ, nparts, zb, lo, hi), "sdg_slab_plan")
    return zb, lo[:nparts], hi[:nparts]


class Slabs:
    """The box split into z-slab partitions with a face exchange per stage
    (sdg_slabs_* in include/sdg_advect.h)."""

    def __init__(self, NeX, NeY, NeZ, p, D1D, Lift_mat, nparts, opt=OPT_OPT1,
                 precision=PREC_FP64, L=(1.0, 1.0, 1.0), stream=None):
        self._h = _vp()
        self.ndof = (p + 1) ** 3 * NeX * NeY * NeZ
        _check(lib.sdg_slabs_create(C.byref(self._h), NeX, NeY, NeZ, p, float(L[0]),
                                    float(L[1]), float(L[2]), _f64(D1D), _f64(Lift_mat), opt,
                                    precision, nparts, stream), "sdg_slabs_create")

    def upload(self, q, u, v, w) -> None:
        arrs = [_f64(x) for x in (q, u, v, w)]
        _check(lib.sdg_slabs_upload(self._h, *[x.ctypes.data for x in arrs]), "sdg_slabs_upload")

    def step(self, dt: float, nstep: int) -> None:
        _check(lib.sdg_slabs_step(self._h, float(dt), int(nstep)), "sdg_slabs_step")

    def download(self) -> np.ndarray:
        out = np.zeros(self.ndof)
        _check(lib.sdg_slabs_download(self._h, out.ctypes.data), "sdg_slabs_download")
        return out

    def exchange_bytes(self) -> int:
        return int(lib.sdg_slabs_exchange_bytes(self._h))

    def close(self) -> None:
        if self._h is not None and self._h.value:
            lib.sdg_slabs_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
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

    def solve_host_pipelined(self, q_in, u, v, w, q_out, dt: float, nstep: int) -> None:
        """Pipelined host-to-host solves; each argument is a list of host
        pointers (e.g. PinnedArray.ptr) of Np*Ne doubles, one per request."""
        n = len(q_in)
        arr = [(_vp * n)(*lst) for lst in (q_in, u, v, w, q_out)]
        _check(lib.sdg_solver_solve_host_pipelined(
            self._h, n, *[C.cast(a, C.POINTER(_vp)) for a in arr], float(dt), int(nstep)),
            "sdg_solver_solve_host_pipelined")

    def minmax(self):
        """(min, max) of the current state (main.f90:76-79)."""
        lo, hi = C.c_double(), C.c_double()
        _check(lib.sdg_solver_minmax(self._h, C.byref(lo), C.byref(hi)), "sdg_solver_minmax")
        return lo.value, hi.value

    def run(self, dt: float, nstep: int, output_interval: int) -> np.ndarray:
        """The reference's time loop with its min/max output: returns an
        (nstep // output_interval, 2) array of (min, max) records."""
        nout = nstep // output_interval if output_interval > 0 else 0
        rec = np.zeros(2 * max(nout, 1))
        _check(lib.sdg_solver_run(self._h, float(dt), int(nstep), int(output_interval),
                                  rec.ctypes.data), "sdg_solver_run")
        return rec[: 2 * nout].reshape(-1, 2)

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


class Ensemble:
    """Independent boxes advanced together, one launch per order and
    RK stage (sdg_ensemble_* in include/sdg_advect.h); FP32 compute, FP64
    state."""

    def __init__(self, dims, orders, dt, ops_by_order, stream=None):
        """dims: list of (NeX,NeY,NeZ); orders: list of p; dt: list;
        ops_by_order: {p: (x1D, D1D, D1D_tr, Lift)}."""
        n = len(orders)
        self.n = n
        self.orders = [int(p) for p in orders]
        self.dims = [tuple(int(x) for x in d) for d in dims]
        self._keep = ops_by_order
        arrs = {p: [np.ascontiguousarray(a, dtype=np.float64) for a in v]
                for p, v in ops_by_order.items()}
        self._arrs = arrs
        Dp = (_vp * 16)()
        Lp = (_vp * 16)()
        Xp = (_vp * 16)()
        for p, (x, D, Dt, L) in arrs.items():
            Dp[p] = D.ctypes.data
            Lp[p] = L.ctypes.data
            Xp[p] = x.ctypes.data
        self._h = _vp()
        _check(lib.sdg_ensemble_create(C.byref(self._h), n,
                                       np.ascontiguousarray(np.array(dims, dtype=np.int32).reshape(-1)),
                                       np.ascontiguousarray(np.array(orders, dtype=np.int32)),
                                       np.ascontiguousarray(np.array(dt, dtype=np.float64)),
                                       C.cast(Dp, C.POINTER(_vp)), C.cast(Lp, C.POINTER(_vp)),
                                       C.cast(Xp, C.POINTER(_vp)), stream),
               "sdg_ensemble_create")

    def ndof(self, i) -> int:
        nx, ny, nz = self.dims[i]
        return (self.orders[i] + 1) ** 3 * nx * ny * nz

    def upload(self, i, q, u, v, w) -> None:
        _check(lib.sdg_ensemble_upload(self._h, i, _f64(q), _f64(u), _f64(v), _f64(w)),
               "sdg_ensemble_upload")

    def init_blob(self, i, centre, sigma, velocity) -> None:
        _check(lib.sdg_ensemble_init_blob(self._h, i, _f64(centre), float(sigma),
                                          _f64(velocity)), "sdg_ensemble_init_blob")

    def tune(self) -> dict:
        _check(lib.sdg_ensemble_tune(self._h), "sdg_ensemble_tune")
        return self.config()

    def set_epb(self, p, epb) -> None:
        _check(lib.sdg_ensemble_set_epb(self._h, p, epb), "sdg_ensemble_set_epb")

    def set_threads(self, threads, p=None) -> None:
        """Block size of every order, or of order p alone."""
        if p is None:
            _check(lib.sdg_ensemble_set_threads(self._h, threads), "sdg_ensemble_set_threads")
        else:
            _check(lib.sdg_ensemble_set_order_threads(self._h, p, threads),
                   "sdg_ensemble_set_order_threads")

    def set_parallel_groups(self, on: bool) -> None:
        """Order groups on parallel graph branches (True) or one stream."""
        _check(lib.sdg_ensemble_set_parallel_groups(self._h, int(bool(on))),
               "sdg_ensemble_set_parallel_groups")

    def set_single_launch(self, on: bool) -> None:
        """One persistent launch per RK stage over every order (True), or one
        launch per order group and stage (False, the default)."""
        _check(lib.sdg_ensemble_set_single_launch(self._h, int(bool(on))),
               "sdg_ensemble_set_single_launch")

    def launches_per_step(self) -> int:
        return lib.sdg_ensemble_launches_per_step(self._h)

    def set_opt(self, opt) -> None:
        """OPT_EVENODD (default): even-odd body; OPT_GENERAL/OPT_OPT1: node body."""
        _check(lib.sdg_ensemble_set_opt(self._h, opt), "sdg_ensemble_set_opt")

    def config(self) -> dict:
        epb = np.zeros(12, dtype=np.int32)
        th, gr = _i(), _i()
        _check(lib.sdg_ensemble_get_config(self._h, epb, C.byref(th), C.byref(gr)),
               "sdg_ensemble_get_config")
        eo = np.zeros(12, dtype=np.int32)
        _check(lib.sdg_ensemble_get_bodies(self._h, eo), "sdg_ensemble_get_bodies")
        tb = np.zeros(12, dtype=np.int32)
        _check(lib.sdg_ensemble_get_threads(self._h, tb), "sdg_ensemble_get_threads")
        orders = sorted(set(self.orders))
        return {"epb": {p: int(epb[p]) for p in orders},
                "body": {p: ("evenodd" if eo[p] else "node") for p in orders},
                "threads_by_order": {p: int(tb[p]) for p in orders},
                "threads": th.value, "grid": gr.value}

    def step(self, nstep: int) -> None:
        _check(lib.sdg_ensemble_step(self._h, int(nstep)), "sdg_ensemble_step")

    def step_timed(self, nstep: int) -> float:
        ms = _d()
        _check(lib.sdg_ensemble_step_timed(self._h, int(nstep), C.byref(ms)),
               "sdg_ensemble_step_timed")
        return ms.value

    def download(self, i) -> np.ndarray:
        out = np.zeros(self.ndof(i))
        _check(lib.sdg_ensemble_download(self._h, i, out), "sdg_ensemble_download")
        return out

    @property
    def total_dofs(self) -> int:
        return lib.sdg_ensemble_total_dofs(self._h)

    def close(self) -> None:
        if self._h is not None and self._h.value:
            lib.sdg_ensemble_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _order_table(ops_by_order):
    arrs = {p: [np.ascontiguousarray(a, dtype=np.float64) for a in v]
            for p, v in ops_by_order.items()}
    D, L, X = (_vp * 16)(), (_vp * 16)(), (_vp * 16)()
    for p, (x, d, dt, lift) in arrs.items():
        D[p], L[p], X[p] = d.ctypes.data, lift.ctypes.data, x.ctypes.data
    return arrs, D, L, X


class Server:
    """Continuous-batching solve server (sdg_server_* in include/sdg_advect.h)."""

    def __init__(self, ops_by_order, hbm_budget_bytes=64 << 30, max_active=512,
                 max_window_steps=8, threads=0, device=0, opt=0, threads_by_order=None,
                 epb_by_order=None, parallel_groups=False):
        """threads_by_order / epb_by_order: {p: value} overrides of the
        batched kernels' launch shape (results do not depend on it)."""
        self._arrs, D, L, X = _order_table(ops_by_order)
        cfg = ServerConfig()
        cfg.device = device
        cfg.opt = opt
        cfg.hbm_budget_bytes = int(hbm_budget_bytes)
        cfg.max_active = max_active
        cfg.max_window_steps = max_window_steps
        cfg.threads = threads
        cfg.parallel_groups = 1 if parallel_groups else 0
        for p, t in (threads_by_order or {}).items():
            cfg.threads_by_order[p] = t
        for p, e in (epb_by_order or {}).items():
            cfg.epb_by_order[p] = e
        self._h = _vp()
        _check(lib.sdg_server_create(C.byref(self._h), C.byref(cfg), C.cast(D, C.POINTER(_vp)),
                                     C.cast(L, C.POINTER(_vp)), C.cast(X, C.POINTER(_vp))),
               "sdg_server_create")
        self._outs = {}

    def submit(self, NeX, NeY, NeZ, p, nstep, dt, centre, sigma, velocity, want_state=False):
        r = Request(NeX, NeY, NeZ, p, nstep, dt, (C.c_double * 3)(*centre), sigma,
                    (C.c_double * 3)(*velocity))
        out = np.zeros((p + 1) ** 3 * NeX * NeY * NeZ) if want_state else None
        t = C.c_uint64()
        _check(lib.sdg_server_submit(self._h, C.byref(r), out.ctypes.data if out is not None
                                     else None, C.byref(t)), "sdg_server_submit")
        self._outs[t.value] = out
        return t.value

    def wait(self, ticket, timeout_s=600.0):
        """Returns (result dict, final state or None)."""
        res = Result()
        st = lib.sdg_server_wait(self._h, ticket, float(timeout_s), C.byref(res))
        out = self._outs.pop(ticket, None) if st != ERR_TIMEOUT else self._outs.get(ticket)
        _check(st, "sdg_server_wait")
        return ({"status": res.status, "latency_s": res.latency_s, "queue_s": res.queue_s,
                 "dofs": res.dofs}, out)

    def stats(self) -> dict:
        s = ServerStats()
        _check(lib.sdg_server_get_stats(self._h, C.byref(s)), "sdg_server_get_stats")
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def reset_stats(self) -> None:
        _check(lib.sdg_server_reset_stats(self._h), "sdg_server_reset_stats")

    def inject_rebuild_failure(self) -> None:
        """Host-side fault injection: the next table rebuild after a request
        completes reports an allocation failure (no device fault)."""
        _check(lib.sdg_server_inject_rebuild_failure(self._h),
               "sdg_server_inject_rebuild_failure")

    def close(self) -> None:
        if self._h is not None and self._h.value:
            lib.sdg_server_destroy(self._h)
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
