"""GPU test of sdg_advect3d_eq_cal_tend_noalloc, the tendency entry point
that allocates nothing (its flux scratch is a fixed device array inside the
library).  It is meant for callers that cannot allocate device memory when
they evaluate the tendency.  The test calls it through the C ABI twice in a
row, on two different meshes, and compares each result with
sdg_advect3d_eq_cal_tend_dev given caller-owned scratch.  This file is named
to be collected last."""
import ctypes as C

import numpy as np
import pytest

import sdg
from helpers import TOL_TEND, Case, rel_l2

pytestmark = pytest.mark.gpu


def _noalloc():
    f = sdg.lib.sdg_advect3d_eq_cal_tend_noalloc
    f.argtypes = [C.c_void_p] * 13 + [C.c_int] * 6 + [C.c_void_p]
    f.restype = C.c_int
    return f


def _device_inputs(c: Case, vmapm=None):
    m = c.mesh
    return [sdg.DeviceArray(a) for a in (c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift,
                                         m.VMapM if vmapm is None else vmapm, m.VMapP,
                                         m.normal_fn, m.Escale, m.Fscale)]


def _with_caller_scratch(c: Case, ins, opt=sdg.OPT_OPT1):
    m = c.mesh
    out = sdg.DeviceArray(np.zeros(m.Np * m.NeA))
    flux = sdg.DeviceArray(n=m.NfpTot * m.Ne)
    err = sdg.DeviceArray(np.zeros(1, dtype=np.int32))
    st = sdg.lib.sdg_advect3d_eq_cal_tend_dev(out.ptr, *[a.ptr for a in ins], m.Nq, m.Np,
                                              m.NfpTot, m.Ne, m.NeA, opt, flux.ptr,
                                              err.ptr, None)
    assert st == 0
    sdg.synchronize()
    assert err.numpy()[0] == 0
    return out.numpy()[: c.nown]


def _without_alloc(c: Case, ins, opt=sdg.OPT_OPT1):
    m = c.mesh
    out = sdg.DeviceArray(np.zeros(m.Np * m.NeA))
    st = _noalloc()(out.ptr, *[a.ptr for a in ins], m.Nq, m.Np, m.NfpTot, m.Ne, m.NeA,
                    opt, None)
    return st, out.numpy()[: c.nown]


def test_noalloc_matches_dev_entry_point_on_two_calls_in_a_row():
    # a larger mesh first, then a smaller one of another order: the second call
    # sees the first call's leftovers in the shared scratch array
    for dims, p in (((4, 3, 5), 3), ((2, 2, 3), 8)):
        c = Case(*dims, p, ic="blob")
        ins = _device_inputs(c)
        want = _with_caller_scratch(c, ins)
        st, got = _without_alloc(c, ins)
        assert st == 0, sdg.lib.sdg_last_error()
        assert rel_l2(got, want) <= TOL_TEND


def test_noalloc_error_flag_is_cleared_between_calls():
    c = Case(2, 2, 2, 2, ic="blob")
    bad = c.mesh.VMapM.copy()
    bad[3] = 0
    st, _ = _without_alloc(c, _device_inputs(c, bad))
    assert st == sdg.ERR_MESH
    st, got = _without_alloc(c, _device_inputs(c))
    assert st == 0
    assert rel_l2(got, c.oracle_tend()) <= TOL_TEND


def test_noalloc_rejects_sizes_beyond_its_array():
    # NfpTot*Ne = 384 * 6000 > 2^21: rejected before any device work
    p, Ne = 7, 6000
    Nq = p + 1
    d = sdg.DeviceArray(n=8)
    st = _noalloc()(*([d.ptr] * 13), Nq, Nq ** 3, 6 * Nq * Nq, Ne, Ne, sdg.OPT_OPT1, None)
    assert st == sdg.ERR_INVALID_ARG
    assert b"at most" in sdg.lib.sdg_last_error()


def test_noalloc_evenodd_matches_dev_entry_point():
    c = Case(3, 2, 4, 6, ic="blob")
    ins = _device_inputs(c)
    st, got = _without_alloc(c, ins, sdg.OPT_EVENODD)
    assert st == 0
    assert np.array_equal(got, _with_caller_scratch(c, ins, sdg.OPT_EVENODD))
    assert rel_l2(got, c.oracle_tend()) <= TOL_TEND
