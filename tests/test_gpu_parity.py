"""GPU parity: every CUDA entry point against the CPU oracle on the same
inputs, through the C ABI.  Tolerances: relative L2 <= 1e-12 per tendency and
<= 1e-10 after nstep for the FP64 form; <= 1e-5 for the FP32-compute form."""
import ctypes as C
import glob
import os

import numpy as np
import pytest

import oracle as O
import sdg
import workloads as W
from helpers import GOLDEN, GOLDEN_CASES, TOL_FP32, TOL_RUN, TOL_TEND, Case, operators, rel_l2

pytestmark = pytest.mark.gpu


def mesh_dims(p):
    if p <= 3:
        return (4, 3, 5)
    if p <= 7:
        return (3, 2, 4)
    return (2, 2, 3)


def solver_for(c: Case, opt=sdg.OPT_OPT1, prec=sdg.PREC_FP64):
    s = sdg.Solver(c.NeX, c.NeY, c.NeZ, c.p, c.D, c.Lift, opt=opt, precision=prec)
    n = c.nown
    s.upload(c.q[:n], c.u[:n], c.v[:n], c.w[:n])
    return s


@pytest.mark.parametrize("p", range(1, 16))
@pytest.mark.parametrize("opt", [sdg.OPT_OPT1, sdg.OPT_GENERAL, sdg.OPT_EVENODD])
def test_fused_stage_tendency_matches_oracle(p, opt):
    c = Case(*mesh_dims(p), p, ic="blob")
    s = solver_for(c, opt)
    dq = s.tendency()
    ref = c.oracle_tend(sdg.OPT_GENERAL if opt == sdg.OPT_GENERAL else sdg.OPT_OPT1)
    assert rel_l2(dq, ref) <= TOL_TEND


OP_SOURCES = ["file", "generated"]


@pytest.mark.parametrize("p", [1, 3, 7, 8, 15])
@pytest.mark.parametrize("source", OP_SOURCES)
@pytest.mark.parametrize("opt,prec", [(sdg.OPT_OPT1, sdg.PREC_FP64),
                                      (sdg.OPT_GENERAL, sdg.PREC_FP64),
                                      (sdg.OPT_EVENODD, sdg.PREC_FP64),
                                      (sdg.OPT_OPT1, sdg.PREC_FP64_EMU),
                                      (sdg.OPT_EVENODD, sdg.PREC_FP64_EMU)])
def test_fp64_forms_on_both_operator_sources(p, source, opt, prec):
    """Every FP64-state form (the fused stage in OPT1, GENERAL and even-odd
    order, the emulated stage in line and even-odd form) against the oracle,
    on the reference's own operator_data/p{p}.dat and on the generator's
    operators: <= 1e-12 per tendency and <= 1e-10 after nstep."""
    c = Case(*mesh_dims(p), p, ic="blob", ops=operators(p, source))
    oopt = O.GENERAL if opt == sdg.OPT_GENERAL else O.OPT1
    s = solver_for(c, opt=opt, prec=prec)
    assert rel_l2(s.tendency(), c.oracle_tend(oopt)) <= TOL_TEND
    nstep = 6 if p < 15 else 3
    s.step(c.dt, nstep)
    assert rel_l2(s.download(), c.oracle_run(nstep, oopt)) <= TOL_RUN


@pytest.mark.parametrize("p", [1, 3, 7, 8, 15])
@pytest.mark.parametrize("source", OP_SOURCES)
@pytest.mark.parametrize("opt", ["OPT1", "GENERAL", "EVENODD"])
def test_dropin_cal_tend_on_both_operator_sources(p, source, opt):
    """The reference-shaped cal_tend (VMap gathers, the caller's geometry) on
    the reference's operator files and on the generator's operators."""
    c = Case(*mesh_dims(p), p, ic="blob", ops=operators(p, source))
    m = c.mesh
    sdg.dg_optr_kernel_setup(opt)
    try:
        dqdt = np.full(m.Np * m.NeA, 7.0)
        sdg.advect3d_eq_cal_tend(dqdt, c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, m.VMapM, m.VMapP,
                                 m.normal_fn, m.Escale, m.Fscale, m.Nq, m.Np, m.NfpTot, m.Ne,
                                 m.NeA)
    finally:
        sdg.dg_optr_kernel_setup("OPT1")
    ref = c.oracle_tend(O.GENERAL if opt == "GENERAL" else O.OPT1)
    assert rel_l2(dqdt[: c.nown], ref) <= TOL_TEND
    assert np.all(dqdt[c.nown:] == 7.0)


@pytest.mark.parametrize("p", [1, 4, 7, 12])
@pytest.mark.parametrize("opt,prec,tol", [(sdg.OPT_OPT1, sdg.PREC_FP64, TOL_TEND),
                                          (sdg.OPT_GENERAL, sdg.PREC_FP64, TOL_TEND),
                                          (sdg.OPT_EVENODD, sdg.PREC_FP64, TOL_TEND),
                                          (sdg.OPT_OPT1, sdg.PREC_FP64_EMU, TOL_TEND),
                                          (sdg.OPT_EVENODD, sdg.PREC_FP64_EMU, TOL_TEND),
                                          (sdg.OPT_OPT1, sdg.PREC_FP32, TOL_FP32),
                                          (sdg.OPT_EVENODD, sdg.PREC_FP32, TOL_FP32)])
def test_single_element_box_is_its_own_neighbour(p, opt, prec, tol):
    """NeX = NeY = NeZ = 1: every face of the element meets its own opposite
    face through the periodic wrap."""
    c = Case(1, 1, 1, p, ic="blob")
    s = solver_for(c, opt=opt, prec=prec)
    ref = c.oracle_tend(sdg.OPT_GENERAL if opt == sdg.OPT_GENERAL else sdg.OPT_OPT1)
    # at p = 1 the exact tendency of this box is zero (all nodes coincide) and
    # the oracle's is rounding noise: measure the error against the size of
    # the terms then, against the tendency otherwise
    den = np.linalg.norm(ref)
    if den < 1e-6 * c.term_scale():
        den = c.term_scale()
    assert np.linalg.norm(s.tendency() - ref) / den <= tol
    s.step(c.dt, 3)
    assert rel_l2(s.download(), c.oracle_run(3)) <= (TOL_RUN if tol == TOL_TEND else tol)


@pytest.mark.parametrize("p", [1, 2, 5, 7, 8, 15])
def test_evenodd_tendency_sine_and_anisotropic_box(p):
    """Even-odd stage: per-direction Escale / Fscale folding on a box with
    three different element sizes, and the sine initial state."""
    c = Case(*mesh_dims(p), p, ic="sine")
    assert rel_l2(solver_for(c, sdg.OPT_EVENODD).tendency(), c.oracle_tend()) <= TOL_TEND
    L = (1.0, 2.5, 0.4)
    m = O.Mesh(c.NeX, c.NeY, c.NeZ, p, c.x1D, L=L)
    ref = O.cal_tend(m, c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, O.OPT1)[: c.nown]
    s = sdg.Solver(c.NeX, c.NeY, c.NeZ, p, c.D, c.Lift, L=L, opt=sdg.OPT_EVENODD)
    n = c.nown
    s.upload(c.q[:n], c.u[:n], c.v[:n], c.w[:n])
    assert rel_l2(s.tendency(), ref) <= TOL_TEND


@pytest.mark.parametrize("p,dims,nstep", [(3, (8, 8, 8), 100), (7, (4, 3, 2), 20),
                                          (10, (2, 2, 2), 5), (1, (1, 2, 3), 30),
                                          (2, (3, 1, 2), 10)])
def test_evenodd_run_matches_oracle(p, dims, nstep):
    c = Case(*dims, p, ic="blob")
    s = solver_for(c, sdg.OPT_EVENODD)
    s.step(c.dt, nstep)
    assert rel_l2(s.download(), c.oracle_run(nstep)) <= TOL_RUN


def test_evenodd_refuses_operators_without_centro_symmetry():
    x, D, Dt, L = operators(4)
    bad = D.copy()
    bad[3] *= 1.0 + 1e-9
    with pytest.raises(sdg.SdgError) as e:
        sdg.Solver(2, 2, 2, 4, bad, L, opt=sdg.OPT_EVENODD)
    assert e.value.status == sdg.ERR_INVALID_ARG
    badL = L.copy()
    badL[7] *= 1.0 + 1e-9
    with pytest.raises(sdg.SdgError):
        sdg.Solver(2, 2, 2, 4, D, badL, opt=sdg.OPT_EVENODD)
    # the node bodies take any operator
    sdg.Solver(2, 2, 2, 4, bad, badL, opt=sdg.OPT_OPT1)


@pytest.mark.parametrize("p", range(1, 16))
@pytest.mark.parametrize("ic", ["blob", "sine"])
@pytest.mark.parametrize("opt", [sdg.OPT_OPT1, sdg.OPT_EVENODD])
def test_emulated_fp64_tendency_matches_oracle(p, ic, opt):
    """Double-float arithmetic on the FP32 pipes meets the FP64 tolerance, in
    the line body and in the even-odd body."""
    c = Case(*mesh_dims(p), p, ic=ic)
    s = solver_for(c, opt=opt, prec=sdg.PREC_FP64_EMU)
    assert rel_l2(s.tendency(), c.oracle_tend()) <= TOL_TEND


@pytest.mark.parametrize("p,dims,nstep,ic", [
    (3, (8, 8, 8), 100, "sine"),      # the reference-sized CPU case
    (7, (4, 3, 2), 20, "blob"),
    (10, (2, 2, 2), 5, "blob"),
    (1, (1, 2, 3), 30, "blob"),       # elements that are their own x-neighbour
])
@pytest.mark.parametrize("prec,opt", [(sdg.PREC_FP64, sdg.OPT_OPT1),
                                      (sdg.PREC_FP64_EMU, sdg.OPT_OPT1),
                                      (sdg.PREC_FP64_EMU, sdg.OPT_EVENODD)])
def test_solver_run_matches_oracle(p, dims, nstep, ic, prec, opt):
    c = Case(*dims, p, ic=ic)
    s = solver_for(c, opt=opt, prec=prec)
    s.step(c.dt, nstep)
    q = s.download()
    assert rel_l2(q, c.oracle_run(nstep)) <= TOL_RUN


@pytest.mark.parametrize("p", range(1, 16))
def test_fp32_evenodd_tendency(p):
    c = Case(*mesh_dims(p), p, ic="blob")
    dq = solver_for(c, opt=sdg.OPT_EVENODD, prec=sdg.PREC_FP32).tendency()
    assert rel_l2(dq, c.oracle_tend()) <= TOL_FP32


@pytest.mark.parametrize("p", [1, 2, 3, 5, 7, 11, 12, 13, 14])
def test_fp32_evenodd_steps(p):
    """The RK stages of the FP32 even-odd kernels (each order's own shape:
    an element a thread, the warp forms, one or two threads a line, blocks
    sized to an element) against the FP64 oracle's steps."""
    c = Case(*mesh_dims(p), p, ic="blob")
    s = solver_for(c, opt=sdg.OPT_EVENODD, prec=sdg.PREC_FP32)
    s.step(c.dt, 3)
    assert rel_l2(s.download(), c.oracle_run(3)) <= TOL_FP32


@pytest.mark.parametrize("prec,opt", [(sdg.PREC_FP64, sdg.OPT_OPT1),
                                      (sdg.PREC_FP64, sdg.OPT_EVENODD),
                                      (sdg.PREC_FP32, sdg.OPT_OPT1),
                                      (sdg.PREC_FP32, sdg.OPT_EVENODD),
                                      (sdg.PREC_FP64_EMU, sdg.OPT_OPT1),
                                      (sdg.PREC_FP64_EMU, sdg.OPT_EVENODD)])
@pytest.mark.parametrize("nstep", [1, 2, 3])
def test_pipelined_host_solves_equal_plain_solves(prec, opt, nstep):
    """Every result buffer (nstep % 3) and so every wait pattern of the
    two-slot pipeline; boxes large enough that copies overlap compute."""
    dims, p = (12, 10, 8), 5
    cases = [Case(*dims, p, ic="blob", seed=W.BASE_SEED + 60 + r) for r in range(5)]
    n = cases[0].nown
    pins = [[sdg.PinnedArray(n) for _ in range(5)] for _ in cases]
    for c, pa in zip(cases, pins):
        for arr, src in zip(pa[:4], (c.q, c.u, c.v, c.w)):
            arr.array[:] = src[:n]
    s = solver_for(cases[0], opt=opt, prec=prec)
    s.solve_host_pipelined([pa[0].ptr for pa in pins], [pa[1].ptr for pa in pins],
                           [pa[2].ptr for pa in pins], [pa[3].ptr for pa in pins],
                           [pa[4].ptr for pa in pins], cases[0].dt, nstep)
    for c, pa in zip(cases, pins):
        ref = solver_for(c, opt=opt, prec=prec)
        ref.step(cases[0].dt, nstep)
        assert np.array_equal(pa[4].array, ref.download())


@pytest.mark.parametrize("p", [5, 7, 11])
@pytest.mark.parametrize("prec", [sdg.PREC_FP64, sdg.PREC_FP64_EMU])
def test_evenodd_steps_follow_a_new_velocity(p, prec):
    """The even-odd stages form the face-flux velocity factors in a step's
    first stage and reuse them in its other two: a velocity uploaded between
    steps must be the one the next step uses.  Checked against the node body
    (which forms them in every stage) through a run whose velocity changes
    sign and direction twice."""
    c = Case(*mesh_dims(p), p, ic="blob")
    n = c.nown
    rng = np.random.default_rng(W.BASE_SEED + 70 + p)
    vels = [(c.u[:n], c.v[:n], c.w[:n]),
            (-0.5 * c.v[:n], 2.0 * c.w[:n], -c.u[:n]),
            tuple(rng.uniform(-0.25, 0.25, n) for _ in range(3))]
    out = []
    for opt in (sdg.OPT_EVENODD, sdg.OPT_OPT1):
        s = sdg.Solver(c.NeX, c.NeY, c.NeZ, p, c.D, c.Lift, opt=opt, precision=prec)
        q = c.q[:n].copy()
        for u, v, w in vels:
            s.upload(q, u, v, w)
            s.step(c.dt, 4)
            q = s.download()
        out.append(q)
    assert rel_l2(out[0], out[1]) <= TOL_RUN


def test_solver_steps_compose():
    c = Case(3, 3, 2, 4, ic="blob")
    a = solver_for(c)
    a.step(c.dt, 6)
    b = solver_for(c)
    for _ in range(3):
        b.step(c.dt, 2)
    assert np.array_equal(a.download(), b.download())


@pytest.mark.parametrize("p", [1, 3, 7, 8, 12])
@pytest.mark.parametrize("opt", ["OPT1", "GENERAL"])
def test_dropin_cal_tend_matches_oracle(p, opt):
    c = Case(*mesh_dims(p), p, ic="blob")
    m = c.mesh
    sdg.dg_optr_kernel_setup(opt)
    dqdt = np.full(m.Np * m.NeA, 7.0)
    sdg.advect3d_eq_cal_tend(dqdt, c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, m.VMapM, m.VMapP,
                             m.normal_fn, m.Escale, m.Fscale, m.Nq, m.Np, m.NfpTot, m.Ne, m.NeA)
    ref = c.oracle_tend(O.OPT1 if opt == "OPT1" else O.GENERAL)
    assert rel_l2(dqdt[: c.nown], ref) <= TOL_TEND
    assert np.all(dqdt[c.nown:] == 7.0)  # only dqdt(:,1:Ne) is written


@pytest.mark.parametrize("p", range(1, 16))
def test_dropin_evenodd_cal_tend_matches_oracle(p):
    """The even-odd tendency kernel behind the reference's cal_tend signature
    (VMap gathers, the caller's flux, per-node Escale)."""
    c = Case(*mesh_dims(p), p, ic="blob")
    m = c.mesh
    sdg.dg_optr_kernel_setup("EVENODD")
    dqdt = np.full(m.Np * m.NeA, 7.0)
    sdg.advect3d_eq_cal_tend(dqdt, c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, m.VMapM, m.VMapP,
                             m.normal_fn, m.Escale, m.Fscale, m.Nq, m.Np, m.NfpTot, m.Ne, m.NeA)
    sdg.dg_optr_kernel_setup("OPT1")
    assert rel_l2(dqdt[: c.nown], c.oracle_tend(O.OPT1)) <= TOL_TEND
    assert np.all(dqdt[c.nown:] == 7.0)


@pytest.mark.parametrize("p", [2, 7, 10])
def test_dropin_evenodd_honours_per_node_escale(p):
    """Escale that varies node by node (not a constant per element and axis):
    the even-odd kernel applies it after the line sums, like the reference."""
    import copy
    c = Case(*mesh_dims(p), p, ic="blob")
    m = copy.copy(c.mesh)
    rng = np.random.default_rng(900 + p)
    m.Escale = c.mesh.Escale * (1.0 + 0.3 * rng.random(c.mesh.Escale.size))
    sdg.dg_optr_kernel_setup("EVENODD")
    dqdt = np.zeros(m.Np * m.NeA)
    sdg.advect3d_eq_cal_tend(dqdt, c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, m.VMapM, m.VMapP,
                             m.normal_fn, m.Escale, m.Fscale, m.Nq, m.Np, m.NfpTot, m.Ne, m.NeA)
    sdg.dg_optr_kernel_setup("OPT1")
    ref = O.cal_tend(m, c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, O.OPT1)[: c.nown]
    assert rel_l2(dqdt[: c.nown], ref) <= TOL_TEND


@pytest.mark.parametrize("opt", ["OPT1", "EVENODD"])
def test_dropin_flux_with_oblique_normals(opt):
    """Normals off the axes (the general u.n branch of the face flux) and
    axis-aligned ones mixed in one mesh."""
    import copy
    c = Case(3, 2, 2, 4, ic="blob")
    m = copy.copy(c.mesh)
    nt = m.NfpTot * m.Ne
    nf = c.mesh.normal_fn.copy().reshape(3, nt)
    rng = np.random.default_rng(77)
    pick = rng.random(nt) < 0.5
    nf[:, pick] += 0.2 * rng.standard_normal((3, int(pick.sum())))
    m.normal_fn = nf.reshape(-1)
    sdg.dg_optr_kernel_setup(opt)
    dqdt = np.zeros(m.Np * m.NeA)
    sdg.advect3d_eq_cal_tend(dqdt, c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, m.VMapM, m.VMapP,
                             m.normal_fn, m.Escale, m.Fscale, m.Nq, m.Np, m.NfpTot, m.Ne, m.NeA)
    sdg.dg_optr_kernel_setup("OPT1")
    ref = O.cal_tend(m, c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, O.OPT1)[: c.nown]
    assert rel_l2(dqdt[: c.nown], ref) <= TOL_TEND


def test_dropin_evenodd_refuses_operators_without_the_symmetry():
    c = Case(2, 2, 2, 5, ic="blob")
    m = c.mesh
    args = (c.q, c.u, c.v, c.w)
    geo = (m.VMapM, m.VMapP, m.normal_fn, m.Escale, m.Fscale, m.Nq, m.Np, m.NfpTot, m.Ne, m.NeA)
    sdg.dg_optr_kernel_setup("EVENODD")
    try:
        badD = c.D.copy()
        badD[3] *= 1.0 + 1e-9
        with pytest.raises(sdg.SdgError) as e:
            sdg.advect3d_eq_cal_tend(np.zeros(m.Np * m.NeA), *args, badD, badD.reshape(
                m.Nq, m.Nq).T.copy().reshape(-1), c.Lift, *geo)
        assert e.value.status == sdg.ERR_INVALID_ARG
        badDt = c.Dt.copy()
        badDt[5] += 1e-6
        with pytest.raises(sdg.SdgError) as e:
            sdg.advect3d_eq_cal_tend(np.zeros(m.Np * m.NeA), *args, c.D, badDt, c.Lift, *geo)
        assert e.value.status == sdg.ERR_INVALID_ARG
        badL = c.Lift.copy()
        badL[m.Np + 9] *= 1.0 + 1e-9
        with pytest.raises(sdg.SdgError) as e:
            sdg.advect3d_eq_cal_tend(np.zeros(m.Np * m.NeA), *args, c.D, c.Dt, badL, *geo)
        assert e.value.status == sdg.ERR_INVALID_ARG
        # the device form reports the same through its flag (2)
        arrs = [sdg.DeviceArray(a) for a in (c.q, c.u, c.v, c.w, c.D, c.Dt, badL, m.VMapM,
                                             m.VMapP, m.normal_fn, m.Escale, m.Fscale)]
        out = sdg.DeviceArray(n=m.Np * m.NeA)
        flux = sdg.DeviceArray(n=m.NfpTot * m.Ne)
        err = sdg.DeviceArray(np.zeros(1, dtype=np.int32))
        assert sdg.lib.sdg_advect3d_eq_cal_tend_dev(out.ptr, *[a.ptr for a in arrs], m.Nq, m.Np,
                                                    m.NfpTot, m.Ne, m.NeA, sdg.OPT_EVENODD,
                                                    flux.ptr, err.ptr, None) == 0
        sdg.synchronize()
        assert err.numpy()[0] == 2
    finally:
        sdg.dg_optr_kernel_setup("OPT1")


@pytest.mark.parametrize("p", range(1, 16))
def test_gradlike_matches_oracle(p):
    x, D, Dt, L = operators(p)
    Nq, Np = p + 1, (p + 1) ** 3
    nel = 7
    f = np.random.default_rng(300 + p).standard_normal(Np * nel)
    got = sdg.tensorprod_gradlike_dirXYZ(D, Dt, f, Nq)
    for e in range(nel):
        ref = O.gradlike(D, Dt, f[e * Np:(e + 1) * Np], Nq)
        for d in range(3):
            assert rel_l2(got[d][e * Np:(e + 1) * Np], ref[d]) <= TOL_TEND
    # device-pointer form on the same data gives the same bits
    dev = [sdg.DeviceArray(n=Np * nel) for _ in range(3)]
    dD, dDt, df = sdg.DeviceArray(D), sdg.DeviceArray(Dt), sdg.DeviceArray(f)
    assert sdg.lib.sdg_tensorprod_gradlike_dirXYZ_dev(*[o.ptr for o in dev], dD.ptr, dDt.ptr,
                                                      df.ptr, Nq, nel, None) == 0
    for d in range(3):
        assert np.array_equal(dev[d].numpy(), got[d])


@pytest.mark.parametrize("p", [1, 6, 9, 15])
def test_single_direction_matvecs_are_gradlike_components(p):
    """matvec_dirX/Y/Z: running sums along one axis, the components of gradlike
    (the oracle's gradlike is the z-along-k form)."""
    x, D, Dt, L = operators(p)
    Nq, Np = p + 1, (p + 1) ** 3
    f = np.random.default_rng(500 + p).standard_normal(Np * 4)
    full = sdg.tensorprod_gradlike_dirXYZ(D, Dt, f, Nq)
    assert np.array_equal(sdg.element_matvec_dir(1, D, f, Nq), full[0])
    assert np.array_equal(sdg.element_matvec_dir(2, Dt, f, Nq), full[1])
    assert np.array_equal(sdg.element_matvec_dir(3, Dt, f, Nq), full[2])
    ref = O.gradlike(D, Dt, f[:Np], Nq)
    for d in range(3):
        assert rel_l2(full[d][:Np], ref[d]) <= TOL_TEND


@pytest.mark.parametrize("p", [1, 4, 7, 8, 10, 15])
def test_divlike_var5_matches_oracle(p):
    x, D, Dt, L = operators(p)
    Nq, Np = p + 1, (p + 1) ** 3
    nel = 3
    rng = np.random.default_rng(400 + p)
    fx, fy, fz = (rng.standard_normal(5 * Np * nel) for _ in range(3))
    got = sdg.tensorprod_divlike_dirXYZ_var5(D, Dt, fx, fy, fz, Nq)
    for e in range(nel):
        sl = slice(5 * Np * e, 5 * Np * (e + 1))
        ref = O.divlike_var5(D, Dt, fx[sl], fy[sl], fz[sl], Nq)
        for d in range(3):
            assert rel_l2(got[d][sl], ref[d]) <= TOL_TEND
    dev = [sdg.DeviceArray(n=5 * Np * nel) for _ in range(3)]
    ins = [sdg.DeviceArray(a) for a in (D, Dt, fx, fy, fz)]
    assert sdg.lib.sdg_tensorprod_divlike_dirXYZ_var5_dev(*[o.ptr for o in dev],
                                                          *[i.ptr for i in ins], Nq, nel,
                                                          None) == 0
    for d in range(3):
        assert np.array_equal(dev[d].numpy(), got[d])


@pytest.mark.parametrize("opt", ["OPT1", "GENERAL", "EVENODD"])
def test_dropin_single_element_box(opt):
    c = Case(1, 1, 1, 9, ic="blob")
    m = c.mesh
    sdg.dg_optr_kernel_setup(opt)
    dqdt = np.zeros(m.Np * m.NeA)
    sdg.advect3d_eq_cal_tend(dqdt, c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, m.VMapM, m.VMapP,
                             m.normal_fn, m.Escale, m.Fscale, m.Nq, m.Np, m.NfpTot, m.Ne, m.NeA)
    sdg.dg_optr_kernel_setup("OPT1")
    ref = c.oracle_tend(O.OPT1 if opt == "OPT1" else O.GENERAL)
    assert rel_l2(dqdt[: c.nown], ref) <= TOL_TEND


def test_dropin_rejects_out_of_range_vmap():
    c = Case(2, 2, 2, 2, ic="blob")
    m = c.mesh
    sdg.dg_optr_kernel_setup("OPT1")
    bad = m.VMapP.copy()
    bad[17] = m.Np * m.NeA + 1
    with pytest.raises(sdg.SdgError) as e:
        sdg.advect3d_eq_cal_tend(np.zeros(m.Np * m.NeA), c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift,
                                 m.VMapM, bad, m.normal_fn, m.Escale, m.Fscale, m.Nq, m.Np,
                                 m.NfpTot, m.Ne, m.NeA)
    assert e.value.status == sdg.ERR_MESH


@pytest.mark.parametrize("p", [1, 5, 9, 15])
def test_operator_kernels_match_oracle(p):
    sdg.dg_optr_kernel_setup("OPT1")
    x, D, Dt, L = operators(p)
    Nq, Np = p + 1, (p + 1) ** 3
    rng = np.random.default_rng(p)
    nel = 5
    fx, fy, fz = (rng.standard_normal(Np * nel) for _ in range(3))
    ox, oy, oz = sdg.tensorprod_divlike_dirXYZ(D, Dt, fx, fy, fz, Nq)
    fl = rng.standard_normal(6 * Nq * Nq * nel)
    lo = sdg.tensorprod_Lift_hexahedral(L, fl, Nq)
    for e in range(nel):
        s = slice(e * Np, (e + 1) * Np)
        rx, ry, rz = O.divlike(D, Dt, fx[s], fy[s], fz[s], Nq, O.OPT1)
        for got, ref in ((ox[s], rx), (oy[s], ry), (oz[s], rz)):
            assert np.max(np.abs(got - ref)) <= 1e-14 * np.abs(D).max() * np.abs(fx).max() * Nq
        rl = O.lift(L, fl[e * 6 * Nq * Nq:(e + 1) * 6 * Nq * Nq], Nq)
        assert np.max(np.abs(lo[s] - rl)) <= 1e-14 * np.abs(L).max() * 6 * np.abs(fl).max()


def test_dev_update_halo_and_rk_stage_match_oracle():
    c = Case(3, 2, 2, 3, ic="blob")
    m = c.mesh
    q = c.q.copy()
    q[m.Np * m.Ne:] = 0.0
    dq = sdg.DeviceArray(q)
    hm = sdg.DeviceArray(m.halo_src_map)
    assert sdg.lib.sdg_update_halo_dev(dq.ptr, hm.ptr, m.Np, m.Ne, m.NhaloNode, None) == 0
    ref = q.copy()
    m.update_halo(ref)
    assert np.array_equal(dq.numpy(), ref)
    rng = np.random.default_rng(3)
    q0 = rng.standard_normal(c.nown)
    t = rng.standard_normal(c.nown)
    for stage in (1, 2, 3):
        qq = rng.standard_normal(c.nown)
        dqq, dq0, dt_ = sdg.DeviceArray(qq), sdg.DeviceArray(q0), sdg.DeviceArray(t)
        assert sdg.lib.sdg_rk_stage_dev(dqq.ptr, dq0.ptr, dt_.ptr, m.Np, m.Ne, stage, 0.01,
                                        None) == 0
        ref = qq.copy()
        O.rk_stage(ref, q0, t, m.Np, m.Ne, stage - 1, 0.01)
        assert np.max(np.abs(dqq.numpy() - ref)) <= 4e-16 * np.abs(ref).max()


@pytest.mark.parametrize("dims,p", [((3, 2, 4), 3), ((1, 2, 3), 2), ((4, 4, 4), 7), ((2, 1, 1), 9),
                                    ((1, 1, 1), 5)])
def test_device_mesh_equals_reference_mesh(dims, p):
    x, D, Dt, L = operators(p)
    m = O.Mesh(*dims, p, x)
    outs = {"VMapM": sdg.DeviceArray(n=m.VMapM.size, dtype=np.int32),
            "VMapP": sdg.DeviceArray(n=m.VMapP.size, dtype=np.int32),
            "normal_fn": sdg.DeviceArray(n=m.normal_fn.size),
            "Escale": sdg.DeviceArray(n=m.Escale.size),
            "Fscale": sdg.DeviceArray(n=m.Fscale.size),
            "pos_en": sdg.DeviceArray(n=m.pos_en.size),
            "halo_src_map": sdg.DeviceArray(n=m.halo_src_map.size, dtype=np.int32)}
    st = sdg.lib.sdg_mesh_setup_dev(*dims, p, 1.0, 1.0, 1.0, x.ctypes.data,
                                    *[outs[k].ptr for k in ("VMapM", "VMapP", "normal_fn", "Escale",
                                                            "Fscale", "pos_en", "halo_src_map")],
                                    None)
    assert st == 0, sdg.lib.sdg_last_error()
    for k, d in outs.items():
        assert np.array_equal(d.numpy(), getattr(m, k)), k


def test_device_only_dropin_path_matches_oracle():
    """Mesh built on the device, then update_halo and cal_tend on device
    arrays: the reference's whole per-stage sequence without host arrays."""
    c = Case(3, 2, 2, 4, ic="blob")
    m = c.mesh
    vm = sdg.DeviceArray(n=m.VMapM.size, dtype=np.int32)
    vp = sdg.DeviceArray(n=m.VMapP.size, dtype=np.int32)
    nf = sdg.DeviceArray(n=m.normal_fn.size)
    es = sdg.DeviceArray(n=m.Escale.size)
    fs = sdg.DeviceArray(n=m.Fscale.size)
    hm = sdg.DeviceArray(n=m.halo_src_map.size, dtype=np.int32)
    assert sdg.lib.sdg_mesh_setup_dev(c.NeX, c.NeY, c.NeZ, c.p, 1.0, 1.0, 1.0, None, vm.ptr, vp.ptr,
                                      nf.ptr, es.ptr, fs.ptr, None, hm.ptr, None) == 0
    fields = []
    for f in (c.q, c.u, c.v, c.w):
        g = f.copy()
        g[c.nown:] = 0.0  # halos are filled on the device
        d = sdg.DeviceArray(g)
        assert sdg.lib.sdg_update_halo_dev(d.ptr, hm.ptr, m.Np, m.Ne, m.NhaloNode, None) == 0
        fields.append(d)
    ops = [sdg.DeviceArray(a) for a in (c.D, c.Dt, c.Lift)]
    out = sdg.DeviceArray(n=m.Np * m.NeA)
    flux = sdg.DeviceArray(n=m.NfpTot * m.Ne)
    err = sdg.DeviceArray(np.zeros(1, dtype=np.int32))
    st = sdg.lib.sdg_advect3d_eq_cal_tend_dev(out.ptr, *[f.ptr for f in fields],
                                              *[o.ptr for o in ops], vm.ptr, vp.ptr, nf.ptr,
                                              es.ptr, fs.ptr, m.Nq, m.Np, m.NfpTot, m.Ne, m.NeA,
                                              sdg.OPT_OPT1, flux.ptr, err.ptr, None)
    assert st == 0
    sdg.synchronize()
    assert err.numpy()[0] == 0
    assert rel_l2(out.numpy()[: c.nown], c.oracle_tend()) <= TOL_TEND


@pytest.mark.parametrize("n", [1, 2, 7, 1000, 4097, 1 << 20])
@pytest.mark.parametrize("offset", [0, 1])
def test_minmax_dev_exact(n, offset):
    rng = np.random.default_rng(n + offset)
    x = rng.standard_normal(n + offset) * 10.0 ** rng.integers(-5, 5, n + offset)
    d = sdg.DeviceArray(x)
    lo, hi = C.c_double(), C.c_double()
    # offset 1 moves the start off a 16-byte boundary (the scalar-load path)
    assert sdg.lib.sdg_minmax_dev(d.ptr + 8 * offset, n, C.byref(lo), C.byref(hi), None) == 0
    assert lo.value == x[offset:].min() and hi.value == x[offset:].max()


def test_minmax_dev_signs_and_infinities():
    x = np.array([3.0, -0.5, np.inf, -np.inf, 1e-300, -1e-300, 0.0])
    d = sdg.DeviceArray(x)
    lo, hi = C.c_double(), C.c_double()
    assert sdg.lib.sdg_minmax_dev(d.ptr, x.size, C.byref(lo), C.byref(hi), None) == 0
    assert lo.value == -np.inf and hi.value == np.inf
    assert sdg.lib.sdg_minmax_dev(d.ptr + 8 * 4, 3, C.byref(lo), C.byref(hi), None) == 0
    assert lo.value == -1e-300 and hi.value == 1e-300


@pytest.mark.parametrize("ic", ["sine", "blob"])
def test_solver_run_minmax_records(ic):
    c = Case(3, 2, 2, 3, ic=ic)
    nstep, every = 7, 2
    ref = O.run(c.mesh, c.q.copy(), c.u, c.v, c.w, c.D, c.Dt, c.Lift, c.dt, nstep, minmax=True)
    s = solver_for(c)
    rec = s.run(c.dt, nstep, every)
    assert rec.shape == (nstep // every, 2)
    want = ref[every - 1 :: every][: nstep // every]
    assert np.allclose(rec, want, rtol=1e-12, atol=1e-14 * np.abs(want).max())
    q = s.download()
    # the state after the loop is the plain stepper's, and the last record is
    # its exact min/max after step 6
    s2 = solver_for(c)
    s2.step(c.dt, 6)
    q6 = s2.download()
    assert rec[-1, 0] == q6.min() and rec[-1, 1] == q6.max()
    assert s2.minmax() == (q6.min(), q6.max())
    s2.step(c.dt, 1)
    assert np.array_equal(q, s2.download())


def test_dev_cal_tend_sets_error_flag():
    c = Case(2, 2, 1, 2, ic="blob")
    m = c.mesh
    bad = m.VMapM.copy()
    bad[0] = 0
    arrs = [sdg.DeviceArray(a) for a in (c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, bad, m.VMapP,
                                         m.normal_fn, m.Escale, m.Fscale)]
    out = sdg.DeviceArray(n=m.Np * m.NeA)
    flux = sdg.DeviceArray(n=m.NfpTot * m.Ne)
    err = sdg.DeviceArray(np.zeros(1, dtype=np.int32))
    st = sdg.lib.sdg_advect3d_eq_cal_tend_dev(out.ptr, *[a.ptr for a in arrs], m.Nq, m.Np,
                                              m.NfpTot, m.Ne, m.NeA, sdg.OPT_OPT1, flux.ptr,
                                              err.ptr, None)
    assert st == 0
    sdg.synchronize()
    assert err.numpy()[0] == 1


def test_check_mesh_accepts_reference_mesh_and_rejects_others():
    c = Case(3, 2, 2, 2, ic="blob")
    m = c.mesh
    s = solver_for(c)
    s.check_mesh(m.VMapM, m.VMapP, m.normal_fn, m.Escale, m.Fscale)
    bad = m.VMapP.copy()
    bad[5], bad[6] = bad[6], bad[5]
    with pytest.raises(sdg.SdgError) as e:
        s.check_mesh(m.VMapM, bad, m.normal_fn, m.Escale, m.Fscale)
    assert e.value.status == sdg.ERR_MESH


@pytest.mark.parametrize("p", [2, 5, 7, 11])
@pytest.mark.parametrize("opt", [sdg.OPT_OPT1, sdg.OPT_EVENODD])
def test_fp32_compute_form_error_and_mass(p, opt):
    c = Case(*mesh_dims(p), p, ic="blob")
    s = solver_for(c, opt=opt, prec=sdg.PREC_FP32)
    nstep = 10
    s.step(c.dt, nstep)
    q = s.download()
    ref = c.oracle_run(nstep)
    assert rel_l2(q, ref) <= TOL_FP32
    m0 = W.mass(c.q, c.x1D, c.NeX, c.NeY, c.NeZ)
    assert abs(W.mass(q, c.x1D, c.NeX, c.NeY, c.NeZ) - m0) <= 1e-6 * abs(m0)


GOLDEN_FILES = GOLDEN_CASES


@pytest.mark.parametrize("path", GOLDEN_FILES, ids=[os.path.basename(p) for p in GOLDEN_FILES])
def test_gpu_matches_golden_fixture(path):
    g = np.load(path)
    NeX, NeY, NeZ, p, nstep = (int(v) for v in g["dims"])
    s = sdg.Solver(NeX, NeY, NeZ, p, g["D"], g["Lift"], opt=sdg.OPT_OPT1)
    s.upload(g["q"], g["u"], g["v"], g["w"])
    assert rel_l2(s.tendency(), g["dqdt_opt1"]) <= TOL_TEND
    s.step(float(g["dt"]), nstep)
    assert rel_l2(s.download(), g["q_final"]) <= TOL_RUN
    s2 = sdg.Solver(NeX, NeY, NeZ, p, g["D"], g["Lift"], opt=sdg.OPT_GENERAL)
    s2.upload(g["q"], g["u"], g["v"], g["w"])
    assert rel_l2(s2.tendency(), g["dqdt_general"]) <= TOL_TEND
    s3 = sdg.Solver(NeX, NeY, NeZ, p, g["D"], g["Lift"], opt=sdg.OPT_EVENODD)
    s3.upload(g["q"], g["u"], g["v"], g["w"])
    assert rel_l2(s3.tendency(), g["dqdt_opt1"]) <= TOL_TEND
    s3.step(float(g["dt"]), nstep)
    assert rel_l2(s3.download(), g["q_final"]) <= TOL_RUN


# ---- full-size properties (p=7, 32^3: 16.8M DOF) -------------------------------

@pytest.fixture(scope="module")
def full_case():
    p, N = 7, 32
    x, D, Dt, L = operators(p)
    q, u, v, w = W.blob(N, N, N, x, W.BASE_SEED)
    return dict(p=p, N=N, x=x, D=D, Dt=Dt, L=L, q=q, u=u, v=v, w=w,
                dt=W.cfl_dt(N, N, N, p, u, v, w))


@pytest.mark.parametrize("prec,opt", [(sdg.PREC_FP64, sdg.OPT_OPT1),
                                      (sdg.PREC_FP64_EMU, sdg.OPT_OPT1),
                                      (sdg.PREC_FP64, sdg.OPT_EVENODD),
                                      (sdg.PREC_FP64_EMU, sdg.OPT_EVENODD)])
def test_full_size_tendency_matches_oracle(full_case, prec, opt):
    f = full_case
    N, p = f["N"], f["p"]
    s = sdg.Solver(N, N, N, p, f["D"], f["L"], opt=opt, precision=prec)
    s.upload(f["q"], f["u"], f["v"], f["w"])
    dq = s.tendency()
    m = O.Mesh(N, N, N, p, f["x"])
    arrs = [W.with_halo(a, m.NeA, m.Np) for a in (f["q"], f["u"], f["v"], f["w"])]
    for a in arrs:
        m.update_halo(a)
    ref = O.cal_tend(m, *arrs, f["D"], f["Dt"], f["L"], O.OPT1)[: m.Np * m.Ne]
    assert rel_l2(dq, ref) <= TOL_TEND


@pytest.mark.parametrize("prec,opt", [(sdg.PREC_FP64, sdg.OPT_OPT1),
                                      (sdg.PREC_FP64_EMU, sdg.OPT_OPT1),
                                      (sdg.PREC_FP64, sdg.OPT_EVENODD),
                                      (sdg.PREC_FP64_EMU, sdg.OPT_EVENODD)])
def test_full_size_mass_conservation_and_shift_invariance(full_case, prec, opt):
    f = full_case
    N, p, Np = f["N"], f["p"], (f["p"] + 1) ** 3
    s = sdg.Solver(N, N, N, p, f["D"], f["L"], opt=opt, precision=prec)
    s.upload(f["q"], f["u"], f["v"], f["w"])
    m0 = W.mass(f["q"], f["x"], N, N, N)
    s.step(f["dt"], 5)
    q = s.download()
    assert abs(W.mass(q, f["x"], N, N, N) - m0) <= 1e-12 * abs(m0)
    # shifting every input by one element along x shifts the result exactly
    def shift(a):
        return np.roll(a.reshape(N, N, N, Np), 1, axis=2).reshape(-1)
    s2 = sdg.Solver(N, N, N, p, f["D"], f["L"], opt=opt, precision=prec)
    s2.upload(shift(f["q"]), shift(f["u"]), shift(f["v"]), shift(f["w"]))
    s2.step(f["dt"], 5)
    assert np.array_equal(s2.download(), shift(q))


# ---- the time loop on the reference's arrays (sdg_advect3d_eq_step_dev) --------

def _step_args(c, m=None):
    m = m or c.mesh
    return (m.VMapM, m.VMapP, m.normal_fn, m.Escale, m.Fscale, m.halo_src_map, m.Nq, m.Np,
            m.NfpTot, m.Ne, m.NeA, m.NhaloNode)


@pytest.mark.parametrize("p", [1, 3, 7, 8, 15])
@pytest.mark.parametrize("opt", [sdg.OPT_OPT1, sdg.OPT_GENERAL, sdg.OPT_EVENODD])
def test_reference_array_step_matches_oracle(p, opt):
    """nstep steps of main.f90's loop through the reference's own arrays
    (VMapM/VMapP into halo slots, normal_fn, per-node Escale, Fscale,
    halo_src_map): the fused even-odd stage and the reference-order sequence
    against the oracle's loop, <= 1e-10 after nstep; the halo slots of the
    result hold the final state."""
    c = Case(*mesh_dims(p), p, ic="blob")
    nstep = 5 if p < 15 else 2
    q = sdg.advect3d_eq_step(c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, *_step_args(c), c.dt,
                             nstep, opt)
    ref = c.oracle_run(nstep, O.GENERAL if opt == sdg.OPT_GENERAL else O.OPT1)
    assert rel_l2(q[: c.nown], ref) <= TOL_RUN
    m = c.mesh
    assert np.array_equal(q[c.nown: c.nown + m.NhaloNode], q[m.halo_src_map - 1])


@pytest.mark.parametrize("opt", [sdg.OPT_OPT1, sdg.OPT_EVENODD])
def test_reference_array_step_honours_normals_and_escale(opt):
    """Oblique normals, per-node Escale and per-face-node Fscale that differ
    from the structured box's: the fused stage uses the caller's arrays."""
    import copy
    c = Case(3, 2, 2, 4, ic="blob")
    m = copy.copy(c.mesh)
    rng = np.random.default_rng(123)
    nt = m.NfpTot * m.Ne
    nf = c.mesh.normal_fn.copy().reshape(3, nt)
    pick = rng.random(nt) < 0.5
    nf[:, pick] += 0.2 * rng.standard_normal((3, int(pick.sum())))
    m.normal_fn = nf.reshape(-1)
    m.Escale = c.mesh.Escale * (1.0 + 0.2 * rng.random(c.mesh.Escale.size))
    m.Fscale = c.mesh.Fscale * (1.0 + 0.2 * rng.random(c.mesh.Fscale.size))
    nstep = 4
    q = sdg.advect3d_eq_step(c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, *_step_args(c, m), c.dt,
                             nstep, opt)
    qq = c.q.copy()
    O.run(m, qq, c.u, c.v, c.w, c.D, c.Dt, c.Lift, c.dt, nstep, O.OPT1)
    assert rel_l2(q[: c.nown], qq[: c.nown]) <= TOL_RUN


def test_reference_array_step_equals_per_stage_calls():
    """The fused even-odd step equals the per-stage device calls of the
    reference's loop (halo, even-odd cal_tend, RK) to rounding."""
    c = Case(4, 3, 2, 5, ic="blob")
    a = sdg.advect3d_eq_step(c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, *_step_args(c), c.dt, 3,
                             sdg.OPT_EVENODD)
    b = sdg.advect3d_eq_step(c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, *_step_args(c), c.dt, 3,
                             sdg.OPT_OPT1)
    assert rel_l2(a, b) <= TOL_RUN


def test_reference_array_step_reports_bad_maps_and_scratch():
    c = Case(2, 2, 2, 3, ic="blob")
    m = c.mesh
    bad = m.VMapP.copy()
    bad[3] = m.Np * m.NeA + 5
    import copy
    mb = copy.copy(m)
    mb.VMapP = bad
    for opt in (sdg.OPT_EVENODD, sdg.OPT_OPT1):
        with pytest.raises(sdg.SdgError) as e:
            sdg.advect3d_eq_step(c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, *_step_args(c, mb), c.dt,
                                 1, opt)
        assert e.value.status == sdg.ERR_MESH
    badmap = m.halo_src_map.copy()
    badmap[0] = 0
    mh = copy.copy(m)
    mh.halo_src_map = badmap
    with pytest.raises(sdg.SdgError) as e:
        sdg.advect3d_eq_step(c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, *_step_args(c, mh), c.dt, 1,
                             sdg.OPT_EVENODD)
    assert e.value.status == sdg.ERR_MESH
    badD = c.D.copy()
    badD[2] *= 1.0 + 1e-9
    with pytest.raises(sdg.SdgError) as e:
        sdg.advect3d_eq_step(c.q, c.u, c.v, c.w, badD, badD.reshape(m.Nq, m.Nq).T.reshape(-1),
                             c.Lift, *_step_args(c), c.dt, 1, sdg.OPT_EVENODD)
    assert e.value.status == sdg.ERR_INVALID_ARG
    # a scratch buffer below the stated size is refused before any launch
    need = sdg.lib.sdg_advect3d_eq_step_scratch_bytes(m.Nq, m.Ne)
    small = sdg.DeviceArray(n=need // 2, dtype=np.uint8)
    qd = sdg.DeviceArray(c.q)
    st = sdg.lib.sdg_advect3d_eq_step_dev(qd.ptr, *[qd.ptr] * 12, m.Nq, m.Np, m.NfpTot, m.Ne,
                                          m.NeA, m.NhaloNode, c.dt, 1, sdg.OPT_EVENODD,
                                          small.ptr, need // 2, qd.ptr, None)
    assert st == sdg.ERR_INVALID_ARG


def test_reference_array_step_mixes_folded_and_per_node_escale():
    """Elements whose Escale is one value per direction (here a different
    value for each element) run with Escale folded into their tables, the
    others node by node; both kinds side by side in one call, against the
    oracle's loop on the same arrays."""
    import copy
    c = Case(3, 2, 3, 5, ic="blob")
    m = copy.copy(c.mesh)
    rng = np.random.default_rng(321)
    Es = c.mesh.Escale.reshape(3, m.Ne, m.Np).copy()
    for e in range(m.Ne):
        if e % 2 == 0:
            Es[:, e, :] *= (1.0 + 0.05 * e)  # uniform per direction, element's own value
        else:
            Es[:, e, :] *= 1.0 + 0.2 * rng.random((3, m.Np))  # node by node
    m.Escale = Es.reshape(-1)
    for opt in (sdg.OPT_EVENODD, sdg.OPT_OPT1):
        q = sdg.advect3d_eq_step(c.q, c.u, c.v, c.w, c.D, c.Dt, c.Lift, *_step_args(c, m), c.dt,
                                 4, opt)
        qq = c.q.copy()
        O.run(m, qq, c.u, c.v, c.w, c.D, c.Dt, c.Lift, c.dt, 4, O.OPT1)
        assert rel_l2(q[: c.nown], qq[: c.nown]) <= TOL_RUN
