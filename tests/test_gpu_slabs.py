"""GPU tests of the z-slab partitions: the box split into 1-4 partitions that
exchange their face planes before every stage gives the single-box solver's
result bit for bit, for every form and uneven splits, down to one layer a
partition."""
import numpy as np
import pytest

import sdg
import workloads as W
from helpers import TOL_RUN, Case, rel_l2

pytestmark = pytest.mark.gpu

FORMS = [(sdg.OPT_OPT1, sdg.PREC_FP64), (sdg.OPT_GENERAL, sdg.PREC_FP64),
         (sdg.OPT_EVENODD, sdg.PREC_FP64), (sdg.OPT_EVENODD, sdg.PREC_FP64_EMU),
         (sdg.OPT_EVENODD, sdg.PREC_FP32), (sdg.OPT_OPT1, sdg.PREC_FP32)]


def run_both(dims, p, nparts, opt, prec, nstep, seed=W.BASE_SEED + 90):
    c = Case(*dims, p, ic="blob", seed=seed)
    n = c.nown
    ref = sdg.Solver(*dims, p, c.D, c.Lift, opt=opt, precision=prec)
    ref.upload(c.q[:n], c.u[:n], c.v[:n], c.w[:n])
    ref.step(c.dt, nstep)
    sl = sdg.Slabs(*dims, p, c.D, c.Lift, nparts, opt=opt, precision=prec)
    sl.upload(c.q[:n], c.u[:n], c.v[:n], c.w[:n])
    sl.step(c.dt, nstep)
    return c, ref.download(), sl.download(), sl


@pytest.mark.parametrize("opt,prec", FORMS)
@pytest.mark.parametrize("nparts", [1, 2, 3, 4])
def test_partitions_equal_the_single_box(opt, prec, nparts):
    c, a, b, _ = run_both((3, 2, 8), 4, nparts, opt, prec, 4)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("p,dims,nparts", [(7, (2, 3, 7), 3), (1, (4, 3, 5), 5),
                                           (2, (1, 1, 6), 4), (8, (2, 2, 3), 3)])
def test_uneven_and_single_layer_partitions(p, dims, nparts):
    for opt, prec in ((sdg.OPT_EVENODD, sdg.PREC_FP64), (sdg.OPT_OPT1, sdg.PREC_FP64)):
        c, a, b, _ = run_both(dims, p, nparts, opt, prec, 3)
        assert np.array_equal(a, b)
        if prec == sdg.PREC_FP64 and opt == sdg.OPT_OPT1:
            assert rel_l2(b, c.oracle_run(3)) <= TOL_RUN


def test_steps_compose_across_calls_and_bytes():
    c = Case(2, 2, 6, 3, ic="blob")
    n = c.nown
    sl = sdg.Slabs(2, 2, 6, 3, c.D, c.Lift, 3, opt=sdg.OPT_EVENODD)
    sl.upload(c.q[:n], c.u[:n], c.v[:n], c.w[:n])
    sl.step(c.dt, 2)
    sl.step(c.dt, 3)
    ref = sdg.Solver(2, 2, 6, 3, c.D, c.Lift, opt=sdg.OPT_EVENODD)
    ref.upload(c.q[:n], c.u[:n], c.v[:n], c.w[:n])
    ref.step(c.dt, 5)
    assert np.array_equal(sl.download(), ref.download())
    # two planes of NeX*NeY*Nq^2 doubles per partition and stage
    assert sl.exchange_bytes() == 8 * 2 * 3 * 2 * 2 * 16


def test_bad_split_is_refused():
    c = Case(2, 2, 3, 2, ic="blob")
    with pytest.raises(sdg.SdgError) as e:
        sdg.Slabs(2, 2, 3, 2, c.D, c.Lift, 4)
    assert e.value.status == sdg.ERR_INVALID_ARG


@pytest.mark.parametrize("p,dims,nparts", [(2, (3, 2, 5), 2), (2, (1, 3, 4), 3),
                                           (3, (2, 1, 5), 2), (3, (5, 3, 3), 3)])
def test_fp32_low_order_partitions(p, dims, nparts):
    """The FP32 even-odd stage at p = 2 and 3 (the warp-cooperative kernels)
    on partitions that start past element 0 of their extended box."""
    _, a, b, _ = run_both(dims, p, nparts, sdg.OPT_EVENODD, sdg.PREC_FP32, 3)
    assert np.array_equal(a, b)
