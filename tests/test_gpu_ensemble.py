"""GPU tests of the batched ensemble (one persistent launch per RK stage over
all instances, CUDA graph per step): every member must equal the standalone
FP32-compute solver bit for bit, stay within the FP32-form tolerance of the
FP64 oracle, and keep those results after the autotuner changes the launch
shape."""
import numpy as np
import pytest

import sdg
import workloads as W
from helpers import TOL_FP32, Case, operators, rel_l2

pytestmark = pytest.mark.gpu

MEMBERS = [((3, 2, 4), 3), ((2, 2, 2), 7), ((4, 4, 1), 1), ((1, 3, 2), 5), ((2, 1, 2), 11),
           ((3, 3, 3), 2), ((2, 2, 3), 9), ((5, 2, 2), 3)]


def build(members, seed0=100):
    ops = {p: operators(p) for _, p in members}
    fields, dts = [], []
    for i, (dims, p) in enumerate(members):
        q, u, v, w = W.blob(*dims, ops[p][0], W.BASE_SEED + seed0 + i)
        fields.append((q, u, v, w))
        dts.append(W.cfl_dt(*dims, p, u, v, w))
    ens = sdg.Ensemble([d for d, _ in members], [p for _, p in members], dts, ops)
    for i, f in enumerate(fields):
        ens.upload(i, *f)
    return ens, fields, dts, ops


def standalone(dims, p, fields, dt, ops, nstep, opt=sdg.OPT_EVENODD):
    s = sdg.Solver(*dims, p, ops[p][1], ops[p][3], opt=opt, precision=sdg.PREC_FP32)
    s.upload(*fields)
    s.step(dt, nstep)
    return s.download()


@pytest.mark.parametrize("opt", [sdg.OPT_EVENODD, sdg.OPT_GENERAL])
def test_members_equal_the_standalone_fp32_solver_bitwise(opt):
    """Even-odd body (the default) and node body (GENERAL running sums)."""
    ens, fields, dts, ops = build(MEMBERS)
    if opt != sdg.OPT_EVENODD:
        ens.set_opt(opt)
    ens.step(4)
    for i, (dims, p) in enumerate(MEMBERS):
        want = standalone(dims, p, fields[i], dts[i], ops, 4, opt)
        assert np.array_equal(ens.download(i), want), (i, dims, p)


def test_switching_the_body_mid_run_keeps_the_state():
    ens, fields, dts, ops = build(MEMBERS[:3], seed0=150)
    ens.step(2)
    ens.set_opt(sdg.OPT_GENERAL)
    ens.step(1)
    ens.set_opt(sdg.OPT_EVENODD)
    ens.step(1)
    for i, (dims, p) in enumerate(MEMBERS[:3]):
        s = sdg.Solver(*dims, p, ops[p][1], ops[p][3], opt=sdg.OPT_EVENODD,
                       precision=sdg.PREC_FP32)
        s.upload(*fields[i])
        s.step(dts[i], 2)
        q = s.download()
        g = sdg.Solver(*dims, p, ops[p][1], ops[p][3], opt=sdg.OPT_GENERAL,
                       precision=sdg.PREC_FP32)
        g.upload(q, *fields[i][1:])
        g.step(dts[i], 1)
        s.upload(g.download(), *fields[i][1:])
        s.step(dts[i], 1)
        assert np.array_equal(ens.download(i), s.download()), i


def test_members_within_fp32_tolerance_of_fp64_oracle():
    members = MEMBERS[:4]
    ens, fields, dts, ops = build(members, seed0=200)
    ens.step(10)
    for i, (dims, p) in enumerate(members):
        c = Case(*dims, p, ic="blob", seed=W.BASE_SEED + 200 + i, ops=ops[p])
        c.dt = dts[i]
        assert rel_l2(ens.download(i), c.oracle_run(10)) <= TOL_FP32


def test_autotuner_keeps_results_and_picks_valid_shapes():
    """The tuner picks a stage body per order; each member then equals the
    standalone solver running that body."""
    ens, fields, dts, ops = build(MEMBERS, seed0=300)
    assert all(b == "evenodd" for b in ens.config()["body"].values())
    cfg = ens.tune()
    assert cfg["threads"] in (0, 128, 256, 512) and cfg["grid"] > 0
    assert set(cfg["threads_by_order"].values()) <= {128, 256, 512}
    assert set(cfg["body"]) == {p for _, p in MEMBERS}
    for p, e in cfg["epb"].items():
        assert e >= 1
    ens.step(3)
    for i, (dims, p) in enumerate(MEMBERS):
        opt = sdg.OPT_EVENODD if cfg["body"][p] == "evenodd" else sdg.OPT_GENERAL
        want = standalone(dims, p, fields[i], dts[i], ops, 3, opt)
        assert np.array_equal(ens.download(i), want), (i, p, cfg["body"][p])


def test_set_opt_overrides_the_tuned_bodies_and_the_tuner_keeps_it():
    ens, fields, dts, ops = build(MEMBERS[:4], seed0=350)
    ens.tune()
    ens.set_opt(sdg.OPT_GENERAL)
    assert all(b == "node" for b in ens.config()["body"].values())
    assert all(b == "node" for b in ens.tune()["body"].values())
    ens.step(2)
    for i, (dims, p) in enumerate(MEMBERS[:4]):
        want = standalone(dims, p, fields[i], dts[i], ops, 2, sdg.OPT_GENERAL)
        assert np.array_equal(ens.download(i), want), i


def test_block_size_per_order_keeps_results():
    ens, fields, dts, ops = build(MEMBERS, seed0=450)
    ens.set_threads(512)
    ens.set_threads(128, p=7)
    ens.set_threads(256, p=3)
    cfg = ens.config()
    assert cfg["threads"] == 0
    assert cfg["threads_by_order"][7] == 128 and cfg["threads_by_order"][3] == 256
    assert cfg["threads_by_order"][11] == 512
    ens.step(3)
    for i, (dims, p) in enumerate(MEMBERS):
        want = standalone(dims, p, fields[i], dts[i], ops, 3)
        assert np.array_equal(ens.download(i), want), (i, p)


def test_parallel_group_branches_keep_results():
    ens, fields, dts, ops = build(MEMBERS, seed0=470)
    ens.set_parallel_groups(True)
    ens.step(2)
    ens.set_parallel_groups(False)
    ens.step(1)
    for i, (dims, p) in enumerate(MEMBERS):
        want = standalone(dims, p, fields[i], dts[i], ops, 3)
        assert np.array_equal(ens.download(i), want), (i, p)


def test_explicit_shapes_and_graph_replay_compose():
    ens, fields, dts, ops = build(MEMBERS[:3], seed0=400)
    ens.set_threads(128)
    ens.set_epb(3, 1)
    ens.step(2)
    ens.set_epb(3, 4)
    ens.step(3)
    for i, (dims, p) in enumerate(MEMBERS[:3]):
        want = standalone(dims, p, fields[i], dts[i], ops, 5)
        assert np.array_equal(ens.download(i), want)


def test_many_one_element_members():
    """600 single-element boxes of every order 1..11 (one element per work
    item, 600 instance headers): a sample equals the standalone solver."""
    members = [((1, 1, 1), 1 + i % 11) for i in range(600)]
    ens, fields, dts, ops = build(members, seed0=600)
    ens.tune()
    ens.step(3)
    for i in range(0, 600, 37):
        dims, p = members[i]
        opt = sdg.OPT_EVENODD if ens.config()["body"][p] == "evenodd" else sdg.OPT_GENERAL
        want = standalone(dims, p, fields[i], dts[i], ops, 3, opt)
        assert np.array_equal(ens.download(i), want), (i, p)


def test_device_initial_condition_matches_host_recipe():
    dims, p = (3, 2, 2), 4
    ops = {p: operators(p)}
    ens = sdg.Ensemble([dims], [p], [1e-3], ops)
    centre, sigma, vel = (0.3, 0.7, 0.55), 0.12, (0.4, -0.2, 0.1)
    ens.init_blob(0, centre, sigma, vel)
    X, Y, Z = W.node_coords(*dims, ops[p][0])

    def mi(d):
        return d - np.round(d)

    q = np.exp(-(mi(X - centre[0]) ** 2 + mi(Y - centre[1]) ** 2 + mi(Z - centre[2]) ** 2)
               / (2 * sigma * sigma))
    assert rel_l2(ens.download(0), q) < 1e-13


def test_bad_ensemble_arguments_are_rejected():
    ops = {3: operators(3)}
    with pytest.raises(sdg.SdgError) as e:
        sdg.Ensemble([(2, 2, 2)], [12], [1e-3], {12: operators(12)})
    assert e.value.status == sdg.ERR_UNSUPPORTED_ORDER
    with pytest.raises(sdg.SdgError) as e:
        sdg.Ensemble([(2, 0, 2)], [3], [1e-3], ops)
    assert e.value.status == sdg.ERR_INVALID_ARG


@pytest.mark.parametrize("opt", [sdg.OPT_EVENODD, sdg.OPT_GENERAL])
def test_single_launch_per_stage_equals_the_per_order_launches(opt):
    """One persistent launch per RK stage over every order (and body) gives
    the per-order launches' bits; switching it on and off mid-run keeps the
    state, and a step is then four launches."""
    ens, fields, dts, ops = build(MEMBERS, seed0=300)
    if opt != sdg.OPT_EVENODD:
        ens.set_opt(opt)
    ens.set_single_launch(True)
    assert ens.launches_per_step() == 4
    ens.step(2)
    ens.set_single_launch(False)
    ens.step(1)
    ens.set_single_launch(True)
    ens.step(1)
    for i, (dims, p) in enumerate(MEMBERS):
        want = standalone(dims, p, fields[i], dts[i], ops, 4, opt)
        assert np.array_equal(ens.download(i), want), (i, dims, p)


def test_low_order_single_box_kernels_equal_the_block_body():
    """The single-box FP32 even-odd stage runs its own kernels at p = 1..3
    (an element a thread, the column form, a warp an element); the ensemble
    runs the block body.  Element counts that fill no whole warp, boxes one
    element wide and single elements included."""
    members = [((2, 2, 2), 2), ((1, 3, 5), 2), ((4, 1, 1), 2), ((1, 1, 1), 3),
               ((3, 5, 1), 3), ((2, 2, 2), 1), ((7, 1, 2), 2), ((1, 2, 7), 3)]
    ens, fields, dts, ops = build(members, seed0=300)
    ens.step(3)
    for i, (dims, p) in enumerate(members):
        want = standalone(dims, p, fields[i], dts[i], ops, 3)
        assert np.array_equal(ens.download(i), want), (i, dims, p)


@pytest.mark.parametrize("p", [2, 3])
def test_low_order_kernels_on_a_box_past_the_32_bit_index_constants(p):
    """4096 x 16 x 16 elements: e * NeX reaches 2^32, so the single-box p = 2
    and 3 kernels find element coordinates by division instead of the 32-bit
    multiply-high constants; the result still equals the block body's."""
    members = [((4096, 16, 16), p)]
    ens, fields, dts, ops = build(members, seed0=400)
    ens.step(1)
    want = standalone(members[0][0], p, fields[0], dts[0], ops, 1)
    assert np.array_equal(ens.download(0), want)
