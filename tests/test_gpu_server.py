"""GPU tests of the continuous-batching server: a request's result is the same
alone and in a mix of requests that arrive while it runs, admission respects
the HBM budget, and waits are bounded on the host."""
import time

import numpy as np
import pytest

import sdg
import workloads as W
from helpers import TOL_FP32, Case, operators, rel_l2

pytestmark = pytest.mark.gpu

ORDERS = (2, 3, 5, 7, 11)


@pytest.fixture(scope="module")
def ops():
    return {p: operators(p) for p in ORDERS}


def req(dims, p, nstep, seed):
    prm = W.blob_params(seed, 0.1)
    vel = (0.6, -0.3, 0.2)
    dt = 0.1 * min(1.0 / d for d in dims) / ((2 * p + 1) * sum(abs(v) for v in vel))
    return dict(NeX=dims[0], NeY=dims[1], NeZ=dims[2], p=p, nstep=nstep, dt=dt,
                centre=prm["centre"], sigma=0.1, velocity=vel)


def mixed_ops(ops):
    """Order 3 with a D1D that lacks the centro-symmetry: that order runs the
    node body while the others run the even-odd body (the mixed kernel)."""
    out = dict(ops)
    x, D, Dt, L = ops[3]
    bad = D.copy()
    bad[1] *= 1.0 + 1e-9
    out[3] = (x, bad, Dt, L)
    return out


@pytest.mark.parametrize("body", ["default", "evenodd", "node", "mixed"])
def test_result_is_the_same_alone_and_in_the_mix(ops, body):
    target = req((3, 4, 2), 5, 40, 11)
    if body == "node":
        srv = sdg.Server(ops, opt=sdg.OPT_GENERAL)
    elif body == "evenodd":
        srv = sdg.Server(ops, opt=sdg.OPT_EVENODD)
    elif body == "mixed":
        srv = sdg.Server(mixed_ops(ops))
    else:
        srv = sdg.Server(ops)
    alone, _ = None, None
    t = srv.submit(**target, want_state=True)
    res, alone = srv.wait(t)
    assert res["status"] == 0
    # the same request amid others: two before it, three arriving while it runs
    others = [req((4, 2, 3), 3, 60, 21), req((2, 2, 2), 11, 30, 22), req((5, 3, 3), 2, 80, 23),
              req((3, 3, 3), 7, 25, 24), req((2, 3, 4), 5, 50, 25)]
    tickets = [srv.submit(**others[0]), srv.submit(**others[1])]
    t2 = srv.submit(**target, want_state=True)
    for o in others[2:]:
        time.sleep(0.002)
        tickets.append(srv.submit(**o))
    res2, mixed = srv.wait(t2)
    for tk in tickets:
        assert srv.wait(tk)[0]["status"] == 0
    assert res2["status"] == 0
    assert np.array_equal(alone, mixed)
    st = srv.stats()
    assert st["completed"] == 7 and st["fatal_status"] == 0
    srv.close()


def test_launch_shape_does_not_change_results(ops):
    rs = [req((3, 4, 2), 5, 12, 41), req((2, 3, 3), 2, 9, 42), req((2, 2, 3), 11, 7, 43),
          req((4, 2, 2), 7, 10, 44)]
    outs = []
    for kw in ({}, dict(threads=512), dict(parallel_groups=True),
               dict(threads_by_order={2: 128, 5: 512, 7: 256, 11: 128},
                    epb_by_order={2: 4, 5: 1, 7: 2})):
        srv = sdg.Server(ops, **kw)
        tks = [srv.submit(**r, want_state=True) for r in rs]
        outs.append([srv.wait(t)[1] for t in tks])
        assert srv.stats()["fatal_status"] == 0
        srv.close()
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            assert np.array_equal(a, b)


def test_default_body_is_the_even_odd_body(ops):
    rs = {2: req((3, 2, 2), 2, 9, 61), 5: req((2, 3, 2), 5, 9, 62)}
    got = {}
    for name, opt in (("default", 0), ("node", sdg.OPT_GENERAL), ("evenodd", sdg.OPT_EVENODD)):
        srv = sdg.Server(ops, opt=opt)
        got[name] = {p: srv.wait(srv.submit(**r, want_state=True))[1] for p, r in rs.items()}
        srv.close()
    assert np.array_equal(got["default"][2], got["evenodd"][2])
    assert np.array_equal(got["default"][5], got["evenodd"][5])
    assert not np.array_equal(got["node"][5], got["evenodd"][5])


def test_bad_server_block_size_is_rejected(ops):
    with pytest.raises(sdg.SdgError) as e:
        sdg.Server(ops, threads_by_order={5: 100})
    assert e.value.status == sdg.ERR_INVALID_ARG


@pytest.mark.parametrize("opt", [0, sdg.OPT_GENERAL])
def test_served_result_matches_fp64_oracle_within_fp32_tolerance(ops, opt):
    r = req((3, 2, 3), 3, 20, 31)
    srv = sdg.Server(ops, opt=opt)
    _, q = srv.wait(srv.submit(**r, want_state=True))
    srv.close()
    p = r["p"]
    c = Case(3, 2, 3, p, ic="blob", ops=ops[p])
    X, Y, Z = W.node_coords(3, 2, 3, ops[p][0])

    def mi(d):
        return d - np.round(d)

    cx, cy, cz = r["centre"]
    q0 = np.exp(-(mi(X - cx) ** 2 + mi(Y - cy) ** 2 + mi(Z - cz) ** 2) / (2 * 0.1 ** 2))
    n = c.nown
    c.q[:n] = q0
    c.u[:n], c.v[:n], c.w[:n] = r["velocity"]
    for f in (c.q, c.u, c.v, c.w):
        c.mesh.update_halo(f)
    c.dt = r["dt"]
    assert rel_l2(q, c.oracle_run(r["nstep"])) <= TOL_FP32


def test_admission_waits_for_memory_and_rejects_what_never_fits(ops):
    big = req((4, 4, 4), 7, 10, 41)
    nbytes = 8 ** 3 * 64 * 36
    srv = sdg.Server(ops, hbm_budget_bytes=int(nbytes * 1.5))  # one at a time
    ts = [srv.submit(**big, want_state=True) for _ in range(3)]
    outs = [srv.wait(t)[1] for t in ts]
    assert all(np.array_equal(outs[0], o) for o in outs[1:])
    huge = req((9, 9, 9), 11, 5, 42)
    with pytest.raises(sdg.SdgError) as e:
        srv.wait(srv.submit(**huge))
    assert e.value.status == sdg.ERR_OUT_OF_MEMORY
    srv.close()


def test_many_concurrent_submitters(ops):
    """200 small requests from four submitting threads while earlier ones
    run: every one completes, and a sample equals the same request alone."""
    import threading
    srv = sdg.Server(ops, max_active=64)
    rs = [req((1 + i % 3, 2, 1 + i % 2), ORDERS[i % len(ORDERS)], 5 + i % 7, 100 + i)
          for i in range(200)]
    tickets = [None] * len(rs)

    def submit(lo):
        for i in range(lo, len(rs), 4):
            tickets[i] = srv.submit(**rs[i], want_state=(i % 25 == 0))

    th = [threading.Thread(target=submit, args=(k,)) for k in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    outs = {}
    for i, tk in enumerate(tickets):
        res, q = srv.wait(tk, timeout_s=600)
        assert res["status"] == 0
        if q is not None:
            outs[i] = q
    assert srv.stats()["completed"] == 200 and srv.stats()["fatal_status"] == 0
    srv.close()
    alone = sdg.Server(ops)
    for i, q in outs.items():
        assert np.array_equal(alone.wait(alone.submit(**rs[i], want_state=True))[1], q), i
    alone.close()


def test_wait_is_bounded(ops):
    srv = sdg.Server(ops)
    t = srv.submit(**req((6, 6, 6), 11, 400, 51))
    with pytest.raises(sdg.SdgError) as e:
        srv.wait(t, timeout_s=1e-4)
    assert e.value.status == sdg.ERR_TIMEOUT
    assert srv.wait(t, timeout_s=600)[0]["status"] == 0
    srv.close()


def test_failed_rebuild_after_a_completion_fails_the_active_requests(ops):
    """Host-side fault injection: when the device tables cannot be rebuilt
    after a request completes, the other active requests (whose old tables
    point at the freed instance) end with the error, the server records it,
    and no further step runs for them.  No device fault is involved."""
    srv = sdg.Server(ops, max_window_steps=4)
    long_req = req((4, 4, 4), 3, 100000, 71)
    t_long = srv.submit(**long_req)
    deadline = time.time() + 60
    while srv.stats()["active"] < 1:
        assert time.time() < deadline
        time.sleep(0.001)
    srv.inject_rebuild_failure()
    t_short = srv.submit(**req((2, 2, 2), 3, 3, 72), want_state=True)
    res, q = srv.wait(t_short, timeout_s=120)
    assert res["status"] == 0 and q is not None and np.all(np.isfinite(q))
    with pytest.raises(sdg.SdgError) as e:
        srv.wait(t_long, timeout_s=120)
    assert e.value.status == sdg.ERR_OUT_OF_MEMORY
    st = srv.stats()
    assert st["fatal_status"] == sdg.ERR_OUT_OF_MEMORY
    assert st["active"] == 0
    steps = st["steps_run"]
    time.sleep(0.2)
    assert srv.stats()["steps_run"] == steps  # nothing is launched any more
    # the server still admits and serves new requests afterwards
    r = req((2, 3, 2), 5, 6, 73)
    res2, q2 = srv.wait(srv.submit(**r, want_state=True))
    assert res2["status"] == 0
    srv.close()
    alone = sdg.Server(ops)
    assert np.array_equal(alone.wait(alone.submit(**r, want_state=True))[1], q2)
    alone.close()
