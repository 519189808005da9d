"""The z-slab partitioning on CPU: the plan (sdg_slab_plan, host-only
arithmetic of the C library) and the exchange protocol run as two gloo
ranks, each holding one partition of a whole-box field, packing the face
planes it sends, exchanging them with send/recv and unpacking them into its
ghost layers -- the bookkeeping the GPU partitions follow, checked against
the neighbour planes of the whole box."""
import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest

from helpers import ROOT

import sdg


def test_plan_covers_every_layer_once():
    for NeZ in range(1, 13):
        for P in range(1, NeZ + 1):
            zb, lo, hi = sdg.slab_plan(NeZ, P)
            assert zb[0] == 0 and zb[-1] == NeZ
            sizes = np.diff(zb)
            assert np.all(sizes >= 1) and sizes.max() - sizes.min() <= 1
            for k in range(P):
                assert lo[k] == (k - 1) % P and hi[k] == (k + 1) % P
                assert hi[lo[k]] == k  # the plan is symmetric


def test_plan_rejects_impossible_splits():
    for NeZ, P in ((4, 5), (4, 0), (0, 1)):
        with pytest.raises(sdg.SdgError) as e:
            sdg.slab_plan(NeZ, P)
        assert e.value.status == sdg.ERR_INVALID_ARG


# ---- the exchange as two ranks ---------------------------------------------------

def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def extend(full, NeX, NeY, NeZ, Nq, z0, nz):
    """Partition layers z0-1 .. z0+nz (periodic) of a whole-box field."""
    lay = NeX * NeY * Nq ** 3
    f = full.reshape(NeZ, lay)
    return np.concatenate([f[(z0 - 1 + l) % NeZ] for l in range(nz + 2)])


def planes(ext, NeX, NeY, Nq, layer, k):
    """The k-plane (k = 0 or Nq-1) of every element of one layer: (NeX*NeY, Nq^2)."""
    np_ = Nq ** 3
    e = ext.reshape(-1, NeX * NeY, np_)[layer]
    return e.reshape(NeX * NeY, Nq, Nq * Nq)[:, k, :].copy()


def _rank_main(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws))
    sys.path.insert(0, os.path.join(ROOT, "scale-dg-kernel-extraction_gb300"))
    import torch
    import torch.distributed as dist
    import sdg as S
    dist.init_process_group("gloo")
    NeX, NeY, NeZ, Nq = 3, 2, 5, 3
    full = np.random.default_rng(7).standard_normal(NeX * NeY * NeZ * Nq ** 3)
    zb, lo_src, hi_src = S.slab_plan(NeZ, ws)
    z0, nz = int(zb[rank]), int(zb[rank + 1] - zb[rank])
    ext = extend(full, NeX, NeY, NeZ, Nq, z0, nz)
    ghosts_before = ext.copy()
    # scramble the ghost layers: the exchange must fill what the stages read
    lay = NeX * NeY * Nq ** 3
    ext[:lay] = -1.0
    ext[(nz + 1) * lay:] = -1.0
    # pack: bottom owned layer's k = 0 plane (down), top owned layer's k = Nq-1 plane (up)
    send_lo = torch.from_numpy(planes(ext, NeX, NeY, Nq, 1, 0))
    send_hi = torch.from_numpy(planes(ext, NeX, NeY, Nq, nz, Nq - 1))
    recv_lo, recv_hi = torch.empty_like(send_lo), torch.empty_like(send_hi)
    # my lower ghost comes from lo_src's top layer, my upper one from hi_src's bottom
    ops = [dist.P2POp(dist.isend, send_hi, int(hi_src[rank])),
           dist.P2POp(dist.isend, send_lo, int(lo_src[rank])),
           dist.P2POp(dist.irecv, recv_lo, int(lo_src[rank])),
           dist.P2POp(dist.irecv, recv_hi, int(hi_src[rank]))]
    for r in dist.batch_isend_irecv(ops):
        r.wait()
    # unpack into the ghost layers' face planes
    e = ext.reshape(nz + 2, NeX * NeY, Nq, Nq * Nq)
    e[0, :, Nq - 1, :] = recv_lo.numpy()
    e[nz + 1, :, 0, :] = recv_hi.numpy()
    ok_lo = np.array_equal(planes(ext, NeX, NeY, Nq, 0, Nq - 1),
                           planes(ghosts_before, NeX, NeY, Nq, 0, Nq - 1))
    ok_hi = np.array_equal(planes(ext, NeX, NeY, Nq, nz + 1, 0),
                           planes(ghosts_before, NeX, NeY, Nq, nz + 1, 0))
    owned = np.array_equal(ext[lay:(nz + 1) * lay], full.reshape(NeZ, lay)[z0:z0 + nz].ravel())
    out.put((rank, ok_lo, ok_hi, owned))
    dist.destroy_process_group()


def test_exchange_fills_ghost_planes_across_two_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    ws, port = 2, _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, ws, port, out)) for r in range(ws)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=180) for _ in range(ws))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ok_lo, ok_hi, owned in res:
        assert ok_lo and ok_hi and owned, rank


def test_create_rejects_bad_partition_counts_before_device_work():
    from helpers import operators
    _, D, _, L = operators(2)
    for P in (0, -3, 5):
        with pytest.raises(sdg.SdgError) as e:
            sdg.Slabs(2, 2, 4, 2, D, L, P)
        assert e.value.status == sdg.ERR_INVALID_ARG
