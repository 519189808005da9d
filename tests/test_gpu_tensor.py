"""GPU tests of the tensor-core FP32 contraction (tcgen05 kind::tf32 with
TF32 pair splitting) at p = 15: the three directional derivatives of
tensorprod_divlike_dirXYZ against the FP64 oracle and against the CUDA-core
FP32 form."""
import numpy as np
import pytest

import oracle as O
import sdg
from helpers import TOL_FP32, operators, rel_l2

pytestmark = pytest.mark.gpu


def fields(nelem, Nq, seed):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal(nelem * Nq ** 3) for _ in range(3)]


@pytest.mark.parametrize("source", ["file", "generated"])
@pytest.mark.parametrize("kind", ["smooth", "random"])
def test_tensor_core_divlike_matches_fp64_oracle(source, kind):
    p, nelem = 15, 6
    Nq = p + 1
    x, D, Dt, L = operators(p, source)
    if kind == "random":
        fx, fy, fz = fields(nelem, Nq, 31)
    else:
        # smooth fields: the contraction cancels as in a real tendency
        xs = np.asarray(x)
        X, Y, Z = np.meshgrid(xs, xs, xs, indexing="ij")
        base = [np.sin(1.3 * X + 0.7 * Y) * np.cos(Z), np.exp(0.3 * X * Y * Z), X * Y + Z ** 3]
        fx, fy, fz = (np.concatenate([(b * (1 + 0.1 * e)).transpose(2, 1, 0).ravel()
                                      for e in range(nelem)]) for b in base)
    # the oracle sees the same FP32-rounded inputs, so only the contraction's
    # arithmetic is measured
    fx, fy, fz = (np.asarray(f, dtype=np.float32).astype(np.float64) for f in (fx, fy, fz))
    got = sdg.tensorprod_divlike_dirXYZ_f32(D, fx, fy, fz, Nq, tensor_cores=True)
    cuda = sdg.tensorprod_divlike_dirXYZ_f32(D, fx, fy, fz, Nq, tensor_cores=False)
    np_ = Nq ** 3
    ref = [np.zeros(nelem * np_) for _ in range(3)]
    for e in range(nelem):
        s = slice(e * np_, (e + 1) * np_)
        ox, oy, oz = O.divlike(D, Dt, fx[s], fy[s], fz[s], Nq, O.GENERAL)
        ref[0][s], ref[1][s], ref[2][s] = ox, oy, oz
    for d in range(3):
        e_tc, e_cc = rel_l2(got[d], ref[d]), rel_l2(cuda[d], ref[d])
        if kind == "random":
            assert e_tc <= TOL_FP32 and e_cc <= TOL_FP32, (d, e_tc, e_cc)
        else:
            # a derivative of a smooth field at p = 15 cancels terms hundreds
            # of times its size.  A TF32 pair holds an operand to 2^-22 and the
            # dropped lo*lo term is 2^-22 of the product, against FP32's 2^-24,
            # so the tensor-core form's error there is a few times the CUDA-core
            # FP32 form's (measured 2.8e-6 against 9.5e-7 in x): both stay
            # within 1e-4 of the FP64 oracle
            assert e_tc <= 1e-4 and e_cc <= 1e-4, (d, e_tc, e_cc)


def test_tensor_core_form_covers_every_tile_of_a_larger_batch():
    """More tiles than CTAs: every element's six tiles are written."""
    p, nelem = 15, 3000
    Nq = p + 1
    x, D, Dt, L = operators(p)
    fx, fy, fz = fields(nelem, Nq, 32)
    got = sdg.tensorprod_divlike_dirXYZ_f32(D, fx, fy, fz, Nq, tensor_cores=True)
    cuda = sdg.tensorprod_divlike_dirXYZ_f32(D, fx, fy, fz, Nq, tensor_cores=False)
    for d in range(3):
        assert np.all(np.isfinite(got[d]))
        assert rel_l2(got[d], cuda[d]) <= TOL_FP32


def test_tensor_core_form_is_refused_below_p15():
    x, D, Dt, L = operators(7)
    f = np.zeros(2 * 8 ** 3)
    with pytest.raises(sdg.SdgError) as e:
        sdg.tensorprod_divlike_dirXYZ_f32(D, f, f, f, 8, tensor_cores=True)
    assert e.value.status == sdg.ERR_UNSUPPORTED_ORDER
    # the CUDA-core form takes any order
    out = sdg.tensorprod_divlike_dirXYZ_f32(D, f, f, f, 8, tensor_cores=False)
    assert all(np.all(o == 0) for o in out)
