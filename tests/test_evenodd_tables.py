"""CPU tests of the even-odd tables the EVENODD forms build on the host: with
them, the pair sums reproduce D1D applied to any line and the lift of the
line's two faces, and operators without the symmetries are refused."""
import os

import numpy as np
import pytest

import oracle as O
import sdg
from helpers import operators


def apply_tables(tab, N, F, gm, gp):
    """out(i) = sum_l D(i,l) F(l) + lift of the two faces, from the tables."""
    H, HR, odd = N // 2, (N + 1) // 2, N & 1
    E = tab[: H * H].reshape(H, H)
    O = tab[H * H: H * H + HR * H].reshape(HR, H)
    o0 = H * H + HR * H
    DM = tab[o0: o0 + odd * H]
    A = tab[o0 + odd * H: o0 + odd * H + HR]
    B = tab[o0 + odd * H + HR: o0 + odd * H + HR + H]
    S = F[:H] + F[::-1][:H]
    Dl = F[:H] - F[::-1][:H]
    gs, gd = gm + gp, gm - gp
    out = np.zeros(N)
    for i in range(H):
        e = E[i] @ S + (DM[i] * F[H] if odd else 0.0) + B[i] * gd
        o = O[i] @ Dl + A[i] * gs
        out[i] = e + o
        out[N - 1 - i] = o - e
    if odd:
        out[H] = O[H] @ Dl + A[H] * gs
    return out


def check_tables(p, D, L):
    N = p + 1
    H, HR, odd = N // 2, (N + 1) // 2, N & 1
    te = H * H + HR * H + odd * H + HR + H
    tab = sdg.evenodd_tables(N, D, L)
    Dm = D.reshape(N, N, order="F")            # D1D(i, l)
    Lm = L.reshape(N, N, N, 6, order="F")      # Lift_mat(i, j, k, f)
    rng = np.random.default_rng(700 + p)
    # the lift columns along each axis at tangential nodes (0, 0): faces 4 / 2
    # (-x / +x), 1 / 3 (-y / +y), 5 / 6 (-z / +z) of the reference's numbering
    cols = [(Lm[:, 0, 0, 3], Lm[:, 0, 0, 1]), (Lm[0, :, 0, 0], Lm[0, :, 0, 2]),
            (Lm[0, 0, :, 4], Lm[0, 0, :, 5])]
    for ax in range(3):
        t = tab[ax * te:(ax + 1) * te]
        lam_m, lam_p = cols[ax]
        for _ in range(3):
            F = rng.standard_normal(N)
            gm, gp = rng.standard_normal(2)
            want = Dm @ F + lam_m * gm + lam_p * gp
            got = apply_tables(t, N, F, gm, gp)
            scale = np.abs(Dm).sum(axis=1).max() * np.abs(F).max() + np.abs(lam_m).max()
            assert np.max(np.abs(got - want)) <= 1e-13 * scale


@pytest.mark.parametrize("p", range(1, 16))
def test_tables_reproduce_derivative_and_lift(p):
    """The reference's operator files have the symmetries to 2.4e-14 (p = 15):
    the tables build from them and reproduce their D1D and lift columns."""
    x, D, Dt, L = operators(p)
    check_tables(p, D, L)


@pytest.mark.parametrize("p", range(1, 16))
def test_tables_of_the_generated_operators(p):
    """The generator's operators have the symmetries exactly: the tables build
    from them and reproduce their D1D and lift columns."""
    x, D, Dt, L = operators(p, "generated")
    check_tables(p, D, L)


def test_tables_refuse_operators_without_the_symmetries():
    x, D, Dt, L = operators(5)
    N = 6
    bad = D.copy()
    bad[4] *= 1.0 + 1e-9
    with pytest.raises(sdg.SdgError) as e:
        sdg.evenodd_tables(N, bad, L)
    assert e.value.status == sdg.ERR_INVALID_ARG
    badL = L.copy()
    badL[N ** 3 + 7] *= 1.0 + 1e-9  # face 2, one tangential node off the column
    with pytest.raises(sdg.SdgError) as e:
        sdg.evenodd_tables(N, D, badL)
    assert e.value.status == sdg.ERR_INVALID_ARG
    with pytest.raises(sdg.SdgError) as e:
        sdg.evenodd_tables(17, np.zeros(17 * 17), np.zeros(6 * 17 ** 3))
    assert e.value.status == sdg.ERR_UNSUPPORTED_ORDER
