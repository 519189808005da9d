"""CPU tests of the oracle: pinned against the reference's operator files and
against known answers of the mathematics, and against the committed golden
fixtures.  No GPU is needed."""
import glob
import hashlib
import importlib.util
import math
import os

import numpy as np
import pytest

import oracle as O
import workloads as W
from helpers import GOLDEN, GOLDEN_CASES, Case, operators, rel_l2


def _fixture_script():
    spec = importlib.util.spec_from_file_location(
        "make_operator_data", os.path.join(GOLDEN, "make_operator_data.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


MOD = _fixture_script()
HAVE_REF = os.path.isdir(MOD.REFERENCE_OPERATOR_DIR)


def write_opfile(path, x, D, L):
    """The p*.dat layout: three records in ES format with 17 significant digits."""
    with open(path, "w") as f:
        for arr in (x, D, L):
            f.write(" ".join(f"{v: .16E}" for v in arr) + "\n")


# ---- operator data ------------------------------------------------------------

@pytest.mark.parametrize("p", range(1, 16))
def test_reference_operator_data_properties(p):
    """The reference's operators (the committed fixture of operator_data/p*.dat):
    GLL end points, D1D_tr the transpose, D1D annihilates constants."""
    x, D, Dt, L = operators(p)
    Nq = p + 1
    assert x.size == Nq and D.size == Nq * Nq and L.size == 6 * Nq ** 3
    assert x[0] == -1.0 and x[-1] == 1.0 and np.all(np.diff(x) > 0)
    assert np.array_equal(Dt.reshape(Nq, Nq), D.reshape(Nq, Nq).T)
    assert np.max(np.abs(D.reshape(Nq, Nq, order="F").sum(axis=1))) < 1e-12 * np.abs(D).max()


@pytest.mark.parametrize("p", range(1, 16))
def test_generated_operators_match_reference_files(p):
    """The product's GLL operator generator reproduces operator_data/p*.dat."""
    x, D, Dt, L = operators(p, "file")
    gx, gD, gDt, gL = operators(p, "generated")
    assert np.max(np.abs(gx - x)) <= 4e-16
    assert np.max(np.abs(gD - D)) <= 2e-14 * np.abs(D).max()
    assert np.max(np.abs(gL - L)) <= 5e-14 * np.abs(L).max()


@pytest.mark.skipif(not HAVE_REF, reason="reference operator_data not mounted")
@pytest.mark.parametrize("p", range(1, 16))
def test_operator_fixture_is_the_reference_files(p):
    """tests/golden/operator_data.npz holds, bit for bit, what the oracle's
    list-directed reader gives for the reference's files, and records their
    digests."""
    path = MOD.source_path(p)
    with open(path, "rb") as f:
        assert hashlib.sha256(f.read()).hexdigest() == W.operator_source_digest(p)
    for a, b in zip(O.read_operator_file(path, p), operators(p, "file")):
        assert np.array_equal(a, b)


@pytest.mark.skipif(not HAVE_REF, reason="reference operator_data not mounted")
@pytest.mark.parametrize("p", [1, 3, 7, 8, 15])
def test_product_reader_matches_oracle_reader_on_reference_files(p):
    import sdg
    path = MOD.source_path(p)
    a = O.read_operator_file(path, p)
    b = sdg.operator_read(path, p)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


@pytest.mark.parametrize("p", [1, 2, 7, 15])
def test_operator_file_roundtrip(tmp_path, p):
    import sdg
    x, D, Dt, L = operators(p)
    path = str(tmp_path / f"p{p}.dat")
    write_opfile(path, x, D, L)
    for rd in (O.read_operator_file, sdg.operator_read):
        rx, rD, rDt, rL = rd(path, p)
        assert np.array_equal(rx, x) and np.array_equal(rD, D) and np.array_equal(rL, L)
        assert np.array_equal(rDt, Dt)


def test_list_directed_read_forms(tmp_path):
    """Fortran list-directed input: D exponents, commas, r*c repeats, records
    spanning lines, and the unread tail of a record is skipped."""
    import sdg
    p = 1
    path = str(tmp_path / "p1.dat")
    with open(path, "w") as f:
        f.write("-1.0D0, 1.0d+00 99.0 99.0\n")          # tail 99s are skipped
        f.write("-0.5 -0.5\n 0.5,0.5\n")                 # record spans two lines
        f.write("48*2.5\n")                              # repeat count
    for rd in (O.read_operator_file, sdg.operator_read):
        x, D, Dt, L = rd(path, p)
        assert list(x) == [-1.0, 1.0]
        assert list(D) == [-0.5, -0.5, 0.5, 0.5]
        assert np.all(L == 2.5) and L.size == 48
    with open(path, "w") as f:
        f.write("-1.0 1.0\n-0.5 -0.5 0.5\n")             # short
    with pytest.raises(IOError):
        O.read_operator_file(path, p)
    with pytest.raises(sdg.SdgError) as e:
        sdg.operator_read(path, p)
    assert e.value.status == sdg.ERR_FILE
    with pytest.raises(sdg.SdgError) as e:
        sdg.operator_read(str(tmp_path / "missing.dat"), p)
    assert e.value.status == sdg.ERR_FILE


@pytest.mark.parametrize("p", [1, 4, 7, 11, 15])
def test_d1d_differentiates_polynomials_exactly(p):
    x, D, Dt, L = operators(p)
    Nq = p + 1
    Dm = D.reshape(Nq, Nq, order="F")
    for m in range(0, p + 1):
        f = x ** m
        df = m * x ** (m - 1) if m > 0 else np.zeros_like(x)
        assert np.max(np.abs(Dm @ f - df)) < 1e-11 * max(1.0, p * p)


@pytest.mark.parametrize("p", [1, 3, 6])
def test_lift_is_inverse_mass_times_face(p):
    """Lift(:,:,:,f) applied to a face field equals M^-1 (face mass) exactly:
    integrating the lifted field with GLL-exact mass gives the face integral."""
    x, D, Dt, L = operators(p)
    Nq = p + 1
    V = np.polynomial.legendre.legvander(x, p) * np.sqrt((2 * np.arange(Nq) + 1) / 2.0)
    M = np.linalg.inv(V @ V.T)
    c_minus = np.linalg.solve(M, np.eye(Nq)[:, 0])
    Lr = L.reshape(Nq, Nq, Nq, 6, order="F")
    assert np.allclose(Lr[:, :, :, 0], c_minus[None, :, None], atol=1e-12 * abs(c_minus).max())
    assert np.allclose(Lr[:, :, :, 3], c_minus[:, None, None], atol=1e-12 * abs(c_minus).max())


# ---- mesh / halo ---------------------------------------------------------------

@pytest.mark.parametrize("dims", [(3, 2, 4), (1, 2, 3), (2, 1, 1)])
def test_halo_and_vmap_follow_the_periodic_neighbour(dims):
    """After update_halo, q(VMapP) equals q at the periodic neighbour's
    opposite-face node, derived independently of mesh_setup's bookkeeping."""
    NeX, NeY, NeZ = dims
    p = 2
    x, D, Dt, L = operators(p)
    m = O.Mesh(NeX, NeY, NeZ, p, x)
    Nq, Np, Nfp = m.Nq, m.Np, m.Nfp
    q = np.zeros(Np * m.NeA)
    q[: Np * m.Ne] = np.random.default_rng(1).standard_normal(Np * m.Ne)
    m.update_halo(q)
    VP = m.VMapP.reshape(m.Ne, 6, Nq, Nq)  # (e, f, b, a)
    VM = m.VMapM.reshape(m.Ne, 6, Nq, Nq)
    opp = [2, 3, 0, 1, 5, 4]
    for e in range(m.Ne):
        ex, ey, ez = e % NeX, (e // NeX) % NeY, e // (NeX * NeY)
        for f in range(6):
            dx, dy, dz = [(0, -1, 0), (1, 0, 0), (0, 1, 0), (-1, 0, 0), (0, 0, -1), (0, 0, 1)][f]
            eP = (ex + dx) % NeX + NeX * ((ey + dy) % NeY) + NeX * NeY * ((ez + dz) % NeZ)
            for b in range(Nq):
                for a in range(Nq):
                    nodeP = VM[eP, opp[f], b, a] - 1 - eP * Np
                    assert q[VP[e, f, b, a] - 1] == q[eP * Np + nodeP]
    assert m.NhaloNode == Nfp * 2 * (NeY * NeZ + NeX * NeZ + NeX * NeY)


def test_workload_coordinates_match_mesh_setup():
    p = 3
    x, D, Dt, L = operators(p)
    m = O.Mesh(3, 2, 4, p, x)
    X, Y, Z = W.node_coords(3, 2, 4, x)
    n = m.Np * m.Ne
    assert np.array_equal(X, m.pos_en[:n])
    assert np.array_equal(Y, m.pos_en[n:2 * n])
    assert np.array_equal(Z, m.pos_en[2 * n:])
    # the reference's own sine initial condition
    q, u, v, w = O.ic_sine(m, (1.0, 0.5, 0.25))
    qs, us, vs, ws = W.sine(3, 2, 4, x, (1.0, 0.5, 0.25))
    assert np.array_equal(q[:n], qs) and np.all(u[:n] == 1.0) and np.all(w[:n] == 0.25)


# ---- known answers of the discretisation -----------------------------------

@pytest.mark.parametrize("p", [1, 4, 9])
def test_free_stream_gives_zero_tendency(p):
    c = Case(2, 3, 2, p, ic="sine")
    c.q[:] = 0.7
    for f in (c.u, c.v, c.w):
        f[:] = 0.0
    c.u[:] = 1.0
    c.v[:] = -0.5
    c.w[:] = 0.25
    dq = c.oracle_tend()
    scale = 0.7 * 1.0 * max(c.mesh.Escale) * np.abs(c.D).max()
    assert np.max(np.abs(dq)) < 1e-13 * scale


def test_tendency_converges_spectrally_to_exact_advection():
    errs = []
    for p in (3, 5, 7):
        c = Case(4, 4, 4, p, ic="sine", vel=(1.0, 0.5, 0.25))
        dq = c.oracle_tend()
        X, Y, Z = W.node_coords(4, 4, 4, c.x1D)
        t = 2 * np.pi
        ex = -(1.0 * t * np.cos(t * X) * np.sin(t * Y) * np.sin(t * Z)
               + 0.5 * t * np.sin(t * X) * np.cos(t * Y) * np.sin(t * Z)
               + 0.25 * t * np.sin(t * X) * np.sin(t * Y) * np.cos(t * Z))
        errs.append(rel_l2(dq, ex))
    assert errs[2] < 1e-5 and errs[0] > errs[1] > errs[2]


def test_reference_ci_case_returns_to_initial_state():
    """input.conf's case (p=7, 4^3, dt=1e-3, velocity 1) advects the sine by a
    distance of dt*nstep; after 0.1 the state matches the translated exact
    solution and min/max (main.f90:76-79) stay within the initial range."""
    c = Case(4, 4, 4, 7, ic="sine", vel=(1.0, 1.0, 1.0))
    c.dt = 1e-3
    q = c.oracle_run(100)
    X, Y, Z = W.node_coords(4, 4, 4, c.x1D)
    t = 2 * np.pi
    exact = np.sin(t * (X - 0.1)) * np.sin(t * (Y - 0.1)) * np.sin(t * (Z - 0.1))
    assert rel_l2(q, exact) < 1e-6
    assert q.max() <= 1.0 + 1e-6 and q.min() >= -1.0 - 1e-6


@pytest.mark.parametrize("p", [2, 7])
def test_mass_is_conserved(p):
    c = Case(3, 2, 3, p, ic="blob")
    m0 = W.mass(c.q, c.x1D, 3, 2, 3)
    q = c.oracle_run(20)
    assert abs(W.mass(q, c.x1D, 3, 2, 3) - m0) < 1e-13 * abs(m0)


@pytest.mark.parametrize("p", [8, 11, 15])
def test_general_and_opt1_orders_agree(p):
    c = Case(2, 1, 2, p, ic="blob")
    a = c.oracle_tend(O.OPT1)
    b = c.oracle_tend(O.GENERAL)
    assert rel_l2(a, b) < 1e-14
    assert not np.array_equal(a, b)  # the split sum really is a different order


@pytest.mark.parametrize("p", [3, 7])
def test_general_equals_opt1_for_low_orders(p):
    c = Case(2, 2, 2, p, ic="blob")
    assert np.array_equal(c.oracle_tend(O.OPT1), c.oracle_tend(O.GENERAL))


# ---- gradlike / divlike_var5 (the next SCALE-DG operator kernels) ----------------------

def _tensor_poly(x, a, b, c):
    """x^a y^b z^c on the element's GLL nodes, (i,j,k) column-major, and its
    three derivatives."""
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    def mono(t, m):
        return t ** m
    def dmono(t, m):
        return m * t ** (m - 1) if m > 0 else np.zeros_like(t)
    f = mono(X, a) * mono(Y, b) * mono(Z, c)
    g = (dmono(X, a) * mono(Y, b) * mono(Z, c), mono(X, a) * dmono(Y, b) * mono(Z, c),
         mono(X, a) * mono(Y, b) * dmono(Z, c))
    return f.ravel(order="F"), [d.ravel(order="F") for d in g]


@pytest.mark.parametrize("p", [1, 3, 7, 8, 12])
def test_gradlike_differentiates_tensor_polynomials(p):
    x, D, Dt, _ = operators(p)
    for a, b, c in [(p, 0, 1), (1, p, 0), (0, 2 % (p + 1), p), (p, p, p)]:
        f, g = _tensor_poly(x, a, b, c)
        out = O.gradlike(D, Dt, f, p + 1)
        for d in range(3):
            assert np.max(np.abs(out[d] - g[d])) < 1e-11 * max(1.0, p ** 3), (a, b, c, d)


@pytest.mark.parametrize("p", [2, 7, 9])
def test_gradlike_z_contracts_along_k(p):
    """The z output is sum_l f(i,j,l) D(k,l) (the template's erb:209 first term
    vec_in(i,1,k)*Mat_tr(1,j) would break this)."""
    x, D, Dt, _ = operators(p)
    Nq = p + 1
    f = np.random.default_rng(p).standard_normal(Nq ** 3)
    F = f.reshape(Nq, Nq, Nq, order="F")
    Dm = D.reshape(Nq, Nq, order="F")
    ox, oy, oz = O.gradlike(D, Dt, f, Nq)
    assert np.allclose(oz.reshape(Nq, Nq, Nq, order="F"), np.einsum("ijl,kl->ijk", F, Dm),
                       rtol=0, atol=1e-13 * np.abs(Dm).max() * Nq)
    assert np.allclose(oy.reshape(Nq, Nq, Nq, order="F"), np.einsum("ilk,jl->ijk", F, Dm),
                       rtol=0, atol=1e-13 * np.abs(Dm).max() * Nq)


@pytest.mark.parametrize("p", [3, 7])
def test_gradlike_equals_divlike_of_one_field_for_low_orders(p):
    x, D, Dt, _ = operators(p)
    f = np.random.default_rng(7 + p).standard_normal((p + 1) ** 3)
    g = O.gradlike(D, Dt, f, p + 1)
    d = O.divlike(D, Dt, f, f, f, p + 1, O.OPT1)
    for a, b in zip(g, d):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("p", [2, 7, 8, 13])
def test_divlike_var5_is_five_opt1_divlikes(p):
    x, D, Dt, _ = operators(p)
    Np = (p + 1) ** 3
    rng = np.random.default_rng(100 + p)
    fx, fy, fz = (rng.standard_normal(5 * Np) for _ in range(3))
    out = O.divlike_var5(D, Dt, fx, fy, fz, p + 1)
    for v in range(5):
        sl = slice(v * Np, (v + 1) * Np)
        ref = O.divlike(D, Dt, fx[sl], fy[sl], fz[sl], p + 1, O.OPT1)
        for a, b in zip(out, ref):
            assert np.array_equal(a[sl], b)


# ---- golden fixtures ---------------------------------------------------------------

GOLDEN_FILES = GOLDEN_CASES


def test_golden_fixtures_exist():
    assert len(GOLDEN_FILES) >= 3


@pytest.mark.parametrize("path", GOLDEN_FILES, ids=[os.path.basename(p) for p in GOLDEN_FILES])
def test_oracle_reproduces_golden_fixture(path):
    g = np.load(path)
    NeX, NeY, NeZ, p, nstep = (int(v) for v in g["dims"])
    m = O.Mesh(NeX, NeY, NeZ, p, g["x1D"])
    n = m.Np * m.Ne
    q, u, v, w = (W.with_halo(g[k], m.NeA, m.Np) for k in ("q", "u", "v", "w"))
    for f in (q, u, v, w):
        m.update_halo(f)
    Dt = g["D"].reshape(p + 1, p + 1).T.copy().reshape(-1)
    for opt, key in ((O.OPT1, "dqdt_opt1"), (O.GENERAL, "dqdt_general")):
        dq = O.cal_tend(m, q, u, v, w, g["D"], Dt, g["Lift"], opt)[:n]
        assert np.array_equal(dq, g[key])
    qq = q.copy()
    O.run(m, qq, u, v, w, g["D"], Dt, g["Lift"], float(g["dt"]), nstep, O.OPT1)
    assert np.array_equal(qq[:n], g["q_final"])
