"""CPU checks of the oracle against identities the reference algorithm satisfies.

The reference ships no tests, golden vectors or known-answer files, so the
oracle is pinned by these identities and by the frozen regression vectors in
tests/golden (see test_golden_cpu.py).
"""
import numpy as np
import pytest

import ib_oracle as O


def _small(**kw):
    p = dict(m=32, n=16, mgridlev=3, dt=0.01, Re=100.0, len=8.0, offsetx=2.0, offsety=2.0,
             rtol=1e-12, atol=1e-13)
    p.update(kw)
    return O.Params(**p)


@pytest.fixture(scope="module")
def orc():
    return O.IBOracle(_small(), [O.cylinder(npts=13)])


def test_dst_is_rodft00(orc):
    # myfft.F90:119 RODFT00: Y_k = 2 sum_j x_j sin(pi (j+1)(k+1)/(N+1)), both axes
    rng = np.random.default_rng(0)
    x = rng.standard_normal((orc.n - 1, orc.m - 1))
    ny, nx = x.shape
    Sx = 2 * np.sin(np.pi * np.outer(np.arange(1, nx + 1), np.arange(1, nx + 1)) / (nx + 1))
    Sy = 2 * np.sin(np.pi * np.outer(np.arange(1, ny + 1), np.arange(1, ny + 1)) / (ny + 1))
    assert np.allclose(orc.dst(x), Sy @ x @ Sx, rtol=0, atol=1e-12 * np.abs(x).sum())
    # involution: S S = 4mn I = normalize (myfft.F90:122)
    assert np.allclose(orc.dst(orc.dst(x)) / orc.normalize, x, atol=1e-13)


def _laplacian(s):
    """5-point Laplacian with zero Dirichlet boundary (the operator ctci inverts)."""
    g = np.pad(s, 1)
    return 4 * s - g[1:-1, 2:] - g[1:-1, :-2] - g[2:, 1:-1] - g[:-2, 1:-1]


def test_ctci_inverts_laplacian(orc):
    rng = np.random.default_rng(1)
    s = rng.standard_normal((orc.n - 1, orc.m - 1))
    assert np.allclose(orc.ctci(_laplacian(s)), s, atol=1e-12)


def test_ainv_is_crank_nicolson_inverse(orc):
    rng = np.random.default_rng(2)
    w = rng.standard_normal((orc.n - 1, orc.m - 1))
    c = 0.5 * orc.p.dt / (orc.delta ** 2) / orc.p.Re
    # lam1i = 1/(1 + c lam): ainv(w + c L w) = w  (myfft.F90:145, 161-173)
    assert np.allclose(orc.ainv(w + c * _laplacian(w)), w, atol=1e-12)


def test_rot_is_minus_curl_transpose(orc):
    rng = np.random.default_rng(3)
    s = rng.standard_normal((orc.n - 1, orc.m - 1))
    hx = rng.standard_normal((orc.n, orc.m + 1)); hy = rng.standard_normal((orc.n + 1, orc.m))
    qx, qy = orc.curl(s, np.zeros(orc.nbc))
    lhs = np.sum(orc.rot(hx, hy) * s)
    rhs = np.sum(hx * qx) + np.sum(hy * qy)
    assert abs(lhs + rhs) < 1e-10 * (abs(lhs) + 1) or abs(lhs - rhs) < 1e-10 * (abs(lhs) + 1)


def test_reg_regT_adjoint(orc):
    rng = np.random.default_rng(4)
    f = rng.standard_normal(orc.nf)
    qx = rng.standard_normal((orc.n, orc.m + 1)); qy = rng.standard_normal((orc.n + 1, orc.m))
    hx, hy = orc.reg(f)
    assert np.isclose(np.sum(hx * qx) + np.sum(hy * qy), f @ orc.regT(qx, qy), rtol=1e-12)


def test_delta_function_moments():
    # grid.F90:955-1003: 6-point smoothed delta (support 3 cells).  Partition of unity and
    # zero first moment hold to the precision of its single-precision literals.
    for x0 in np.linspace(0.0, 1.0, 11):
        p = np.arange(-4, 5)
        d = O.deltafnc_vec(p - x0, 0.0, 1.0)
        assert abs(d.sum() - 1.0) < 2e-6
        assert abs((d * (p - x0)).sum()) < 2e-6
    assert O.deltafnc(3.0001, 0.0, 1.0) == 0.0
    assert np.isclose(O.deltafnc(0.3, 0.0, 1.0), O.deltafnc_vec(0.3, 0.0, 1.0), rtol=1e-15)


def test_weights_sum_to_one(orc):
    assert np.allclose(orc.reg_w.sum(axis=1), 1.0, atol=5e-6)


def test_get_bc_interpolates_linear_field(orc):
    # coarse field linear in (I,J): boundary values are the linear function at fine points
    m, n = orc.m, orc.n
    I = np.arange(2, m + 1)[None, :]; J = np.arange(2, n + 1)[:, None]
    s = 0.3 * I + 0.7 * J + 0 * I * J
    ring = orc.get_bc(s.astype(float), 1.0)
    p = np.arange(m + 1)
    assert np.allclose(ring[orc.bottom:orc.bottom + m + 1], 0.3 * (m // 4 + 1 + p / 2) + 0.7 * (n // 4 + 1))
    q = np.arange(n + 1)
    assert np.allclose(ring[orc.left:orc.left + n + 1], 0.3 * (m // 4 + 1) + 0.7 * (n // 4 + 1 + q / 2))


def test_coarsify_constant_field(orc):
    w = np.full((orc.n - 1, orc.m - 1), 2.0)
    c = orc.coarsify(w, np.zeros_like(w))
    m, n = orc.m, orc.n
    centre = c[n // 4: 3 * n // 4 - 1, m // 4: 3 * m // 4 - 1]
    assert np.allclose(centre, 8.0)     # full-weighting sum of 2: 2 + 0.5*8 + 0.25*8 = 8
    assert np.count_nonzero(c) == centre.size


def test_uniform_flow_without_body_stays_irrotational():
    o = O.IBOracle(_small(), [])
    for _ in range(3):
        o.advance()
    assert max(np.abs(w).max() for w in o.omega) < 1e-12
    # the flux is the uniform frame flux: q itself stays zero
    assert max(np.abs(q).max() for q in o.qx) < 1e-12


def test_schur_operator_nearly_symmetric_positive(orc):
    # The multi-level Poisson solve couples levels with full weighting (coarsify) and
    # interpolation (get_bc), which are not exact adjoints, so E A^-1 E^T is symmetric only
    # to about 1e-3; the reference nevertheless factors its upper triangle by Cholesky
    # (variables.F90:554-562), which needs the symmetric part to be positive definite.
    nf = orc.nf
    M = np.array([orc.a_times(e, with_b=False) for e in np.eye(nf)]).T
    assert np.abs(M - M.T).max() < 1e-3 * np.abs(M).max()
    assert np.linalg.eigvalsh(0.5 * (M + M.T)).min() > 0


def test_torsional_btimes_is_rank_one():
    o = O.IBOracle(_small(len=4.0, offsetx=1.0, offsety=1.0), [O.torsional_plate(npts=9)])
    B = np.array([o.b_times(e) for e in np.eye(o.nf)]).T
    assert np.linalg.matrix_rank(B, tol=1e-9 * np.abs(B).max()) == 1
    assert np.allclose(B, B.T)


def test_gmres_matches_direct_solve(orc):
    rng = np.random.default_rng(5)
    b = rng.standard_normal(orc.nf)
    x, its, reason = orc.gmres(b, np.zeros(orc.nf), lambda v: orc.a_times(v, with_b=False))
    M = np.array([orc.a_times(e, with_b=False) for e in np.eye(orc.nf)]).T
    assert reason > 0
    assert np.allclose(M @ x, b, atol=1e-8 * np.abs(b).max())
