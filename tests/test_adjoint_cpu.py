"""The oracle's discrete adjoint of the step (oracle/ib_adjoint.py) pinned by central finite
differences of the oracle's own forward, and each transpose by its dot-product identity
<A x, y> = <x, A^T y>."""
import numpy as np
import pytest

import ib_adjoint as A
import ib_oracle as O


def _oracle(L=3, num_stat=True):
    p = O.Params(m=32, n=16, mgridlev=L, dt=0.02, Re=100.0, len=4.0, offsetx=1.0, offsety=1.0, num_stat=num_stat,
                 motion=(-1.0, 0.0, 0.0, 0.3, 0.0))
    return O.IBOracle(p, [O.cylinder(npts=10, diameter=0.8, xc=0.3, yc=0.0)])


def _coefs(N):
    t = np.arange(N, dtype=np.float64)
    return np.stack([-1.0 + 0.1 * np.sin(t), 0.2 * np.cos(t), 0.3 * np.sin(0.5 * t)], 1)


def test_transposes_satisfy_the_dot_product_identity():
    o = _oracle()
    ad = A.Adjoint(o)
    rng = np.random.default_rng(0)
    m, n = o.m, o.n
    vert = lambda: rng.standard_normal((n - 1, m - 1))
    ux = lambda: rng.standard_normal((n, m + 1))
    vy = lambda: rng.standard_normal((n + 1, m))
    ring = lambda: rng.standard_normal(o.nbc)
    # rot / curl (with ring)
    hx, hy, lam = ux(), vy(), vert()
    rx, ry = ad.rot_T(lam)
    assert np.isclose(np.sum(o.rot(hx, hy) * lam), np.sum(hx * rx) + np.sum(hy * ry), rtol=1e-13)
    s, sb, lx, ly = vert(), ring(), ux(), vy()
    cx, cy = o.curl(s, sb)
    ts, tr = ad.curl_T(lx, ly)
    assert np.isclose(np.sum(cx * lx) + np.sum(cy * ly), np.sum(s * ts) + np.sum(sb * tr), rtol=1e-13)
    # get_bc, apply_bc
    r = ring()
    assert np.isclose(np.sum(o.get_bc(s, 0.25) * r), np.sum(s * ad.get_bc_T(r, 0.25)), rtol=1e-13)
    v = vert()
    av = o.apply_bc(np.zeros_like(v), r, 0.7)
    assert np.isclose(np.sum(av * v), np.sum(r * ad.apply_bc_T(v, 0.7)), rtol=1e-13)
    # coarsify (the coarse centre overwritten)
    fine, coarse, lf, lc = vert(), vert(), vert(), vert()
    out = o.coarsify(fine, coarse.copy())
    lf2, lc2 = lf * 0.0, lc.copy()
    ad.coarsify_T(lf2, lc2)
    assert np.isclose(np.sum(out * lc), np.sum(fine * lf2) + np.sum(coarse * lc2), rtol=1e-13)
    # nonlinear: linear in each argument with the others fixed
    om, qx, qy, bc = vert(), ux(), vy(), ring()
    lx, ly = ux(), vy()
    lom, lqx, lqy, lbc = ad.nonlinear_T(om, qx, qy, bc, lx, ly)
    for d_om, d_qx, d_qy, d_bc, adj in ((vert(), 0 * qx, 0 * qy, 0 * bc, "om"), (0 * om, ux(), 0 * qy, 0 * bc, "qx"),
                                         (0 * om, 0 * qx, vy(), 0 * bc, "qy"), (0 * om, 0 * qx, 0 * qy, ring(), "bc")):
        if adj in ("om", "bc"):   # linear in (omega, bc) together with q fixed
            nx, ny = o.nonlinear(d_om, qx, qy, d_bc)
        else:                     # linear in q with omega and bc fixed
            nx, ny = o.nonlinear(om, d_qx, d_qy, bc)
        lhs = np.sum(nx * lx) + np.sum(ny * ly)
        rhs = {"om": np.sum(d_om * lom), "bc": np.sum(d_bc * lbc), "qx": np.sum(d_qx * lqx),
               "qy": np.sum(d_qy * lqy)}[adj]
        assert np.isclose(lhs, rhs, rtol=1e-12), adj


@pytest.mark.parametrize("L,num_stat", [(2, True), (3, True), (3, False)])
def test_gradient_matches_central_differences(L, num_stat):
    # num_stat = F: the Schur system solved with its dense matrix, the reverse with its transpose
    N = 6
    coefs = _coefs(N)
    W = np.random.default_rng(1).standard_normal((N, 1, 2))

    def J(c):
        ad = A.Adjoint(_oracle(L, num_stat))
        return float(np.sum(W * ad.forward(c))), ad

    J0, ad = J(coefs)
    g = ad.backward(W)
    h = 1e-6
    for (n, i) in [(0, 0), (2, 1), (5, 2), (3, 0), (1, 2), (4, 1)]:
        cp = coefs.copy(); cp[n, i] += h
        cm = coefs.copy(); cm[n, i] -= h
        fd = (J(cp)[0] - J(cm)[0]) / (2 * h)
        assert abs(g[n, i] - fd) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(g).max()), (n, i, g[n, i], fd)


def test_forward_equals_the_oracle_step():
    # the adjoint's forward is IBOracle.advance with the frame flux of the coefficients
    o1, o2 = _oracle(), _oracle()
    ad = A.Adjoint(o1)
    c = np.array([-1.0, 0.0, 0.0])
    for _ in range(3):
        ad.step(c)
        o2.advance()
    for k in range(o1.L):
        assert np.allclose(o1.omega[k], o2.omega[k], rtol=0, atol=1e-13 * np.abs(o2.omega[k]).max())


def _sd_oracle(cols=None):
    import ib_subdomain as SD
    p = O.Params(m=64, n=32, mgridlev=3, dt=0.01, Re=100.0, len=4.0, offsetx=1.0, offsety=1.0, num_stat=False,
                 motion=(-1.0, 0.0, 0.0, 0.3, 0.0))
    o = O.IBOracle(p, [O.cylinder(npts=8, diameter=0.3, xc=0.1, yc=0.0)])
    o.sd = SD.SubDomain(o, True, -0.25, 0.5, -0.25, 0.25, 0.0625)
    if cols is None:
        o.sd.precompute()
    else:
        o.sd.cols = cols
    return o


def test_subdomain_gradient_matches_central_differences():
    # the sub-domain method: lumat and its transpose, P E_o and E_o^T P^T
    N = 4
    coefs = _coefs(N)
    W = np.random.default_rng(2).standard_normal((N, 1, 2))
    cols = _sd_oracle().sd.cols

    def J(c):
        ad = A.Adjoint(_sd_oracle(cols))
        return float(np.sum(W * ad.forward(c))), ad

    J0, ad = J(coefs)
    g = ad.backward(W)
    h = 1e-6
    for (n, i) in [(0, 0), (1, 2), (3, 1)]:
        cp = coefs.copy(); cp[n, i] += h
        cm = coefs.copy(); cm[n, i] -= h
        fd = (J(cp)[0] - J(cm)[0]) / (2 * h)
        assert abs(g[n, i] - fd) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(g).max()), (n, i, g[n, i], fd)
