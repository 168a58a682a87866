"""The oracle's pressure recovery (operators_pressure.F90:110-437) against identities the
reference's algorithm satisfies: ddti (myfft.F90:192-203) inverts the 5-point D D^T of the cell
grid with zero values outside it; uniform flow past no body has pressure coefficient zero on
every level (its coarsest ring is |u|^2/2, every finer ring copies the constant, and the
dynamic part cancels it)."""
import numpy as np

import ib_oracle as O
from helpers import SMALL, rel, small_plate


def _o(bodies=()):
    kw = {k: v for k, v in SMALL.items() if k in O.Params.__dataclass_fields__}
    return O.IBOracle(O.Params(**kw), list(bodies))


def test_ddti_inverts_ddt():
    o = _o()
    rng = np.random.default_rng(3)
    r = rng.standard_normal((o.n, o.m))
    p = o.ddti(r)
    P = np.pad(p, 1)
    lap = P[1:-1, 2:] + P[1:-1, :-2] + P[2:, 1:-1] + P[:-2, 1:-1] - 4.0 * p
    assert rel(lap, r) < 1e-12


def test_uniform_flow_zero_pressure_coefficient():
    o = _o()
    o.advance()
    for k, p in enumerate(o.calculate_pressure()):
        assert np.abs(p).max() < 1e-12, (k, np.abs(p).max())


def test_pressure_after_steps_is_finite_and_varies():
    b = small_plate()
    o = _o([O.Body(x=b.x, y=b.y, fam=2, gamma0_deg=b.gamma0_deg, itheta=b.itheta, ktheta=b.ktheta)])
    for _ in range(2):
        o.advance()
    p = o.calculate_pressure()
    assert all(np.isfinite(x).all() for x in p)
    assert np.abs(p[0]).max() > 1e-3      # the body loads the flow
