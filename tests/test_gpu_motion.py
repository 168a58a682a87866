"""Prescribed rigid-body motion (timestepper.F90:262-331, 479; user.F90:87-174): the host
moves the body (IB_VEC_XB/YB) and gives its velocity (IB_VEC_UB) before each step, and -delta
u_B joins every Schur right-hand side.  A heaving cylinder with points two grid spacings apart
(a well-conditioned Schur operator), both solvers run to rtol 1e-14, against the oracle."""
import math

import numpy as np
import pytest

from helpers import SMALL, pair, rel
from ib_parallel_gb300 import geometry as GEO

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("num_stat", [False])
def test_heaving_cylinder(num_stat):
    kw = dict(SMALL, rtol=1e-14, atol=1e-16, num_stat=num_stat)
    body = GEO.cylinder(npts=13)
    o, g = pair(kw, [body])
    A, w, dt = 0.1, 2.0 * math.pi * 0.5, kw["dt"]
    for step in range(1, 5):
        t = step * dt
        yoff, v = A * math.sin(w * t), A * w * math.cos(w * t)
        xb = np.r_[body.x, body.x]
        yb = np.r_[body.y, body.y] + yoff
        ub = np.r_[np.zeros(body.npts), np.full(body.npts, v)]
        g.set_vector("xb", xb); g.set_vector("yb", yb); g.set_vector("ub", ub)
        o.xb, o.yb, o.ub = xb.copy(), yb.copy(), ub.copy()
        o.setup_reg()
        o.advance()
        g.advance()
        tol = 1e-11 if step == 1 else 1e-10
        for k in range(o.L):
            assert rel(g.get_field("omega", k), o.omega[k]) < tol, (step, k)
        assert rel(g.get_vector("f"), o.f) < tol
        cx, cy = g.forces()
        ox, oy = o.force_coeffs(o.f)
        assert rel(np.r_[cx, cy], np.r_[ox, oy]) < tol
    assert abs(cy[0]) > 1e-6     # the heave loads the body
    g.close()
