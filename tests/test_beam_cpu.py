"""The Euler-Bernoulli beam (body family 3) of the oracle against beam theory.  The reference
declares the family and leaves it empty (operators_struct.F90:104-106 and the other family-3
branches), so these identities pin the formulation instead: Hermite-cubic elements give the
exact cantilever tip deflection P L^3 / (3 EI) under a tip load, the first natural frequency
1.8751^2 sqrt(EI / (rho L^4)), and the trapezoidal Newmark update conserves the energy of free
vibration; coupled to the fluid, the FSI iterations converge."""
import math

import numpy as np

import ib_oracle as O
from helpers import PLATE
from ib_parallel_gb300 import geometry as GEO


def _beam(npts=21, nel=10, rho=0.5, EI=1e-3, dt=1e-3):
    b = GEO.beam_plate(npts, 1.0, 10.0, rho, EI, nelem=nel)
    return O.BeamBody(O.Body(x=b.x, y=b.y, fam=3, itheta=rho, ktheta=EI, nelem=nel), 0, dt)


def test_cantilever_tip_load():
    bm = _beam()
    F = np.zeros(bm.ndof)
    F[-2] = 2.0e-4                                # tip transverse load P
    q = np.linalg.solve(bm.K, F)
    assert abs(q[-2] - 2.0e-4 / (3.0 * 1e-3)) < 1e-12 * 2.0e-4 / 3e-3 * 1e3
    # the body points follow the deflected shape, along the beam's normal
    bm.q = q
    px, py = bm.positions()
    d = np.hypot(px - bm.x0, py - bm.y0)
    assert abs(d[-1] - abs(q[-2])) < 1e-14 and d[0] == 0.0


def test_first_natural_frequency():
    import scipy.linalg as sla
    bm = _beam(npts=21, nel=20)
    w2 = sla.eigh(bm.K, bm.M, eigvals_only=True)
    w1 = math.sqrt(w2[0])
    exact = 1.875104068711961 ** 2 * math.sqrt(1e-3 / 0.5)
    assert abs(w1 / exact - 1.0) < 1e-5


def test_newmark_conserves_energy():
    bm = _beam()
    F = np.zeros(bm.ndof)
    F[-2] = 1.0e-4
    bm.q = np.linalg.solve(bm.K, F)               # released from the static tip-load shape
    bm.qdd = bm.Mi @ (-bm.K @ bm.q)
    energy = lambda: 0.5 * bm.qd @ bm.M @ bm.qd + 0.5 * bm.q @ bm.K @ bm.q
    e0 = energy()
    zero = np.zeros(2 * bm.npts)
    for _ in range(2000):
        bm.save()
        bm.dx(zero, 0.01)
    assert abs(energy() / e0 - 1.0) < 1e-9
    assert abs(bm.q[-2]) < abs(np.linalg.solve(bm.K, F)[-2]) * 1.01   # it oscillates, bounded


def test_coupled_steps_converge():
    b = GEO.beam_plate(9, 1.0, 10.0, 0.5, 1e-2)
    kw = {k: v for k, v in PLATE.items() if k in O.Params.__dataclass_fields__}
    o = O.IBOracle(O.Params(**kw), [O.Body(x=b.x, y=b.y, fam=3, itheta=b.itheta, ktheta=b.ktheta)])
    for _ in range(3):
        o.advance()
        assert 1 < o.fsi_iter < 20
    assert o.beams[0].q[-2] > 0.0                 # the flow lifts the nose-down plate's tip
