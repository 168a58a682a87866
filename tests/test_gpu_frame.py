"""The frame's motion set per step (ib_set_frame, in place of the reference's motion_potential +
motion_rotation, variables.F90:299-360): the fluxes it forms against those of creation and of
the oracle, and steps of a frame that changes every step against the oracle, which forms q0
from motion_grid at every step (timestepper.F90:18-556)."""
import math

import numpy as np
import pytest

from helpers import SMALL, pair, rel, small_cylinder
from ib_parallel_gb300 import ibgpu as G

pytestmark = pytest.mark.gpu

KW = dict(SMALL, motion=(-1.0, 0.2, 0.3, 0.1, -0.05))


def _fluxes(g):
    return [(g.get_field("q0x", k), g.get_field("q0y", k)) for k in range(KW["mgridlev"])]


def test_configured_motion_reproduces_the_creation_fluxes():
    g = G.Simulation(G.Params(**KW), [small_cylinder()])
    before = _fluxes(g)
    g.set_frame(*KW["motion"][:3])
    for (ax, ay), (bx, by) in zip(before, _fluxes(g)):
        assert np.array_equal(ax, bx) and np.array_equal(ay, by)
    g.close()


def test_another_frame_matches_the_oracle_fluxes():
    fr = (0.5, -0.7, 1.3)
    o, _ = pair(dict(KW, motion=fr + KW["motion"][3:]), [small_cylinder()])
    g = G.Simulation(G.Params(**KW), [small_cylinder()])
    g.set_frame(*fr)
    q0x, q0y = o.frame_flux(0)
    for k, (ax, ay) in enumerate(_fluxes(g)):
        assert rel(ax, q0x[k]) < 1e-15 and rel(ay, q0y[k]) < 1e-15, k
    with pytest.raises(G.IbError):
        g.set_frame(float("nan"), 0.0, 0.0)
    g.close()


@pytest.mark.parametrize("num_stat", [True, False])
def test_steps_of_a_turning_frame_match_the_oracle(num_stat):
    kw = dict(KW, num_stat=num_stat, rtol=1e-14, atol=1e-16)
    o, g = pair(kw, [small_cylinder()])
    for step in range(1, 6):
        a = 0.2 * math.sin(0.7 * step)
        fr = (-math.cos(a), -math.sin(a), -0.14 * math.cos(0.7 * step))
        g.set_frame(*fr)
        o.p.motion = fr + KW["motion"][3:]
        g.advance()
        o.advance()
        tol = 1e-11 if step == 1 else 1e-10
        for k in range(o.L):
            assert rel(g.get_field("omega", k), o.omega[k]) < tol, (step, k)
        cx, cy = g.forces()
        ox, oy = o.force_coeffs(o.f)
        assert rel(np.r_[cx, cy], np.r_[ox, oy]) < tol, step
    g.close()


def test_step_outputs_follow_the_state():
    # once the host has read a step's forces, later steps copy their force coefficients and
    # hinge angles to pinned memory before they finish, and the getters read them there; any
    # other entry point (here the forces set directly) makes the getters go to the device again
    from helpers import PLATE, small_plate
    g = G.Simulation(G.Params(**PLATE), [small_plate()])
    th = np.zeros(1)

    def theta():
        G._check(g.lib.ib_get_body_state(g.h, G._ptr(th), None, None), "ib_get_body_state")
        return th.copy()

    g.advance()
    g.forces()
    for _ in range(3):
        g.advance()
        cx, cy = g.forces()
        t = theta()
        g.synchronize()                      # any other call: the next reads go to the device
        cx2, cy2 = g.forces()
        assert np.array_equal(cx, cx2) and np.array_equal(cy, cy2)
        assert np.array_equal(t, theta()) and np.array_equal(t, g.body_state()[0])
    f = g.get_vector("f")
    g.set_vector("f", 2.0 * f)
    cx3, _ = g.forces()
    assert np.allclose(cx3, 2.0 * cx2, rtol=1e-14, atol=0)
    g.close()
