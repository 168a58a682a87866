"""The ring maps: the predictor's and vort2flux's coarse-to-fine recursions with the chain of
level solves collapsed (levels solved together with zero boundary data, boundary data from
precomputed dense products, final solves together), against the oracle and against the
level-by-level chain (IB_RING_MAPS=0)."""
import numpy as np
import pytest

import ib_oracle as O
from helpers import PLATE, SMALL, pair, rel, small_cylinder, small_plate
from ib_parallel_gb300 import ibgpu as G

pytestmark = pytest.mark.gpu


def _cyl_body():
    cyl = O.cylinder(npts=10, diameter=0.8, xc=0.3, yc=0.0)
    return G.Body(x=cyl.x.copy(), y=cyl.y.copy(), fam=1)


def test_ring_maps_in_use(monkeypatch):
    # only with IB_RING_MAPS=1, from 3 levels on
    monkeypatch.delenv("IB_RING_MAPS", raising=False)
    g = G.Simulation(G.Params(**dict(SMALL, mgridlev=5)), [small_cylinder()])
    assert not g.ring_maps()["on"]
    g.close()
    monkeypatch.setenv("IB_RING_MAPS", "1")
    for L, on in ((2, False), (3, True), (4, True), (5, True)):
        g = G.Simulation(G.Params(**dict(SMALL, mgridlev=L)), [small_cylinder()])
        rm = g.ring_maps()
        assert rm["on"] == on, L
        if on:
            assert rm["bytes"] > 0 and rm["ms"] > 0.0
        g.close()
    monkeypatch.setenv("IB_RING_MAPS", "0")
    g = G.Simulation(G.Params(**dict(SMALL, mgridlev=5)), [small_cylinder()])
    assert not g.ring_maps()["on"]
    g.close()


@pytest.mark.parametrize("L", [3, 4, 5])
def test_vort2flux_by_ring_maps(monkeypatch, L):
    # operators_fluid.F90:237-377 on random vorticity of every level (the full recursion)
    monkeypatch.setenv("IB_RING_MAPS", "1")
    o, g = pair(dict(SMALL, mgridlev=L), [small_cylinder()])
    assert g.ring_maps()["on"]
    rng = np.random.default_rng(40 + L)
    w = [rng.standard_normal((o.n - 1, o.m - 1)) for _ in range(L)]
    wg, sg, qxg, qyg = g.vort2flux([x.copy() for x in w])
    wo = [x.copy() for x in w]
    so, qxo, qyo = o.vort2flux(wo)
    for k in range(L):
        assert rel(wg[k], wo[k]) < 1e-13
        assert rel(sg[k], so[k]) < 1e-12, k
        assert rel(qxg[k], qxo[k]) < 1e-12, k
        assert rel(qyg[k], qyo[k]) < 1e-12, k
    g.close()


@pytest.mark.parametrize("L", [3, 4, 5])
def test_steps_by_ring_maps(monkeypatch, L):
    # 30 steps of a stationary cylinder (direct solve) on a coarse grid, so that the coarser
    # levels carry vorticity: every level against the oracle, and against the same steps
    # through the level-by-level chain
    kw = dict(m=32, n=16, mgridlev=L, dt=0.05, Re=100.0, len=4.0, offsetx=1.0, offsety=1.0, num_stat=True,
              autotune=False)
    monkeypatch.setenv("IB_RING_MAPS", "1")
    o, g = pair(kw, [_cyl_body()])
    assert g.ring_maps()["on"]
    monkeypatch.setenv("IB_RING_MAPS", "0")
    h = G.Simulation(G.Params(**kw), [_cyl_body()])
    assert not h.ring_maps()["on"]
    for step in range(30):
        o.advance()
        g.advance()
        h.advance()
        if step in (0, 29):
            for k in range(L):
                assert rel(g.get_field("omega", k), o.omega[k]) < 1e-10, (step, k)
                assert rel(g.get_field("omega", k), h.get_field("omega", k)) < 1e-12, (step, k)
                assert rel(g.get_field("s", k), h.get_field("s", k)) < 1e-12, (step, k)
            assert rel(g.forces(), h.forces()) < 1e-11
    g.close()
    h.close()


def test_moving_plate_by_ring_maps(monkeypatch):
    # the hinged plate (GMRES on the influence band, FSI iterations on the device) at 4 levels:
    # the same FSI iterations and the same motion as through the level-by-level chain
    kw = dict(PLATE, mgridlev=4, rtol=1e-12, atol=1e-14)
    monkeypatch.setenv("IB_RING_MAPS", "1")
    g = G.Simulation(G.Params(**kw), [small_plate()])
    assert g.ring_maps()["on"]
    monkeypatch.setenv("IB_RING_MAPS", "0")
    h = G.Simulation(G.Params(**kw), [small_plate()])
    for step in range(8):
        g.advance()
        h.advance()
        assert g.counters()[1] == h.counters()[1], step
    assert rel(g.body_state()[0], h.body_state()[0]) < 1e-10
    for k in range(4):
        assert rel(g.get_field("omega", k), h.get_field("omega", k)) < 1e-10
    g.close()
    h.close()
