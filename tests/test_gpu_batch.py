"""Batches of independent simulations (ib_batch_*): uneven grids and bodies advanced
together must give, simulation by simulation, exactly the results of advancing each alone
through ib_advance (the same kernels in the same order on each simulation's stream), and report
each simulation's own status."""
import ctypes as C

import numpy as np
import pytest

from helpers import PLATE, SMALL, small_cylinder, small_plate
from ib_parallel_gb300 import geometry as GEO
from ib_parallel_gb300 import ibgpu as G

pytestmark = pytest.mark.gpu


def _runs():
    return [
        (G.Params(**PLATE), [small_plate()]),
        (G.Params(**dict(SMALL, m=96, n=48)), [small_cylinder()]),
        (G.Params(**dict(PLATE, m=128, n=64, Re=300.0)),
         [GEO.torsional_plate(npts=17, length=1.0, gamma0_deg=-15.0, itheta=0.2, ktheta=2e-3)]),
        (G.Params(**dict(SMALL, num_stat=True)), [small_cylinder()]),
    ]


def test_batch_equals_plain_runs():
    runs = _runs()
    batch = G.Batch(runs)
    plain = [G.Simulation(p, b) for p, b in runs]
    for step in range(4):
        assert batch.advance() == [0] * len(runs)
        for s in plain:
            s.advance()
        for i, (s, t) in enumerate(zip(plain, batch.sims)):
            assert s.counters() == t.counters(), (step, i)
    for i, (s, t) in enumerate(zip(plain, batch.sims)):
        for k in range(s.params.mgridlev):
            assert np.array_equal(s.get_field("omega", k), t.get_field("omega", k)), (i, k)
            assert np.array_equal(s.get_field("qx", k), t.get_field("qx", k)), (i, k)
        assert np.array_equal(s.get_vector("f"), t.get_vector("f")), i
        assert np.array_equal(s.body_state()[0], t.body_state()[0]), i
        s.close()
    batch.close()


def test_batch_status_per_simulation():
    runs = _runs()[:2] + [(G.Params(**dict(PLATE, gmres_max_it=2, fsi_max_it=1)), [small_plate()])]
    batch = G.Batch(runs)
    for _ in range(2):
        st = batch.advance(check=False)
        assert st == [0, 0, 4], st
    assert batch.sims[0].counters()[1] > 0
    # a simulation's handle stays the batch's
    assert batch.lib.ib_destroy(batch.sims[0].h) == 1
    batch.close()


def test_batch_rejects_bad_member():
    runs = _runs()[:1] + [(G.Params(**dict(SMALL, m=30)), [])]
    with pytest.raises(G.IbError, match="simulation 1"):
        G.Batch(runs)
