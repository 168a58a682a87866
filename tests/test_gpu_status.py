"""Failure status of ib_advance (timestepper.F90:318, 363-366; variables.F90:574).

The reference never reads its KSP convergence reason and leaves the FSI loop silently after
1000 iterations.  ib_advance completes the step the same way and then reports: IB_ERR_GMRES
when a Krylov solve of the step stopped without converging, IB_ERR_FSI when the FSI
iterations stopped at fsi_max_it without reaching fsi_tol.  The loops are made to end early
by their own caps (gmres_max_it, fsi_max_it): nothing faults, nothing waits.  Step 1 runs the
FSI iterations from the host (the influence band is built there); later steps of the moving
plate run them in the device loop, whose counters carry the status back.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import PLATE, SMALL, small_cylinder, small_plate
from ib_parallel_gb300 import ibgpu as G

pytestmark = pytest.mark.gpu

IB_ERR_GMRES, IB_ERR_FSI = 4, 5


def _advance(g):
    it = C.c_int()
    rc = g.lib.ib_advance(g.h, C.byref(it))
    return rc, g.lib.ib_last_error().decode()


@pytest.mark.parametrize("schur_mode", [0, 1])
def test_plate_gmres_cap_reported(schur_mode):
    g = G.Simulation(G.Params(**dict(PLATE, gmres_max_it=2, fsi_max_it=1, schur_mode=schur_mode)),
                     [small_plate()])
    for step in range(3):
        rc, msg = _advance(g)
        assert rc == IB_ERR_GMRES, (step, rc, msg)
        assert "KSP reason -3" in msg
        ksp, fsi = g.counters()
        assert ksp == 2 * fsi and fsi == 2      # every solve stopped at its cap; loop capped too
        assert np.isfinite(g.get_field("omega", 0)).all()
    g.close()


def test_plate_fsi_cap_reported():
    ref = G.Simulation(G.Params(**PLATE), [small_plate()])
    g = G.Simulation(G.Params(**dict(PLATE, fsi_max_it=1)), [small_plate()])
    for step in range(3):
        ref.advance()
        assert ref.counters()[1] > 2           # the problem needs more than 2 FSI iterations
        rc, msg = _advance(g)
        assert rc == IB_ERR_FSI, (step, rc, msg)
        assert "fsi_max_it" in msg
        assert g.counters()[1] == 2            # fsi_count <= fsi_max_it: fsi_max_it + 1 iterations
    ref.close()
    g.close()


def test_rigid_gmres_cap_reported_then_recovers():
    g = G.Simulation(G.Params(**dict(SMALL, gmres_max_it=3)), [small_cylinder()])
    rc, msg = _advance(g)
    assert rc == IB_ERR_GMRES and "KSP reason" in msg
    g.close()
    ok = G.Simulation(G.Params(**SMALL), [small_cylinder()])
    for _ in range(2):
        rc, msg = _advance(ok)
        assert rc == G.IB_OK, msg
    ok.close()
