"""The CUDA path (through the C ABI) against the committed regression vectors."""
from pathlib import Path

import numpy as np
import pytest

from ib_parallel_gb300 import geometry as GEO
from ib_parallel_gb300 import ibgpu as G

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"

CYL = dict(m=64, n=32, mgridlev=3, dt=0.01, Re=100.0, len=8.0, offsetx=2.0, offsety=2.0,
           fsi_tol=1e-9, atol=1e-12, rtol=1e-11, num_stat=True, autotune=False)


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("steps,name,tol", [(1, "cylinder64x32_direct_1step.npz", 1e-11),
                                            (10, "cylinder64x32_direct_10steps.npz", 1e-9)])
def test_cylinder_direct(steps, name, tol):
    ref = np.load(GOLD / name)
    sim = G.Simulation(G.Params(**CYL), [GEO.cylinder(npts=25)])
    for _ in range(steps):
        sim.advance()
    assert _rel(sim.get_field("omega", 0), ref["omega0"]) < tol
    assert _rel(sim.get_field("omega", 1), ref["omega1"]) < tol
    assert _rel(sim.get_field("omega", 2), ref["omega2"]) < tol
    assert _rel(sim.get_field("s", 0), ref["s0"]) < tol
    assert _rel(sim.get_field("qx", 0), ref["qx0"]) < tol
    assert _rel(sim.get_field("qy", 0), ref["qy0"]) < tol
    assert _rel(sim.get_vector("f"), ref["f"]) < tol
    assert _rel(sim.get_vector("f_rdst"), ref["f_rdst"]) < tol
    cx, cy = sim.forces()
    assert _rel(np.r_[cx, cy], np.r_[ref["cx"], ref["cy"]]) < tol
    sim.close()
