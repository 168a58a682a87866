"""ib_calculate_pressure (operators_pressure.F90:110-437) against the oracle on the same state:
the GPU's state after a few steps goes to the oracle through the restart file, so both recover
the pressure from identical fields.  The level solves (ddti) invert the cell grid's D D^T,
whose lowest modes have condition ~(2n/pi)^2, hence 1e-11 on the small grids and 1e-10 at
800x400."""
import numpy as np
import pytest

import ib_oracle as O
from helpers import PLATE, SMALL, pair, rel, small_cylinder, small_plate
from ib_parallel_gb300 import geometry as GEO
from ib_parallel_gb300 import ibgpu as G
from test_gpu_fullsize import _pair

pytestmark = pytest.mark.gpu


def _check(o, g, tmp_path, tol):
    path = tmp_path / "data00.var"
    g.write_variables(path)
    O.restore(o, O.read_variables(path), itime=0)
    pg = g.pressure()
    po = o.calculate_pressure()
    for k in range(o.L):
        assert rel(pg[k], po[k]) < tol, (k, rel(pg[k], po[k]))
    return pg


@pytest.mark.parametrize("case", ["cylinder", "plate"])
def test_pressure_matches_oracle(case, tmp_path):
    kw, body = (SMALL, small_cylinder()) if case == "cylinder" else (PLATE, small_plate())
    o, g = pair(kw, [body])
    for _ in range(3):
        g.advance()
    _check(o, g, tmp_path, 1e-11)
    # the pressure file: the index range, then one record per level
    g.write_pressure(tmp_path / "pressure00.var")
    recs = O.read_records(tmp_path / "pressure00.var")
    assert len(recs) == 1 + kw["mgridlev"]
    assert list(np.frombuffer(recs[0], "<i4")) == [1, kw["m"], kw["m"], 1, kw["n"], kw["n"]]
    g.close()


def test_pressure_fullsize(tmp_path):
    p, bodies = GEO.config_plate_800x400()
    o, g = _pair(p, bodies)
    for _ in range(2):
        g.advance()
    _check(o, g, tmp_path, 1e-10)
    g.close()


def test_uniform_flow_zero_pressure():
    g = G.Simulation(G.Params(**SMALL), [])
    g.advance()
    for k, pk in enumerate(g.pressure()):
        assert np.abs(pk).max() < 1e-12, k
    g.close()


def test_transform_timing_paths_run():
    g = G.Simulation(G.Params(**dict(SMALL, m=128, n=64)), [])
    assert g.time_pass(2, 3) > 0.0 and g.time_pass(3, 3) > 0.0
    g.close()
