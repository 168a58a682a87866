"""ib_write_variables / ib_read_variables: the reference's restart file (variables.F90:709-913)
written from and read into a GPU context, checked against the oracle's reader and writer of
the same layout (the one output/getdata.m reads) and by restarting runs."""
import numpy as np
import pytest

import ib_oracle as O
from helpers import PLATE, SMALL, pair, rel, small_cylinder, small_plate
from ib_parallel_gb300 import ibgpu as G

pytestmark = pytest.mark.gpu


def _fields(g, L):
    return {nm: [g.get_field(nm, k) for k in range(L)] for nm in ("omega", "s", "qx", "qy", "q0x", "q0y", "rhs_old")}


def test_gpu_file_read_by_oracle(tmp_path):
    o, g = pair(PLATE, [small_plate()])
    for _ in range(3):
        g.advance()
    path = tmp_path / "data00_0000003.var"
    g.write_variables(path)
    d = O.read_variables(path)
    L = PLATE["mgridlev"]
    fl = _fields(g, L)
    assert (d["m"], d["n"], d["mgridlev"], d["nb"]) == (PLATE["m"], PLATE["n"], L, o.nb)
    for k in range(L):
        for nm in ("omega", "s", "qx", "qy", "rhs_old"):
            assert np.array_equal(d[nm][k], fl[nm][k]), (nm, k)
        assert np.array_equal(d["q0px"][k] + d["q0rx"][k], fl["q0x"][k])
        assert np.array_equal(d["q0py"][k] + d["q0ry"][k], fl["q0y"][k])
    assert np.array_equal(d["f"], g.get_vector("f")) and np.array_equal(d["xb"], g.get_vector("xb"))
    assert np.array_equal(d["f_rdst"], g.get_vector("f_rdst"))
    th, thd, thdd = g.body_state()
    assert np.array_equal(d["theta"], th) and np.array_equal(d["thetadd"], thdd)
    # the oracle writes the same layout, record for record
    O.write_variables(o, tmp_path / "oracle.var")
    assert [len(r) for r in O.read_records(tmp_path / "oracle.var")] == [len(r) for r in O.read_records(path)]
    g.close()


def test_oracle_file_read_by_gpu(tmp_path):
    o, g = pair(PLATE, [small_plate()])
    for _ in range(2):
        o.advance()
    path = tmp_path / "data00_0000002.var"
    O.write_variables(o, path)
    g.read_variables(path, 2)
    for k in range(o.L):
        assert np.array_equal(g.get_field("omega", k), o.omega[k])
        assert np.array_equal(g.get_field("qx", k), o.qx[k])
        assert np.array_equal(g.get_field("rhs_old", k), o.rhs_old[k])
    assert np.array_equal(g.get_vector("xb"), o.xb) and np.array_equal(g.body_state()[0], o.theta)
    g.close()


def test_restart_direct_solve_is_exact(tmp_path):
    kw = dict(SMALL, num_stat=True)
    a = G.Simulation(G.Params(**kw), [small_cylinder()])
    for _ in range(3):
        a.advance()
    path = tmp_path / "data00_0000003.var"
    a.write_variables(path)
    b = G.Simulation(G.Params(**kw), [small_cylinder()])
    b.read_variables(path, 3)
    for _ in range(3):
        a.advance()
        b.advance()
    for k in range(kw["mgridlev"]):
        assert np.array_equal(a.get_field("omega", k), b.get_field("omega", k))
        assert np.array_equal(a.get_field("s", k), b.get_field("s", k))
    assert np.array_equal(a.get_vector("f"), b.get_vector("f"))
    a.close()
    b.close()


def test_restart_from_gpu_file_matches_oracle(tmp_path):
    # the GPU's file restarts the oracle (which factorises, as the GPU does after a restart);
    # the direct solve has no Krylov stopping point, so the next steps agree to round-off
    kw = dict(SMALL, num_stat=True)
    o, g = pair(kw, [small_cylinder()])
    for _ in range(3):
        g.advance()
    path = tmp_path / "data00_0000003.var"
    g.write_variables(path)
    O.restore(o, O.read_variables(path), itime=3)
    o.preprocess()
    for _ in range(2):
        o.advance()
        g.advance()
    for k in range(o.L):
        assert rel(g.get_field("omega", k), o.omega[k]) < 1e-11
    assert rel(g.get_vector("f"), o.f) < 1e-11
    g.close()


def test_restart_moving_plate(tmp_path):
    a = G.Simulation(G.Params(**PLATE), [small_plate()])
    for _ in range(3):
        a.advance()
    path = tmp_path / "data00_0000003.var"
    a.write_variables(path)
    b = G.Simulation(G.Params(**PLATE), [small_plate()])
    b.read_variables(path, 3)
    for _ in range(3):
        a.advance()
        b.advance()
        assert a.counters()[1] == b.counters()[1]
    # the restarted context builds its influence band around the positions read: the same
    # operator, assembled in another order, so agreement is to the solver's round-off
    assert rel(a.body_state()[0], b.body_state()[0]) < 1e-9
    assert rel(a.get_field("omega", 0), b.get_field("omega", 0)) < 1e-8


def test_read_rejects_other_grid(tmp_path):
    a = G.Simulation(G.Params(**PLATE), [small_plate()])
    path = tmp_path / "x.var"
    a.write_variables(path)
    b = G.Simulation(G.Params(**dict(PLATE, m=96)), [small_plate()])
    with pytest.raises(G.IbError):
        b.read_variables(path, 0)
    a.close()
    b.close()
