"""The reference's input files through the library's C ABI (no GPU needed): the namelist
&read_parameters of input/ib.inp (parameters.F90:51-78) and the body files
input/body.NNN.inp (grid.F90:252-288), the NACA 00XX generator (input/airfoil*/naca00_ibfm.m,
restated) and the prescribed pitching motion."""
import math
from pathlib import Path

import numpy as np
import pytest

from ib_parallel_gb300 import geometry as GEO
from ib_parallel_gb300 import ibgpu as G

REF_INPUT = Path("/root/reference/input")


def test_namelist_fortran_forms(tmp_path):
    p = tmp_path / "ib.inp"
    p.write_text("! a comment line\n&read_parameters  istart=0, ISTOP = 20 ,isave=5\n"
                 " m = 128, n=64  dt = 1.0D-3, Re= 250.,  ! trailing comment\n"
                 " fsi_tol=1.E-9 atol = 1e-10, rtol=2.5d-11, len=4.0, offsetx=1.5, offsety = 2,\n"
                 " mgridlev=4, compute_pressure=.TRUE., num_stat=F, motion_prescribed=t, dimen=2\n/\n")
    params, rc = GEO.read_namelist(p)
    assert (params.m, params.n, params.mgridlev) == (128, 64, 4)
    assert params.dt == 1e-3 and params.Re == 250.0 and params.rtol == 2.5e-11 and params.offsety == 2.0
    assert params.num_stat is False and rc["compute_pressure"] == 1 and rc["motion_prescribed"] == 1
    assert rc["istop"] == 20 and rc["isave"] == 5 and rc["dimen"] == 2


def test_namelist_round_trip_and_errors(tmp_path):
    params = G.Params(m=800, n=400, mgridlev=5, dt=1e-3, Re=500.0, len=8.0, offsetx=1.0, offsety=2.0,
                      fsi_tol=1e-10, atol=1e-10, rtol=1e-10, num_stat=True)
    p = tmp_path / "ib.inp"
    GEO.write_namelist(p, params, {"istop": 2000, "isave": 100})
    back, rc = GEO.read_namelist(p)
    for k in ("m", "n", "mgridlev", "dt", "Re", "len", "offsetx", "offsety", "fsi_tol", "atol", "rtol", "num_stat"):
        assert getattr(back, k) == getattr(params, k), k
    assert rc["istop"] == 2000 and rc["isave"] == 100
    (tmp_path / "bad.inp").write_text("&read_parameters m=8, bogus=1 /\n")
    with pytest.raises(G.IbError, match="unknown namelist item"):
        GEO.read_namelist(tmp_path / "bad.inp")
    (tmp_path / "bad2.inp").write_text("&read_parameters m=8.5 /\n")
    with pytest.raises(G.IbError, match="bad value"):
        GEO.read_namelist(tmp_path / "bad2.inp")


def test_body_files_round_trip(tmp_path):
    plate = GEO.torsional_plate(npts=29, gamma0_deg=-19.0, itheta=1e-3, ktheta=1e-3)
    cyl = GEO.cylinder(npts=78)
    GEO.write_body_file(tmp_path / "body.001.inp", cyl)
    GEO.write_body_file(tmp_path / "body.002.inp", plate)
    GEO.write_namelist(tmp_path / "ib.inp", G.Params(m=64, n=32, mgridlev=3, dt=0.01, Re=100.0, len=8.0,
                                                     offsetx=2.0, offsety=2.0))
    params, rc, bodies = GEO.load_input(tmp_path)
    assert [b.fam for b in bodies] == [1, 2] and params.m == 64
    # the files carry 16 decimals, as the reference's MATLAB writers print them
    assert np.allclose(bodies[0].x, cyl.x, rtol=0, atol=1e-16) and np.allclose(bodies[1].y, plate.y, rtol=0, atol=1e-16)
    assert bodies[1].gamma0_deg == -19.0 and bodies[1].itheta == 1e-3 and bodies[1].ctheta == 0.0


def test_body_file_with_extra_line_rejected(tmp_path):
    # input/cylinder/build_cylinder.m writes a line 'F' before the family, which the
    # reference's READ of an integer family (grid.F90:258) cannot take
    p = tmp_path / "body.001.inp"
    p.write_text("3 \nF \n1 \n0.0 0.0\n1.0 0.0\n0.0 1.0\n")
    with pytest.raises(G.IbError, match="family"):
        GEO.read_body_file(p)


@pytest.mark.skipif(not (REF_INPUT / "ib.inp").exists(), reason="the reference's input files are not here")
def test_reference_input_directory():
    params, rc, bodies = GEO.load_input(REF_INPUT)
    assert (params.m, params.n, params.mgridlev) == (860, 860, 5)
    assert params.dt == 0.0004375 and params.Re == 1000.0 and params.fsi_tol == 1e-7
    assert rc["sub_domain"] == 1 and rc["compute_pressure"] == 1 and rc["istop"] == 10
    assert [b.npts for b in bodies] == [287, 29] and [b.fam for b in bodies] == [1, 2]
    assert bodies[1].gamma0_deg == -19.0 and bodies[1].ktheta == 1e-3
    ds = np.hypot(np.diff(bodies[1].x), np.diff(bodies[1].y))
    assert np.allclose(ds, ds[0], rtol=1e-9)


def test_naca0012_generator():
    ds = 0.01
    x, y = GEO.naca00(12.0, ds, 1.0, 0.0)
    d = np.hypot(np.diff(x), np.diff(y))
    assert np.allclose(d, ds, rtol=1e-9)                  # every neighbour pair ds apart
    n = len(x) // 2
    assert np.array_equal(x[:n][::-1], x[n:]) and np.array_equal(y[:n][::-1], -y[n:])
    assert abs(x.max() - 1.0) < ds and x.min() > 0.0       # chord within a spacing of 1
    assert abs(2 * y.max() - 0.12) < 0.01                  # 12% thick
    xr, yr = GEO.naca00(12.0, ds, 1.0, 10.0)
    assert yr[0] < 0.0                                     # nose up: the trailing edge drops
    assert np.allclose(np.hypot(xr, yr), np.hypot(x, y))


def test_pitching_motion_velocity():
    x, y = GEO.naca00(12.0, 0.02, 1.0, 0.0)
    t, h = 0.37, 1e-6
    xb, yb, ub = GEO.pitching_motion(x, y, t, 10.0, 0.2, 0.3)
    xp, yp, _ = GEO.pitching_motion(x, y, t + h, 10.0, 0.2, 0.3)
    xm, ym, _ = GEO.pitching_motion(x, y, t - h, 10.0, 0.2, 0.3)
    n = len(x)
    assert np.allclose(ub[:n], (xp[:n] - xm[:n]) / (2 * h), atol=1e-8)
    assert np.allclose(ub[n:], (yp[:n] - ym[:n]) / (2 * h), atol=1e-8)
    assert np.array_equal(xb[:n], xb[n:])
