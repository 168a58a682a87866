"""The oracle's sub-domain method (grid.F90:320-352, 572-951; timestepper.F90:368-405, 500-516,
602-770; operators_struct.F90:840-980) pinned by what the reference's construction implies:
the cloud's layout, E E^T's sparsity, the symmetry of the fluid operator before the drop, the
drop rule, bilinear interpolation reproducing linear functions, the exact operator recovered
where the body points are cloud points, the sd_precomputed.chd records, and steps close to the
standard method's."""
import struct

import numpy as np
import pytest

import ib_oracle as O
import ib_subdomain as SD
from helpers import PLATE

CLOUD = (-0.25, 1.25, -0.25, 0.25, 0.0625)   # sdxi, sdxe, sdyi, sdye, delta_sd


def _oracle(bodies, **kw):
    p = O.Params(**{k: v for k, v in dict(PLATE, **kw).items() if k in O.Params.__dataclass_fields__})
    return O.IBOracle(p, bodies)


def _plate(**kw):
    args = dict(npts=17, length=1.0, gamma0_deg=-10.0, itheta=0.5 / 3.0, ktheta=1e-3)
    args.update(kw)
    return O.torsional_plate(**args)


@pytest.fixture(scope="module")
def plate_sd():
    o = _oracle([_plate()])
    sd = SD.SubDomain(o, True, *CLOUD)
    full = {}
    for j in range(sd.nf_sd):
        full[j] = sd.column(j)
    sd.cols = [sd.drop(j, full[j]) for j in range(sd.nf_sd)]
    return o, sd, full


def test_cloud_layout():
    cyl = O.cylinder(npts=25, diameter=0.3, xc=0.5, yc=0.0)
    o = _oracle([cyl, _plate(x0=0.0, y0=0.0)])
    sd = SD.SubDomain(o, False, *CLOUD)
    assert (sd.nx, sd.ny) == (25, 9)
    assert sd.nr_sd == 25 and sd.nb_sd == 25 + 25 * 9 and sd.nf_sd == 2 * sd.nb_sd
    assert np.array_equal(sd.px[:25], cyl.x) and np.array_equal(sd.py[:25], cyl.y)
    # the rectangle, x fastest, after the rigid points
    assert sd.px[25 + 1] - sd.px[25] == pytest.approx(0.0625) and sd.py[25 + 25] - sd.py[25] == pytest.approx(0.0625)
    # x components then y components; the rigid unknowns map onto their own points
    assert np.array_equal(sd.ucomp[:sd.nb_sd], np.ones(sd.nb_sd)) and (sd.ucomp[sd.nb_sd:] == 2).all()
    assert list(sd.rigid_pt[:3]) == [0, 1, 2] and list(sd.rigid_pt[25:28]) == [0, 1, 2]
    assert (sd.rigid_pt[50:] == -1).all()


def test_cloud_must_keep_its_blocks_inside_the_grid():
    o = _oracle([_plate()])
    with pytest.raises(ValueError):
        SD.SubDomain(o, True, -0.25, 1.25, -0.40, 0.25, 0.0625)   # a row 9 cells from the bottom


def test_sparsity_is_block_overlap(plate_sd):
    o, sd, _ = plate_sd
    for k in (0, 7, sd.nb_sd // 2, sd.nb_sd - 1):
        d = np.maximum(np.abs(sd.gix - sd.gix[k]), np.abs(sd.giy - sd.giy[k]))
        assert np.array_equal(sd.cand[k], np.nonzero(d <= 20)[0])
        rows = sd.rows_of(k)
        assert np.array_equal(rows, np.concatenate([sd.cand[k], sd.cand[k] + sd.nb_sd]))
        assert np.all(np.diff(rows) > 0)


def test_fluid_operator_is_nearly_symmetric_before_the_drop(plate_sd):
    # E curl G rot E^T: symmetric but for the nested grids' boundary coupling (coarsify and the
    # coarse ring are not each other's transposes), a few 1e-5 here
    _, sd, full = plate_sd
    B = np.array([full[j] for j in range(sd.nf_sd)]).T   # B[:, j] = column j on every unknown
    assert np.abs(B - B.T).max() < 1e-4 * np.abs(B).max()
    assert (np.diag(B) > 0).all()


def test_drop_rule(plate_sd):
    _, sd, full = plate_sd
    for j in range(0, sd.nf_sd, 37):
        rows, vals = sd.cols[j]
        cand = sd.rows_of(j)
        thr = SD.DROPTOL * full[j][j]
        kept = cand[np.abs(full[j][cand]) > thr]
        assert np.array_equal(rows, kept) and np.array_equal(vals, full[j][kept])
        assert j in rows
    assert SD.DROPTOL == float(np.float32(7.0e-3)) and SD.DROPTOL != 7.0e-3


def test_bilinear_interpolation(plate_sd):
    o, sd, _ = plate_sd
    idx, w = sd.interp()
    assert np.allclose(w.sum(axis=1), 1.0, rtol=0, atol=1e-15)
    pt = idx % sd.nb_sd
    # linear functions are reproduced exactly (up to round-off)
    assert np.abs((w * sd.px[pt]).sum(axis=1) - o.xb).max() < 1e-14
    assert np.abs((w * sd.py[pt]).sum(axis=1) - o.yb).max() < 1e-14
    # y unknowns interpolate from y components
    assert (idx[o.comp == 2] >= sd.nb_sd).all() and (idx[o.comp == 1] < sd.nb_sd).all()


def test_leaving_the_cloud_is_an_error():
    o = _oracle([_plate()])
    sd = SD.SubDomain(o, True, -0.25, 0.5, -0.25, 0.25, 0.0625)   # the plate reaches x = 0.98
    with pytest.raises(ValueError):
        sd.interp()


def test_exact_operator_where_body_points_are_cloud_points():
    # a flat plate whose points are cloud points: P selects them, so lumat's fluid part is B on
    # those unknowns, the exact Schur operator except for the dropped entries
    plate = _plate(npts=9, gamma0_deg=0.0)
    o = _oracle([plate])
    sd = SD.SubDomain(o, True, *CLOUD)
    idx, w = sd.interp()
    assert set(np.unique(w)) == {0.0, 1.0} and (w[:, 0] == 1.0).all()
    sel = sorted(set(idx[:, 0]) | set(idx[:, 0]))
    sd.precompute(columns=sel)
    sd.cols = [c if c is not None else (np.zeros(0, np.int64), np.zeros(0)) for c in sd.cols]
    M = sd.lumat(idx, w)
    nf = o.nf
    S = np.zeros((nf, nf))
    body = np.zeros((nf, nf))
    for l in range(nf):
        e = np.zeros(nf); e[l] = 1.0
        S[:, l] = o.a_times(e, with_b=False)   # the exact fluid part
        body[:, l] = o.b_times(e)
    # lumat = body + P B^T P^T: with P a selection, the fluid part is S transposed where B kept
    # the entry (column k of B is S's row k) and zero where the drop tolerance removed it
    Mf = M - body
    St = S.T
    kept = Mf != 0.0
    diag = np.diag(S)
    assert np.abs(Mf - St)[kept].max() <= 1e-12 * np.abs(S).max()
    assert (np.abs(St[~kept]) <= SD.DROPTOL * diag[:, None].repeat(nf, 1)[~kept]).all()
    assert (~kept).sum() > 0 and kept.sum() > nf


def test_chd_records_round_trip(plate_sd, tmp_path):
    _, sd, _ = plate_sd
    path = tmp_path / "sd_precomputed.chd"
    sd.write_chd(path)
    data = path.read_bytes()
    n0 = len(sd.cols[0][0])
    assert struct.unpack_from("<iii", data, 0) == (4, n0, 4)
    assert struct.unpack_from("<i", data, 12)[0] == 12 * n0
    assert struct.unpack_from("<i", data, 16 + 8 * n0)[0] == sd.cols[0][0][0] + 1   # 1-based rows
    other = SD.SubDomain(sd.o, True, *CLOUD)
    other.read_chd(path)
    for (r1, v1), (r2, v2) in zip(sd.cols, other.cols):
        assert np.array_equal(r1, r2) and np.array_equal(v1, v2)


def test_steps_close_to_the_standard_method(plate_sd):
    o, sd, _ = plate_sd
    std = _oracle([_plate()])
    osd = _oracle([_plate()])
    osd.sd = SD.SubDomain(osd, True, *CLOUD)
    osd.sd.cols = sd.cols
    for _ in range(3):
        std.advance()
        osd.advance()
    # an approximation of the same operator: the hinge angle within 1%
    assert abs(osd.theta[0] - std.theta[0]) < 1e-2 * abs(std.theta[0])
    assert osd.fsi_iter >= 2 and osd.ksp_iter > 0
