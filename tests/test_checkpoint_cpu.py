"""The restart file output/dataRR_IIIIIII.var (variables.F90:709-913) in the oracle.

The layout is the reference's Fortran unformatted stream as its own reader output/getdata.m
parses it: each WRITE is a record framed by its byte length (4-byte integer) before and
after, integers 4 bytes, reals 8.  Checked here: the record sequence and header values, a
write/read round trip, and that a run restarted from the file continues exactly as the run
that wrote it.
"""
import numpy as np
import pytest

import ib_oracle as O
from helpers import PLATE, small_plate


def _oracle():
    b = small_plate()
    kw = {k: v for k, v in PLATE.items() if k in O.Params.__dataclass_fields__}
    return O.IBOracle(O.Params(**kw), [O.Body(x=b.x.copy(), y=b.y.copy(), fam=2, gamma0_deg=b.gamma0_deg,
                                              itheta=b.itheta, ktheta=b.ktheta)])


def test_record_layout(tmp_path):
    o = _oracle()
    for _ in range(2):
        o.advance()
    path = tmp_path / "data00_0000002.var"
    O.write_variables(o, path)
    recs = O.read_records(path)
    L, m, n, nf = o.L, o.m, o.n, o.nf
    # 5 header records, 8 per level, rhs_old, frame, force range, f, xb, yb, mt_body, theta, f_rdst
    assert len(recs) == 5 + 8 * L + 1 + 1 + 1 + 3 + 1 + 1 + 1
    assert list(np.frombuffer(recs[0], "<i4")) == [m, n, L, o.nb]
    assert list(np.frombuffer(recs[2], "<i4")) == [2, m, m - 1, 2, n, n - 1]
    assert list(np.frombuffer(recs[3], "<i4")) == [1, m + 1, m + 1, 1, n, n]
    assert list(np.frombuffer(recs[4], "<i4")) == [1, m, m, 1, n + 1, n + 1]
    assert len(recs[5]) == 8 * (m - 1) * (n - 1) and len(recs[7]) == 8 * (m + 1) * n
    assert len(recs[5 + 8 * L]) == 8 * L * (m - 1) * (n - 1)          # rhs_old, every level
    raw = path.read_bytes()
    assert np.frombuffer(raw[:4], "<i4")[0] == 16 and np.frombuffer(raw[20:24], "<i4")[0] == 16
    d = O.read_variables(path)
    assert d["mt_body"] == 1 and d["xfm"] == nf and d["xfi"] == 1 and d["xfe"] == nf
    for k in range(L):
        assert np.array_equal(d["omega"][k], o.omega[k]) and np.array_equal(d["qy"][k], o.qy[k])
        assert np.array_equal(d["q0px"][k] + d["q0rx"][k], o.q0x[k])
        assert np.array_equal(d["rhs_old"][k], o.rhs_old[k])
    assert np.array_equal(d["theta"], o.theta) and np.array_equal(d["f_rdst"], o.f_rdst)


def test_restart_continues_exactly(tmp_path):
    a = _oracle()
    for _ in range(2):
        a.advance()
    path = tmp_path / "data00_0000002.var"
    O.write_variables(a, path)
    b = _oracle()
    O.restore(b, O.read_variables(path), itime=2)
    for _ in range(2):
        a.advance()
        b.advance()
    assert a.itime == b.itime == 4
    for k in range(a.L):
        assert np.array_equal(a.omega[k], b.omega[k])
    assert np.array_equal(a.f, b.f) and np.array_equal(a.theta, b.theta)


def test_bad_framing_rejected(tmp_path):
    o = _oracle()
    path = tmp_path / "x.var"
    O.write_variables(o, path)
    raw = bytearray(path.read_bytes())
    raw[-1] ^= 0x40                      # corrupt the last record's trailing marker
    path.write_bytes(bytes(raw))
    with pytest.raises(ValueError):
        O.read_records(path)
