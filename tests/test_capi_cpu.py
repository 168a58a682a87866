"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/ib_gpu.h declares (no compute call is made without a GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    text = (ROOT / "include" / "ib_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ib_[A-Za-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from ib_parallel_gb300 import build
    path = build.build()
    return ctypes.CDLL(str(path))


def test_header_declares_entry_points():
    names = _declared()
    assert "ib_advance" in names and "ib_schur_apply" in names and len(names) >= 35


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_lists_every_symbol():
    from ib_parallel_gb300 import ibgpu
    assert sorted(ibgpu.EXPORTS) == _declared()


def test_binding_loads_and_reports_version():
    from ib_parallel_gb300 import ibgpu
    lib = ibgpu.load()
    assert lib.ib_version() == 1


def test_errors_are_reported_without_gpu_work():
    from ib_parallel_gb300 import ibgpu as G
    lib = G.load()
    # invalid grid (not divisible by 4): rejected on the host before any device call
    p = G.Params(m=30, n=16, mgridlev=2, dt=0.01, Re=100, len=4, offsetx=1, offsety=1).to_c()
    h = ctypes.c_void_p()
    rc = lib.ib_create(ctypes.byref(p), None, 0, ctypes.byref(h))
    assert rc == 1
    assert b"divisible by 4" in lib.ib_last_error()
    # null context
    assert lib.ib_advance(None, None) == 1


def _bodies(*specs):
    """A ctypes array of IbBody from (npts, fam, itheta) triples, with its coordinate arrays."""
    import numpy as np
    from ib_parallel_gb300 import ibgpu as G
    arr = (G.IbBody * max(1, len(specs)))()
    keep = []
    for i, (npts, fam, itheta) in enumerate(specs):
        x = np.linspace(0.0, 0.5, npts)
        y = np.zeros(npts)
        keep += [x, y]
        arr[i].npts, arr[i].fam, arr[i].itheta = npts, fam, itheta
        arr[i].x = x.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        arr[i].y = y.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    return arr, keep


@pytest.mark.parametrize("case, message", [
    ("mgridlev", b"mgridlev out of range"),
    ("dt", b"must be positive"),
    ("no_body_list", b"bad body list"),
    ("one_point", b"needs >= 2 points"),
    ("family", b"body family must be 1"),
    ("no_inertia", b"itheta > 0"),
    ("beam_mass", b"mass per length"),
    ("rigid_after_torsional", b"rigid bodies must precede"),
])
def test_create_rejects_bad_input_on_the_host(case, message):
    # every one of these is rejected by ib_create before it touches a device
    from ib_parallel_gb300 import ibgpu as G
    lib = G.load()
    kw = dict(m=32, n=16, mgridlev=2, dt=0.01, Re=100, len=4, offsetx=1, offsety=1)
    specs = [(5, 1, 0.0)]
    if case == "mgridlev":
        kw["mgridlev"] = 0
    elif case == "dt":
        kw["dt"] = 0.0
    elif case == "one_point":
        specs = [(1, 1, 0.0)]
    elif case == "family":
        specs = [(5, 4, 0.0)]
    elif case == "beam_mass":
        specs = [(5, 3, 0.0)]
    elif case == "no_inertia":
        specs = [(5, 2, 0.0)]
    elif case == "rigid_after_torsional":
        specs = [(5, 2, 0.1), (5, 1, 0.0)]
    p = G.Params(**kw).to_c()
    arr, keep = _bodies(*specs)
    h = ctypes.c_void_p()
    bodies = None if case == "no_body_list" else arr
    rc = lib.ib_create(ctypes.byref(p), bodies, len(specs), ctypes.byref(h))
    assert rc == 1, (case, rc, lib.ib_last_error())
    assert message in lib.ib_last_error(), (case, lib.ib_last_error())
    assert not h.value
