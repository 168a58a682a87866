"""ib_ctci_static: the context-free Poisson solve that allocates no device memory.

Some callers cannot allocate device memory when they need the solve (a host that reserves
its device memory once at start-up, a time loop that must not pay cudaFree's device-wide
synchronisation, code that holds no IbCtx).  For them the solve keeps its scratch in a
static device array.  Its results must match the oracle's ctci (myfft.F90:177-188) and the
context path's ib_ctci on the same input, call after call: the static array it shares
between calls keeps the previous call's contents, and a later call must not depend on them.
One test runs it in a fresh process before any context exists, the way such a caller would;
the others run after the rest of the suite has loaded the library and run its own kernels
(the file is named so that pytest collects it last).
"""
import ctypes as C
import os
import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest

import ib_oracle as O
from helpers import SMALL, rel
from ib_parallel_gb300 import ibgpu as G

ROOT = Path(__file__).resolve().parent.parent

TOL_OP = 1e-13   # same tolerance as the other single-transform tests
IB_ERR_ARG = 1


def _oracle_ctci(m, n, x):
    o = O.IBOracle(O.Params(m=m, n=n, mgridlev=1, dt=0.01, Re=100.0, len=8.0, offsetx=2.0, offsety=2.0), [])
    return o.ctci(x)


def _static(lib, m, n, vort_dev, s_dev, stream):
    return lib.ib_ctci_static(m, n, C.c_void_p(vort_dev.data_ptr()), C.c_void_p(s_dev.data_ptr()),
                              C.c_void_p(stream))


@pytest.mark.gpu
@pytest.mark.parametrize("m,n", [(64, 32), (120, 36)])
def test_ctci_static_matches_ctci(m, n):
    import torch

    lib = G.load()
    sim = G.Simulation(G.Params(**dict(SMALL, m=m, n=n, mgridlev=2)), [])
    rng = np.random.default_rng(7 * m + n)
    stream = torch.cuda.Stream()
    try:
        for call in range(2):   # two calls in a row, different inputs
            x = rng.standard_normal((n - 1, m - 1)) * (1.0 + 10.0 * call)
            want = sim.ctci(x)
            assert rel(want, _oracle_ctci(m, n, x)) < TOL_OP
            vort = torch.from_numpy(x).cuda()
            # the output starts as garbage, so a result left over from the previous call cannot pass
            s = torch.full_like(vort, float("nan"))
            torch.cuda.synchronize()
            rc = _static(lib, m, n, vort, s, stream.cuda_stream)
            assert rc == G.IB_OK, lib.ib_last_error().decode()
            stream.synchronize()
            got = s.cpu().numpy()
            assert np.isfinite(got).all()
            assert rel(got, want) < TOL_OP, (call, rel(got, want))
            assert rel(got, _oracle_ctci(m, n, x)) < TOL_OP
    finally:
        sim.close()


_FRESH = textwrap.dedent("""
    import ctypes as C, sys
    import numpy as np
    sys.path[:0] = [{root!r}, {oracle!r}]
    import torch
    import ib_oracle as O
    from ib_parallel_gb300 import ibgpu as G
    lib = G.load()
    m, n = 96, 48
    o = O.IBOracle(O.Params(m=m, n=n, mgridlev=1, dt=0.01, Re=100.0, len=8.0, offsetx=2.0, offsety=2.0), [])
    rng = np.random.default_rng(11)
    stream = torch.cuda.Stream()
    worst = 0.0
    for call in range(2):
        x = rng.standard_normal((n - 1, m - 1)) * (1.0 + 5.0 * call)
        vort = torch.from_numpy(x).cuda()
        s = torch.full_like(vort, float("nan"))
        torch.cuda.synchronize()
        rc = lib.ib_ctci_static(m, n, C.c_void_p(vort.data_ptr()), C.c_void_p(s.data_ptr()),
                                C.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.ib_last_error().decode()
        stream.synchronize()
        got = s.cpu().numpy()
        want = o.ctci(x)
        worst = max(worst, float(np.abs(got - want).max() / np.abs(want).max()))
    # only now a context, whose own ctci must agree with the static solve's last result
    sim = G.Simulation(G.Params(m=m, n=n, mgridlev=1, dt=0.01, Re=100.0, len=8.0, offsetx=2.0, offsety=2.0,
                                autotune=False), [])
    ctx = sim.ctci(x)
    sim.close()
    worst = max(worst, float(np.abs(got - ctx).max() / np.abs(ctx).max()))
    print("WORST", worst)
""")


@pytest.mark.gpu
def test_ctci_static_first_in_fresh_process():
    # the first call of a process that has created no context and launched no kernel of the
    # library: the set-up (symbol address, tables) happens on this call
    code = _FRESH.format(root=str(ROOT), oracle=str(ROOT / "oracle"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600,
                       env=dict(os.environ))
    assert r.returncode == 0, r.stdout + r.stderr
    worst = float(r.stdout.split("WORST")[1].split()[0])
    assert worst < TOL_OP, worst


@pytest.mark.gpu
def test_ctci_static_rejects_host_arrays():
    lib = G.load()
    m, n = 64, 32
    x = np.zeros((n - 1, m - 1))
    y = np.zeros_like(x)
    rc = lib.ib_ctci_static(m, n, x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p), None)
    assert rc == IB_ERR_ARG
    assert "device" in lib.ib_last_error().decode()


def test_ctci_static_rejects_oversized_grid():
    # checked before any CUDA call, so the dummy (never dereferenced) pointers are safe
    lib = G.load()
    dummy = C.c_void_p(0x1000)
    for m, n in [(1920, 960), (1280, 640)]:
        rc = lib.ib_ctci_static(m, n, dummy, dummy, None)
        assert rc == IB_ERR_ARG
        assert "16 MiB" in lib.ib_last_error().decode()
    rc = lib.ib_ctci_static(64, 30, dummy, dummy, None)
    assert rc == IB_ERR_ARG
