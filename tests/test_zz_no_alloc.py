"""ib_ctci_static: the context-free Poisson solve that allocates no device memory.

Its results must match the context path's ib_ctci (myfft.F90:177-188) on the same input,
call after call: the static scratch array it shares between calls keeps the previous
call's contents, and a later call must not depend on them.  The file is named so that
pytest collects it last, after the other tests have loaded the library and run their own
kernels in this process.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import SMALL, rel
from ib_parallel_gb300 import ibgpu as G

TOL_OP = 1e-13   # same tolerance as the other single-transform tests
IB_ERR_ARG = 1


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
    finally:
        sim.close()


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
