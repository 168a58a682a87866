"""Euler-Bernoulli beams (body family 3) on the GPU against the oracle's formulation: the
structure operators one by one, steps conditional on the Krylov solve (one FSI iteration a step,
the oracle handed the GPU's solution), steps through the assembled operator against steps
through the matrix-free one, and the 800x400x5 flexible plate with both solvers run tight."""
import numpy as np
import pytest

import ib_oracle as O
from helpers import PLATE, pair, rel
from ib_parallel_gb300 import geometry as GEO
from ib_parallel_gb300 import ibgpu as G

pytestmark = pytest.mark.gpu


def _beam():
    return GEO.beam_plate(9, 1.0, 10.0, 0.5, 1e-2)


def test_beam_operators():
    o, g = pair(PLATE, [_beam()])
    rng = np.random.default_rng(4)
    bm = o.beams[0]
    for _ in range(2):
        f = 1e-2 * rng.standard_normal(o.nf)
        x = rng.standard_normal(o.nf)
        assert rel(g.struct_btimes(x), o.b_times(x)) < 1e-13
        err_o = o.compute_dx(f)
        o.setup_reg()   # ib_struct_dx rebuilds the weights at the new positions as well
        err_g = g.struct_dx(f)
        assert abs(err_g - err_o) <= 1e-12 * err_o
        q, qd, qdd = g.beam_state()
        assert rel(q, bm.q) < 1e-12 and rel(qd, bm.qd) < 1e-12 and rel(qdd, bm.qdd) < 1e-12
        assert rel(g.get_vector("xb"), o.xb) < 1e-14 and rel(g.get_vector("yb"), o.yb) < 1e-14
        # with q0 = 0 (no step has saved the state) compute_rhs cancels to zero in exact
        # arithmetic: compare against the size of its terms, delta (2/dt) |q|
        scale = o.delta * 2.0 / PLATE["dt"] * np.abs(bm.q).max()
        assert np.abs(g.struct_rhs() - o.compute_rhs()).max() < 1e-12 * scale
        assert rel(g.schur_apply(x), o.a_times(x)) < 1e-12
    g.close()


def test_beam_conditional_on_solve():
    o, g = pair(dict(PLATE, fsi_tol=5.0), [_beam()])
    for step in range(10):
        g.advance()
        fg = g.get_vector("f")
        its, fsi = g.counters()
        assert fsi == 1
        o.gmres = lambda b, x0, op, fg=fg, its=its: (fg.copy(), its, 2)
        o.advance()
        tol = 1e-11 if step == 0 else 1e-10
        for k in range(o.L):
            assert rel(g.get_field("omega", k), o.omega[k]) < tol, (step, k)
        assert rel(g.beam_state()[0], o.beams[0].q) < tol
        assert rel(g.get_vector("xb"), o.xb) < tol and rel(g.get_vector("f_rdst"), o.f_rdst) < tol
    g.close()


def test_beam_assembled_matches_matrix_free():
    gi = G.Simulation(G.Params(**PLATE), [_beam()])
    gm = G.Simulation(G.Params(**dict(PLATE, schur_mode=1)), [_beam()])
    for _ in range(4):
        gi.advance()
        gm.advance()
        assert gi.counters()[1] == gm.counters()[1]
        assert rel(gi.beam_state()[0], gm.beam_state()[0]) < 1e-8
    assert gi.influence_stats()["assemblies"] >= 4
    gi.close()
    gm.close()


def test_beam_plate800x400_tight():
    from test_gpu_fullsize import _compare, _pair
    import scipy.fft as sfft
    import os
    p, bodies = GEO.config_beam_800x400()
    o, g = _pair(p, bodies, rtol=1e-14, atol=1e-16, fsi_tol=1e-12)
    with sfft.set_workers(os.cpu_count() or 1):
        for step in range(2):
            o.advance()
            g.advance()
            assert g.counters()[1] == o.fsi_iter
            _compare(o, g, 1e-11 if step == 0 else 1e-10)
            assert rel(g.beam_state()[0], o.beams[0].q) < (1e-11 if step == 0 else 1e-10)
    g.close()
