"""Influence-matrix form of the Schur operator (a_times2, operators_fluid.F90:14-120).

The assembled fluid matrix S_f = P^T K P must equal the matrix-free operator column by
column (the same linear map evaluated in another order: round-off only) and the oracle's
a_times on unit vectors; steps through the assembled operator must match steps through the
matrix-free one; moving the stencils out of the band rebuilds it; stencils that touch the
domain boundary fall back to the matrix-free operator.
"""
import os

import numpy as np
import pytest

from helpers import PLATE, SMALL, pair, rel, small_cylinder, small_plate
from ib_parallel_gb300 import ibgpu as G

pytestmark = pytest.mark.gpu

TOL_MAT = 1e-11   # assembled vs matrix-free operator (FP64 round-off of ~50-term sums)


def _without_coarse_responses(make):
    old = os.environ.get("IB_COARSE_RESP")
    os.environ["IB_COARSE_RESP"] = "0"
    try:
        return make()
    finally:
        if old is None:
            del os.environ["IB_COARSE_RESP"]
        else:
            os.environ["IB_COARSE_RESP"] = old


def _matrix_free(g):
    eye = np.eye(g.nf)
    return np.stack([g.schur_apply(eye[l], with_b=False) for l in range(g.nf)], axis=1)


@pytest.mark.parametrize("case", ["cylinder", "plate"])
def test_assembled_matches_matrix_free_and_oracle(case):
    kw, body = (SMALL, small_cylinder()) if case == "cylinder" else (PLATE, small_plate())
    o, g = pair(kw, [body])
    S = g.schur_matrix()
    assert S is not None
    assert rel(S, _matrix_free(g)) < TOL_MAT
    eye = np.eye(o.nf)
    So = np.stack([o.a_times(eye[l], with_b=False) for l in range(o.nf)], axis=1)
    assert rel(S, So) < TOL_MAT
    st = g.influence_stats()
    assert st["builds"] == 1 and st["band_vertices"] % 64 == 0 and st["fallbacks"] == 0
    g.close()


def test_steps_match_matrix_free():
    body = small_plate()
    gi = G.Simulation(G.Params(**PLATE), [body])
    gm = G.Simulation(G.Params(**dict(PLATE, schur_mode=1)), [body])
    for _ in range(4):
        gi.advance()
        gm.advance()
        ti, _, _ = gi.body_state()
        tm, _, _ = gm.body_state()
        assert rel(ti, tm) < 1e-8
        assert gi.counters()[1] == gm.counters()[1]
    for k in range(PLATE["mgridlev"]):
        assert rel(gi.get_field("omega", k), gm.get_field("omega", k)) < 1e-7
    assert rel(gi.get_vector("f"), gm.get_vector("f")) < 1e-7
    st = gi.influence_stats()
    assert st["builds"] == 1 and st["assemblies"] >= 4
    assert gm.influence_stats()["assemblies"] == 0
    gi.close()
    gm.close()


def test_fused_solver_matches_graph_solver():
    # the one-kernel GMRES performs the graph solver's operations in the same order
    body = small_plate()
    gf = G.Simulation(G.Params(**PLATE), [body])
    gg = G.Simulation(G.Params(**dict(PLATE, schur_mode=2)), [body])
    for _ in range(3):
        gf.advance()
        gg.advance()
        assert gf.counters() == gg.counters()
        assert np.array_equal(gf.get_vector("f"), gg.get_vector("f"))
        assert np.array_equal(gf.body_state()[0], gg.body_state()[0])
    assert np.array_equal(gf.get_field("omega", 0), gg.get_field("omega", 0))
    gf.close()
    gg.close()


def test_band_rebuild_after_move():
    o, g = pair(dict(PLATE, influence_margin=2), [small_plate()])
    assert g.schur_matrix() is not None
    d = PLATE["len"] / PLATE["m"]
    xb = g.get_vector("xb") + 12.0 * d      # beyond margin + tile slack (<= 2 + 7): patches leave the band
    yb = g.get_vector("yb") + 3.0 * d
    G._check(g.lib.ib_reg_prep(g.h, G._ptr(xb), G._ptr(yb)), "ib_reg_prep")
    S = g.schur_matrix()
    assert S is not None
    assert g.influence_stats()["builds"] == 2
    assert rel(S, _matrix_free(g)) < TOL_MAT
    g.close()


def test_boundary_stencils_fall_back():
    o, g = pair(PLATE, [small_plate()])
    d = PLATE["len"] / PLATE["m"]
    xb = g.get_vector("xb")
    yb = g.get_vector("yb")
    # leftmost stencil origin at face index 4: inside the grid, but its vertex patch reaches
    # the boundary column (streamfunction from the ring)
    shift = (3.0 + 0.25) * d - PLATE["offsetx"] - xb.min()
    G._check(g.lib.ib_reg_prep(g.h, G._ptr(xb + shift), G._ptr(yb)), "ib_reg_prep")
    assert g.schur_matrix() is None
    assert g.influence_stats()["fallbacks"] >= 1
    g.close()


def test_device_fsi_loop_matches_host_loop():
    # the FSI iterations run as one graph with a device-side loop condition; with per-phase
    # timing on they run from the host, one launch per kernel: the same kernels in the same order
    body = small_plate()
    gd = G.Simulation(G.Params(**PLATE), [body])
    gh = G.Simulation(G.Params(**PLATE), [body])
    gh.step_profile(1)
    for _ in range(4):
        gd.advance()
        gh.advance()
        assert gd.counters() == gh.counters()
        assert np.array_equal(gd.get_vector("f"), gh.get_vector("f"))
        assert np.array_equal(gd.body_state()[0], gh.body_state()[0])
    for k in range(PLATE["mgridlev"]):
        assert np.array_equal(gd.get_field("omega", k), gh.get_field("omega", k))
    assert gd.influence_stats()["assemblies"] == gh.influence_stats()["assemblies"]
    gd.close()
    gh.close()


def test_schur_with_points_on_grid_lines():
    # 400x200 on [-1,7]x[-2,2] (delta = 0.02): the plate's hinge at the origin lies on a grid
    # line in x and in y, so its outermost stencil points sit exactly 3 cells away, where the
    # reference's delta function has a ~1e-8 step; the operator must still match the oracle's
    from ib_parallel_gb300 import geometry as GEO
    kw = dict(m=400, n=200, mgridlev=1, dt=1e-3, Re=500.0, len=8.0, offsetx=1.0, offsety=2.0, autotune=False)
    o, g = pair(kw, [GEO.torsional_plate(51, 1.0, -10.0)])
    rng = np.random.default_rng(9)
    x = rng.standard_normal(o.nf)
    assert rel(g.schur_apply(x, with_b=False), o.a_times(x, with_b=False)) < 1e-12
    assert rel(g.schur_apply(x), o.a_times(x)) < 1e-12
    S = g.schur_matrix()
    assert S is not None
    So = np.stack([o.a_times(e, with_b=False) for e in np.eye(o.nf)], axis=1)
    assert rel(S, So) < TOL_MAT
    g.close()


def test_coarse_responses_match_the_per_column_chain():
    # the band's columns with the coarse levels summed from per-vertex responses against the same
    # columns with each column's own coarse chain (IB_COARSE_RESP=0): round-off apart; a rebuild
    # around moved stencils solves only the vertices it has no response for yet
    body = small_plate()
    a = G.Simulation(G.Params(**dict(PLATE, influence_margin=2)), [body])
    b = _without_coarse_responses(lambda: G.Simulation(G.Params(**dict(PLATE, influence_margin=2)), [body]))
    Sa, Sb = a.schur_matrix(), b.schur_matrix()
    assert Sa is not None and Sb is not None
    assert rel(Sa, Sb) < 1e-13
    assert rel(Sa, _matrix_free(a)) < TOL_MAT
    ca, cb = a.coarse_stats(), b.coarse_stats()
    assert ca["enabled"] and ca["solves"] > 0 and ca["held"] == ca["solves"] and ca["bytes"] > 0
    assert not cb["enabled"] and cb["solves"] == 0
    d = PLATE["len"] / PLATE["m"]
    for g in (a, b):
        xb = g.get_vector("xb") + 12.0 * d
        yb = g.get_vector("yb") + 3.0 * d
        G._check(g.lib.ib_reg_prep(g.h, G._ptr(xb), G._ptr(yb)), "ib_reg_prep")
    Sa, Sb = a.schur_matrix(), b.schur_matrix()
    assert a.influence_stats()["builds"] == 2 and b.influence_stats()["builds"] == 2
    assert rel(Sa, Sb) < 1e-13
    ca2 = a.coarse_stats()
    assert ca["solves"] < ca2["solves"] < 2 * ca["solves"] and ca2["held"] == ca2["solves"]
    a.close()
    b.close()


@pytest.mark.parametrize("levels", [2, 4])
def test_coarse_responses_at_other_level_counts(levels):
    # two levels (the coarsest level's responses alone) and four (two levels of sums between)
    body = small_plate()
    kw = dict(PLATE, mgridlev=levels)
    a = G.Simulation(G.Params(**kw), [body])
    b = _without_coarse_responses(lambda: G.Simulation(G.Params(**kw), [body]))
    Sa, Sb = a.schur_matrix(), b.schur_matrix()
    assert Sa is not None and Sb is not None
    assert rel(Sa, _matrix_free(a)) < TOL_MAT
    assert rel(Sa, Sb) < 1e-13
    assert a.coarse_stats()["solves"] > 0
    a.close()
    b.close()
