"""The whole step as one CUDA graph against the same step run phase by phase.

From the second step on, ib_advance launches one graph: the predictor, the first vort2flux,
the forces (the device FSI loop, the direct solve, or nothing without bodies) and the
correction, which in the FSI case sits under an if node that a gate kernel opens when the host
loop of timestepper.F90:318 would add no iteration.  IB_WHOLE_STEP=0 runs the same kernels
phase by phase with a host readback between the FSI loop and the correction.  No kernel
accumulates in floating point atomically, so both runs agree bit for bit: fields, forces,
positions, structure state and counters, including steps whose device loop leaves the
influence band with iterations still to run (the gate leaves the loop and the correction to
the host) and steps stopped by the FSI cap.
"""
import os

import numpy as np
import pytest

from helpers import PLATE, SMALL, small_cylinder, small_plate
from ib_parallel_gb300 import geometry as GEO
from ib_parallel_gb300 import ibgpu as G

pytestmark = pytest.mark.gpu


def _make(params, bodies, whole):
    old = os.environ.get("IB_WHOLE_STEP")
    os.environ["IB_WHOLE_STEP"] = "1" if whole else "0"
    try:
        return G.Simulation(params if isinstance(params, G.Params) else G.Params(**params), bodies)
    finally:
        if old is None:
            del os.environ["IB_WHOLE_STEP"]
        else:
            os.environ["IB_WHOLE_STEP"] = old


def _state(g, levels):
    out = {}
    for k in range(levels):
        out[f"omega{k}"] = g.get_field("omega", k)
        out[f"s{k}"] = g.get_field("s", k)
    for name in ("qx", "qy", "rhs_old"):
        out[name] = g.get_field(name, 0)
    if g.nf:
        for name in ("f", "f_rdst", "xb", "yb"):
            out[name] = g.get_vector(name)
        out["forces"] = np.concatenate(g.forces())
    if g.ntors:
        out["body"] = np.concatenate(g.body_state())
    out["counters"] = np.array(g.counters(), dtype=np.float64)
    return out


def _run_pair(params, bodies, steps, expect_rc=G.IB_OK):
    a = _make(params, bodies, True)
    b = _make(params, bodies, False)
    for step in range(steps):
        ra = a.lib.ib_advance(a.h, None)
        rb = b.lib.ib_advance(b.h, None)
        assert ra == rb and ra in (G.IB_OK, expect_rc), (step, ra, rb)
        levels = a.params.mgridlev
        sa, sb = _state(a, levels), _state(b, levels)
        for key in sa:
            assert np.array_equal(sa[key], sb[key]), (step, key, np.abs(sa[key] - sb[key]).max())
    stats_a, stats_b = a.step_graph_stats(), b.step_graph_stats()
    assert stats_b["graph"] == 0 and stats_b["phased"] == steps
    a.close()
    b.close()
    return stats_a


def test_plate_device_loop_steps_as_one_graph():
    stats = _run_pair(PLATE, [small_plate()], 8)
    # step 1 builds the influence band from the host; every later step is one graph
    assert stats == {"graph": 7, "gate_closed": 0, "phased": 1}, stats


def test_plate_band_exits_leave_the_loop_to_the_host():
    # a light plate released at 45 degrees incidence swings towards the flow (about 0.6 rad in
    # the first 50 steps of dt = 0.02); with one vertex of slack around the stencils its
    # patches leave the influence band mid-loop within the first dozen steps: the gate keeps
    # the correction for the host, which rebuilds the band and finishes the loop, and the next
    # step captures a new whole-step graph on the new band
    plate = GEO.torsional_plate(npts=17, length=1.0, gamma0_deg=-45.0, itheta=0.05, ktheta=0.0)
    stats = _run_pair(dict(PLATE, influence_margin=1, dt=0.02), [plate], 30)
    assert stats["graph"] >= 20 and stats["gate_closed"] >= 1, stats


def test_plate_fsi_cap_in_one_graph():
    # the loop stops at fsi_max_it + 1 iterations: the gate opens, the step reports IB_ERR_FSI
    stats = _run_pair(dict(PLATE, fsi_max_it=1), [small_plate()], 4, expect_rc=5)
    assert stats["graph"] == 3 and stats["gate_closed"] == 0, stats


def test_direct_solve_steps_as_one_graph():
    stats = _run_pair(dict(SMALL, num_stat=True), [small_cylinder()], 6)
    assert stats == {"graph": 5, "gate_closed": 0, "phased": 1}, stats


def test_no_body_steps_as_one_graph():
    stats = _run_pair(SMALL, [], 5)
    assert stats["graph"] == 4 and stats["phased"] == 1, stats


def test_full_size_plate_as_one_graph():
    p, bodies = GEO.config_plate_800x400()
    p.autotune = False   # the same launch shapes in both contexts
    stats = _run_pair(p, bodies, 4)
    assert stats["graph"] == 3, stats
