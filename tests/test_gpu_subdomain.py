"""The sub-domain precomputed-Schur method on the GPU against the oracle's restatement
(oracle/ib_subdomain.py): B column by column with the same pattern after the drop tolerance,
the FSI operator lumat = body + P B^T P^T, the sd_precomputed.chd file both ways, steps
conditional on the Krylov solve (one FSI iteration a step, the oracle handed the GPU's forces),
free-running steps, a stationary rigid body inside the cloud, and a body leaving the cloud."""
import os

import numpy as np
import pytest

import ib_oracle as O
import ib_subdomain as SD
from helpers import PLATE, SMALL, pair, rel, small_plate
from ib_parallel_gb300 import geometry as GEO
from ib_parallel_gb300 import ibgpu as G

pytestmark = pytest.mark.gpu

CLOUD = (-0.25, 1.25, -0.25, 0.25, 0.0625)   # sdxi, sdxe, sdyi, sdye, delta_sd
RIGID_CLOUD = (-0.75, 1.0, -0.625, 0.625, 0.125)


def _setup(o, g, cloud, full_rect=True):
    g.subdomain_setup(*cloud, full_rectangular=full_rect)
    o.sd = SD.SubDomain(o, full_rect, *cloud)


def _compare_matrices(sd_gpu_cols, sd_oracle):
    for j, ((rg, vg), (ro, vo)) in enumerate(zip(sd_gpu_cols, sd_oracle.cols)):
        assert np.array_equal(rg, ro), j
        assert rel(vg, vo) < 1e-11, (j, rel(vg, vo))


@pytest.fixture(scope="module")
def plate_pair(tmp_path_factory):
    o, g = pair(PLATE, [small_plate()])
    _setup(o, g, CLOUD)
    g.subdomain_precompute()
    path = tmp_path_factory.mktemp("sd") / "sd_precomputed.chd"
    g.write_subdomain_matrix(path)
    gpu = SD.SubDomain(o, True, *CLOUD)
    gpu.read_chd(path)
    return o, g, gpu, path


def test_matrix_matches_the_oracle(plate_pair):
    o, g, gpu, _ = plate_pair
    o.sd.precompute()
    _compare_matrices(gpu.cols, o.sd)
    st = g.subdomain_stats()
    assert st["unknowns"] == o.sd.nf_sd and st["columns"] == o.sd.nf_sd
    assert st["kept"] == sum(len(r) for r, _ in gpu.cols)
    assert st["candidates"] == sum(len(o.sd.rows_of(j)) for j in range(o.sd.nf_sd))


def test_operator_matches_the_oracle(plate_pair):
    o, g, gpu, _ = plate_pair
    o.sd.cols = gpu.cols                # the same thinned B on both sides
    idx, w = o.sd.interp()
    assert rel(g.subdomain_operator(), o.sd.lumat(idx, w)) < 1e-13


def test_steps_conditional_on_the_solve(plate_pair):
    _, _, gpu, path = plate_pair
    o, g = pair(dict(PLATE, fsi_tol=5.0), [small_plate()])
    _setup(o, g, CLOUD)
    g.read_subdomain_matrix(path)
    o.sd.cols = gpu.cols
    for step in range(8):
        g.advance()
        fg = g.get_vector("f")
        its, fsi = g.counters()
        assert fsi == 1
        o.gmres = lambda b, x0, op, fg=fg, its=its: (fg.copy(), its, 2)
        o.advance()
        tol = 1e-11 if step == 0 else 1e-10
        for k in range(o.L):
            assert rel(g.get_field("omega", k), o.omega[k]) < tol, (step, k)
        assert rel(g.get_vector("xb"), o.xb) < tol and rel(g.get_vector("f_rdst"), o.f_rdst) < tol
        assert abs(g.body_state()[0][0] - o.theta[0]) < tol * max(abs(o.theta[0]), 1e-12)
    g.close()


def test_free_running_steps(plate_pair):
    _, _, gpu, path = plate_pair
    o, g = pair(dict(PLATE, rtol=1e-12, fsi_tol=1e-11), [small_plate()])
    _setup(o, g, CLOUD)
    g.read_subdomain_matrix(path)
    o.sd.cols = gpu.cols
    for step in range(6):
        g.advance()
        o.advance()
        assert rel(g.get_field("omega", 0), o.omega[0]) < 1e-7, step
        assert abs(g.body_state()[0][0] - o.theta[0]) < 1e-7 * abs(o.theta[0]), step
    assert g.counters()[1] >= 2
    assert g.step_graph_stats()["graph"] >= 3   # the later steps ran the FSI loop on the device
    g.close()


def test_device_fsi_loop_matches_host_loop(plate_pair):
    # from the second step the sub-domain's FSI iterations (P at the new positions, lumat, the
    # solve, the structure update) run as the device loop inside the step's graph; with per-phase
    # timing on they run from the host: the same kernels in the same order
    _, _, _, path = plate_pair
    kw = dict(PLATE, rtol=1e-12, fsi_tol=1e-11)
    gd = G.Simulation(G.Params(**kw), [small_plate()])
    gh = G.Simulation(G.Params(**kw), [small_plate()])
    for g in (gd, gh):
        g.subdomain_setup(*CLOUD)
        g.read_subdomain_matrix(path)
    gh.step_profile(1)
    for _ in range(5):
        gd.advance()
        gh.advance()
        assert gd.counters() == gh.counters()
        assert np.array_equal(gd.get_vector("f"), gh.get_vector("f"))
        assert np.array_equal(gd.get_vector("xb"), gh.get_vector("xb"))
        assert np.array_equal(gd.body_state()[0], gh.body_state()[0])
    for k in range(PLATE["mgridlev"]):
        assert np.array_equal(gd.get_field("omega", k), gh.get_field("omega", k))
    assert gd.step_graph_stats()["graph"] >= 3 and gh.step_graph_stats()["graph"] == 0
    gd.close()
    gh.close()


def test_coarse_responses_match_the_per_column_chain(plate_pair, tmp_path):
    # the precompute's columns with the coarse levels summed from per-vertex responses against
    # the same columns with each column's own coarse chain (IB_COARSE_RESP=0)
    o, g, gpu, _ = plate_pair
    assert g.coarse_stats()["solves"] > 0
    old = os.environ.get("IB_COARSE_RESP")
    os.environ["IB_COARSE_RESP"] = "0"
    try:
        h = G.Simulation(G.Params(**PLATE), [small_plate()])
    finally:
        if old is None:
            del os.environ["IB_COARSE_RESP"]
        else:
            os.environ["IB_COARSE_RESP"] = old
    h.subdomain_setup(*CLOUD)
    h.subdomain_precompute()
    assert h.coarse_stats()["solves"] == 0
    path = tmp_path / "chain.chd"
    h.write_subdomain_matrix(path)
    chain = SD.SubDomain(o, True, *CLOUD)
    chain.read_chd(path)
    for j, ((rg, vg), (rc, vc)) in enumerate(zip(gpu.cols, chain.cols)):
        assert np.array_equal(rg, rc), j
        assert rel(vg, vc) < 1e-13, (j, rel(vg, vc))
    h.close()


def test_computed_and_read_matrices_step_alike(plate_pair):
    _, _, _, path = plate_pair
    a = G.Simulation(G.Params(**PLATE), [small_plate()])
    b = G.Simulation(G.Params(**PLATE), [small_plate()])
    a.subdomain_setup(*CLOUD)
    b.subdomain_setup(*CLOUD)
    b.read_subdomain_matrix(path)      # sub_domain_precomputed = T
    for _ in range(3):
        a.advance()
        b.advance()
    assert np.array_equal(a.get_field("omega", 0), b.get_field("omega", 0))
    assert b.subdomain_stats()["columns"] == 0 and a.subdomain_stats()["columns"] > 0
    a.close()
    b.close()


def test_rigid_body_points_lead_the_cloud():
    # a stationary cylinder whose points are the first cloud points (full_rectangular = F):
    # its unknowns take their own points' B entries exactly
    cyl = GEO.cylinder(npts=25)
    o, g = pair(dict(SMALL, fsi_tol=5.0), [cyl])
    _setup(o, g, RIGID_CLOUD, full_rect=False)
    g.subdomain_precompute()
    o.sd.precompute()
    import tempfile, os
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "sd.chd")
        g.write_subdomain_matrix(path)
        gpu = SD.SubDomain(o, False, *RIGID_CLOUD)
        gpu.read_chd(path)
    _compare_matrices(gpu.cols, o.sd)
    o.sd.cols = gpu.cols
    idx, w = o.sd.interp()
    assert (w[:, 0] == 1.0).all() and (w[:, 1:] == 0.0).all()
    assert rel(g.subdomain_operator(), o.sd.lumat(idx, w)) < 1e-13
    for step in range(3):
        g.advance()
        fg = g.get_vector("f")
        its, _ = g.counters()
        o.gmres = lambda b, x0, op, fg=fg, its=its: (fg.copy(), its, 2)
        o.advance()
        assert rel(g.get_field("omega", 0), o.omega[0]) < 1e-10, step
    g.close()


def test_setup_rejects_a_cloud_near_the_boundary():
    g = G.Simulation(G.Params(**PLATE), [small_plate()])
    with pytest.raises(G.IbError, match="within 11 cells"):
        g.subdomain_setup(-0.25, 1.25, -0.40, 0.25, 0.0625)
    g.close()


def test_a_body_leaving_the_cloud_ends_the_step_with_a_domain_error():
    # the stencils outside the cloud take its nearest cell (no access outside it); the solves are
    # capped so that the step ends quickly, and the error word reports the exit
    g = G.Simulation(G.Params(**dict(PLATE, gmres_max_it=20, fsi_max_it=1)), [small_plate()])
    g.subdomain_setup(-0.25, 0.5, -0.25, 0.25, 0.0625)   # the plate reaches x = 0.98
    with pytest.raises(G.IbError, match="IB_ERR_DOMAIN"):
        g.advance()
    g.close()


def test_full_size_columns_and_operator(tmp_path):
    # the bench's 800x400x5 plate and its 121 x 51 cloud (12342 unknowns): sampled columns of B
    # and the FSI operator lumat against the oracle
    p, bodies = GEO.config_plate_800x400()
    p.autotune = False
    cloud = GEO.subdomain_800x400()
    g = G.Simulation(p, bodies)
    g.subdomain_setup(*cloud)
    g.subdomain_precompute()
    path = tmp_path / "sd_800x400.chd"
    g.write_subdomain_matrix(path)
    po = O.Params(**{k: getattr(p, k) for k in O.Params.__dataclass_fields__ if hasattr(p, k)})
    ob = [O.Body(x=b.x.copy(), y=b.y.copy(), fam=b.fam, gamma0_deg=b.gamma0_deg, itheta=b.itheta,
                 ktheta=b.ktheta, ctheta=b.ctheta) for b in bodies]
    o = O.IBOracle(po, ob)
    sd = SD.SubDomain(o, True, *cloud)
    sd.read_chd(path)
    assert sd.nf_sd == 12342
    for j in (0, 3050, 6171 + 3050, sd.nf_sd - 1):
        rows, vals = sd.drop(j, sd.column(j))
        assert np.array_equal(rows, sd.cols[j][0]), j
        assert rel(sd.cols[j][1], vals) < 1e-11, (j, rel(sd.cols[j][1], vals))
    o.sd = sd
    idx, w = sd.interp()
    assert rel(g.subdomain_operator(), sd.lumat(idx, w)) < 1e-12
    g.close()
