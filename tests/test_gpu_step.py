"""Step-level parity of the CUDA path with the oracle (timestepper.F90:18-556).

The reference's Krylov solve (PETSc GMRES(30), classical Gram-Schmidt without
refinement) amplifies round-off: in the oracle alone a 1e-15 relative
perturbation of the Schur matvec changes the solved force by ~1e-9 after one
step of the 64x32 cylinder (iteration counts 268 vs 275).  Parity is therefore
checked three ways:
  * direct solve (num_stat, the reference's Cholesky path): everything to 1e-11;
  * conditional: the oracle takes the GPU's GMRES solution for its solve, and
    every other quantity of the step must match to 1e-11;
  * free running: both solve with their own GMRES; fields within the solver's
    round-off sensitivity (1e-6) and Krylov iteration counts within a factor 2
    (restarted GMRES with CGS reaches its tolerance after a round-off-dependent
    number of cycles).
At these small sizes the body points lie about one grid spacing apart and the Schur
operator's condition number is ~1e3-1e4, so even GMRES run to rtol 1e-14 leaves the force
1e-11 to 1e-10 away from a direct solve: the tight free-running check is made at the
benchmark size instead (tests/test_gpu_fullsize.py), where the operator is well conditioned.
"""
import numpy as np
import pytest

from helpers import PLATE, SMALL, pair, rel, small_cylinder, small_plate

pytestmark = pytest.mark.gpu


def _compare(o, g, tol, forces=True):
    worst = 0.0
    for k in range(o.L):
        for name, ref in (("omega", o.omega[k]), ("s", o.s[k]), ("qx", o.qx[k]), ("qy", o.qy[k])):
            e = rel(g.get_field(name, k), ref)
            worst = max(worst, e)
            assert e < tol, (name, k, e)
    if o.nf and forces:
        assert rel(g.get_vector("f"), o.f) < tol
        assert rel(g.get_vector("f_rdst"), o.f_rdst) < tol
        cx, cy = g.forces()
        ox, oy = o.force_coeffs(o.f)
        assert rel(np.r_[cx, cy], np.r_[ox, oy]) < tol
    return worst


def test_cylinder_direct_solve():
    kw = dict(SMALL, num_stat=True)
    o, g = pair(kw, [small_cylinder()])
    o.advance(); g.advance()
    _compare(o, g, 1e-11)
    for _ in range(9):
        o.advance(); g.advance()
    _compare(o, g, 1e-9)
    g.close()


def test_cylinder_conditional_on_solve():
    o, g = pair(SMALL, [small_cylinder()])
    for step in range(10):
        g.advance()
        fg = g.get_vector("f")
        its_g, _ = g.counters()
        o.gmres = lambda b, x0, op, fg=fg, its=its_g: (fg.copy(), its, 2)
        o.advance()
        tol = 1e-11 if step == 0 else 1e-10
        _compare(o, g, tol)
    g.close()


def test_cylinder_free_running():
    o, g = pair(SMALL, [small_cylinder()])
    for step in range(5):
        o.advance(); g.advance()
        kg, _ = g.counters()
        assert 0.5 <= kg / o.ksp_iter <= 2.0, (kg, o.ksp_iter)
    _compare(o, g, 1e-6)
    g.close()


def test_plate_fsi_steps():
    o, g = pair(PLATE, [small_plate()])
    for step in range(3):
        o.advance(); g.advance()
        th, _, _ = g.body_state()
        assert rel(th, o.theta) < 1e-7
        _, fsi = g.counters()
        assert fsi == o.fsi_iter
    _compare(o, g, 1e-6)
    xb = g.get_vector("xb")
    assert rel(xb, o.xb) < 1e-9
    g.close()


def test_plate_conditional_on_solve():
    # one FSI iteration a step (fsi_tol above any error), the oracle handed the GPU's solve:
    # structure right-hand side, regT, redistribution, compute_dx, the new weights and the
    # correction with the moved stencils must all match
    o, g = pair(dict(PLATE, fsi_tol=5.0), [small_plate()])
    for step in range(10):
        g.advance()
        fg = g.get_vector("f")
        its_g, fsi = g.counters()
        assert fsi == 1
        o.gmres = lambda b, x0, op, fg=fg, its=its_g: (fg.copy(), its, 2)
        o.advance()
        tol = 1e-11 if step == 0 else 1e-10
        _compare(o, g, tol)
        th, _, _ = g.body_state()
        assert rel(th, o.theta) < tol
        assert rel(g.get_vector("xb"), o.xb) < tol
    g.close()



@pytest.mark.parametrize("L", [2, 3])
def test_coarse_levels_beside_the_finer_grid(L):
    # a coarse grid spacing puts vorticity on the coarser levels beside the finer grid (their
    # centre rows outside the centre columns, which coarsify does not rewrite) within a few
    # steps, and over 60 steps the wake leaves the finest grid downstream: those points are the
    # predictor's on every level, as the oracle's
    from ib_parallel_gb300 import ibgpu as G
    import ib_oracle as O
    kw = dict(m=32, n=16, mgridlev=L, dt=0.05, Re=100.0, len=4.0, offsetx=1.0, offsety=1.0, num_stat=True,
              autotune=False)
    cyl = O.cylinder(npts=10, diameter=0.8, xc=0.3, yc=0.0)
    o, g = pair(kw, [G.Body(x=cyl.x.copy(), y=cyl.y.copy(), fam=1)])
    n, m = kw["n"], kw["m"]
    for step in range(60):
        o.advance()
        g.advance()
        if step in (1, 59):
            for k in range(L):
                assert rel(g.get_field("omega", k), o.omega[k]) < 1e-10, (step, k)
    beside = o.omega[1][n // 4: 3 * n // 4 - 1, 3 * m // 4 - 1:]
    assert np.abs(beside).max() > 1e-3 * np.abs(o.omega[1]).max()   # the wake has reached them
    g.close()
