"""Seeded body geometries and the benchmark configurations.

The reference builds its ``input/body.NNN.inp`` files with MATLAB scripts
(``input/cylinder/build_cylinder.m``, ``input/*/build_plate.m``,
``input/airfoil*/naca00_ibfm.m``); these functions restate the shapes.
"""
from __future__ import annotations

import math

import numpy as np

from .ibgpu import Body, Params

PI = 4.0 * math.atan(1.0)


def cylinder(npts: int = 157, diameter: float = 1.0, xc: float = 0.0, yc: float = 0.0) -> Body:
    th = 2.0 * PI * np.arange(npts) / npts
    return Body(x=xc + 0.5 * diameter * np.cos(th), y=yc + 0.5 * diameter * np.sin(th), fam=1)


def torsional_plate(npts: int = 201, length: float = 1.0, gamma0_deg: float = -10.0,
                    itheta: float = 0.5 / 3.0, ktheta: float = 1e-3, ctheta: float = 0.0,
                    x0: float = 0.0, y0: float = 0.0) -> Body:
    """Flat plate hinged at (x0, y0) on a torsional spring (family 2)."""
    g = gamma0_deg * PI / 180.0
    j = np.arange(npts, dtype=np.float64)
    ds = length / (npts - 1)
    return Body(x=x0 + j * ds * math.cos(g), y=y0 + j * ds * math.sin(g), fam=2, gamma0_deg=gamma0_deg,
                itheta=itheta, ktheta=ktheta, ctheta=ctheta)


def beam_plate(npts: int = 51, length: float = 1.0, incidence_deg: float = 10.0, mass_ratio: float = 0.5,
               stiffness: float = 1e-3, nelem: int = 0, x0: float = 0.0, y0: float = 0.0) -> Body:
    """Flexible plate (family 3: Euler-Bernoulli beam) clamped at (x0, y0), nose-down incidence."""
    g = -math.radians(incidence_deg)
    j = np.arange(npts, dtype=np.float64)
    ds = length / (npts - 1)
    return Body(x=x0 + j * ds * math.cos(g), y=y0 + j * ds * math.sin(g), fam=3, itheta=mass_ratio,
                ktheta=stiffness, nelem=nelem)


def config_beam_800x400(npts: int = 51) -> tuple:
    """BASELINE's flexible plate as a beam: length 1 at 10 degrees, mass ratio 0.5, bending
    stiffness 0.001, Re=500, 800x400 on [-1,7]x[-2,2], 5 levels, dt=1e-3, tolerances 1e-10;
    51 points two grid spacings apart (25 elements) instead of 201 (half a spacing, where the
    Schur operator is singular), no seeded tip perturbation (the beam starts straight)."""
    p = Params(m=800, n=400, mgridlev=5, dt=1e-3, Re=500.0, len=8.0, offsetx=1.0, offsety=2.0,
               fsi_tol=1e-10, atol=1e-10, rtol=1e-10)
    return p, [beam_plate(npts, 1.0, 10.0, 0.5, 1e-3)]


def config_cylinder_400x200() -> tuple:
    """Rigid cylinder, Re=100, 400x200 on [-2,6]x[-2,2], 3 levels, dt=0.004, 157 points."""
    p = Params(m=400, n=200, mgridlev=3, dt=0.004, Re=100.0, len=8.0, offsetx=2.0, offsety=2.0,
               fsi_tol=1e-10, atol=1e-10, rtol=1e-10)
    return p, [cylinder(157)]


def config_plate_800x400(seed: int = 0, npts: int = 51) -> tuple:
    """Hinged flat plate (torsional analogue of the flexible plate): length 1, 10 degrees
    incidence with a seeded 0.01 tip perturbation, Re=500, 800x400 on [-1,7]x[-2,2],
    5 levels, dt=1e-3, GMRES and FSI tolerance 1e-10.

    51 body points put the Lagrangian spacing at twice the grid spacing, the spacing the
    reference's own inputs use.  At one or half a grid spacing (101 or 201 points) the
    Schur operator is close to singular and GMRES(30) with classical Gram-Schmidt does not
    reach 1e-10 (2000 iterations without convergence on the half-size grid), so the FSI
    loop of timestepper.F90:318 never terminates."""
    rng = np.random.default_rng(seed)
    tip = 0.01 * rng.standard_normal()
    gamma0 = -10.0 + math.degrees(math.asin(max(-1.0, min(1.0, tip))))
    p = Params(m=800, n=400, mgridlev=5, dt=1e-3, Re=500.0, len=8.0, offsetx=1.0, offsety=2.0,
               fsi_tol=1e-10, atol=1e-10, rtol=1e-10)
    return p, [torsional_plate(npts, 1.0, gamma0, itheta=0.5 / 3.0, ktheta=1e-3)]


def config_pitching_600x300(ds_cells: float = 2.0) -> tuple:
    """The adjoint workload: a rigid NACA 0012 of chord 1 held in its own frame (leading edge at the
    origin, pitching about the quarter chord, the frame's centre), Re=200, 600x300 on
    [-1.5,4.5]x[-1.5,1.5], 4 levels, dt=0.002, the direct solve.  Its points are ds_cells grid
    spacings apart (2: 101 points): at 250 points (0.8 spacings) the Schur matrix is singular to
    working precision, as for the plate (tests/test_conditioning_cpu.py)."""
    p = Params(m=600, n=300, mgridlev=4, dt=0.002, Re=200.0, len=6.0, offsetx=1.5, offsety=1.5, num_stat=True,
               motion=(-1.0, 0.0, 0.0, 0.25, 0.0))
    x, y = naca00(12.0, ds=ds_cells * p.len / p.m)
    return p, [Body(x=x, y=y, fam=1)]


def subdomain_800x400() -> tuple:
    """The sub-domain cloud of the 800x400 plate (sub_domain = T, fully rectangular): the
    rectangle [-0.1, 1.1] x [-0.35, 0.15] around the plate's swept region at the grid spacing
    0.01, 121 x 51 points (12342 unknowns).  Returns (sdxi, sdxe, sdyi, sdye, delta_sd)."""
    return (-0.1, 1.1, -0.35, 0.15, 0.01)


# ---------------------------------------------------------------------------------------------
# The reference's input files (input/ib.inp, input/body.NNN.inp), read through the library's C
# ABI (ib_read_namelist, ib_read_body, ib_count_bodies) and written in the same layout.
# ---------------------------------------------------------------------------------------------
RUN_CONTROL_KEYS = ("istart", "istop", "isave", "irestart", "compute_pressure", "dimen", "motion_prescribed",
                    "sub_domain", "sub_domain_full_rectangular", "sub_domain_precomputed", "sdxi", "sdxe", "sdyi",
                    "sdye", "delta_sd")


def read_namelist(path, params: Params = None) -> tuple:
    """input (parameters.F90:51-78): the &read_parameters group of the file at path.  Returns the
    Params (items absent from the file keep params' values) and the run-control items."""
    import ctypes as C
    import dataclasses
    import os

    from . import ibgpu as G
    base = params if params is not None else Params(m=0, n=0, mgridlev=0, dt=0.0, Re=0.0, len=0.0, offsetx=0.0,
                                                    offsety=0.0)
    cp = base.to_c()
    rc = G.IbRunControl()
    G._check(G.load().ib_read_namelist(os.fsencode(path), C.byref(cp), C.byref(rc)), "ib_read_namelist")
    out = dataclasses.replace(base, m=cp.m, n=cp.n, mgridlev=cp.mgridlev, dt=cp.dt, Re=cp.Re, len=cp.len,
                              offsetx=cp.offsetx, offsety=cp.offsety, fsi_tol=cp.fsi_tol, atol=cp.atol,
                              rtol=cp.rtol, num_stat=bool(cp.num_stat))
    return out, {k: getattr(rc, k) for k in RUN_CONTROL_KEYS}


def read_body_file(path) -> Body:
    """One input/body.NNN.inp (grid.F90:252-288)."""
    import ctypes as C
    import os

    from . import ibgpu as G
    lib = G.load()
    b = G.IbBody()
    cap = 0
    x = y = np.zeros(1)
    for _ in range(2):   # the first call reports the point count when the arrays are too small
        rc = lib.ib_read_body(os.fsencode(path), C.byref(b), x.ctypes.data_as(C.POINTER(C.c_double)),
                              y.ctypes.data_as(C.POINTER(C.c_double)), cap)
        if rc == G.IB_OK:
            break
        if b.npts > cap:
            cap = b.npts
            x, y = np.zeros(cap), np.zeros(cap)
            continue
        G._check(rc, "ib_read_body")
    G._check(rc, "ib_read_body")
    return Body(x=x[:b.npts].copy(), y=y[:b.npts].copy(), fam=b.fam, gamma0_deg=b.gamma0_deg,
                alpha0_deg=b.alpha0_deg, itheta=b.itheta, ktheta=b.ktheta, ctheta=b.ctheta, nelem=b.nelem)


def load_input(directory) -> tuple:
    """The run an input directory describes (ib.inp and body.001.inp, body.002.inp, ...)."""
    import ctypes as C
    import os
    from pathlib import Path

    from . import ibgpu as G
    d = Path(directory)
    params, rc = read_namelist(d / "ib.inp")
    n = C.c_int(0)
    G._check(G.load().ib_count_bodies(os.fsencode(d), C.byref(n)), "ib_count_bodies")
    return params, rc, [read_body_file(d / f"body.{i + 1:03d}.inp") for i in range(n.value)]


def write_body_file(path, body: Body) -> None:
    """A body file in the layout grid.F90:252-288 reads (as input/*/build_*.m write it)."""
    lines = [f"{body.npts:<6d} ", f"{int(body.fam):<6d} "]
    if body.fam == 2:
        lines += [f"{v:.16f}" for v in (body.gamma0_deg, body.alpha0_deg, body.itheta, body.ktheta, body.ctheta)]
    elif body.fam == 3:
        lines += [repr(float(body.itheta)), repr(float(body.ktheta)), str(int(body.nelem))]
    lines += [f"{xv:<20.16f} {yv:<20.16f}" for xv, yv in zip(body.x, body.y)]
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def write_namelist(path, params: Params, run_control: dict = None) -> None:
    """An input/ib.inp for params (and the run-control items given)."""
    def fmt(v):
        if isinstance(v, bool):
            return "T" if v else "F"
        if isinstance(v, int):
            return str(v)
        return repr(float(v))
    items = dict(M=params.m, N=params.n, DT=params.dt, Re=params.Re, FSI_TOL=params.fsi_tol, ATOL=params.atol,
                 RTOL=params.rtol, LEN=params.len, OFFSETX=params.offsetx, OFFSETY=params.offsety,
                 MGRIDLEV=params.mgridlev, num_stat=bool(params.num_stat))
    for k, v in (run_control or {}).items():
        items[k.upper()] = bool(v) if k in ("compute_pressure", "motion_prescribed", "sub_domain",
                                            "sub_domain_full_rectangular", "sub_domain_precomputed") else v
    with open(path, "w") as fh:
        fh.write("&READ_PARAMETERS\n" + "".join(f"{k} = {fmt(v)},\n" for k, v in items.items()) + "/\n")


# ---------------------------------------------------------------------------------------------
# NACA 00XX airfoil with points a fixed distance apart (the method of input/airfoil*/
# naca00_ibfm.m, restated): the half-thickness 5 t c (0.2969 sqrt(x/c) - 0.1260 (x/c)
# - 0.3516 (x/c)^2 + 0.2843 (x/c)^3 - 0.1036 (x/c)^4) -- the last coefficient closes the
# trailing edge -- is walked from the point where it equals ds/2 (so the two leading-edge points
# are ds apart) in steps of straight-line distance ds, stopping where the surface, past
# mid-chord, comes within ds/2 of the centreline; the lower surface mirrors the upper.  The
# nominal chord is grown until the last kept point sits at the requested chord.  Points run
# from the trailing edge over the upper surface to the leading edge and back along the lower
# surface, then are rotated by the angle of attack (nose up for alpha > 0).
# ---------------------------------------------------------------------------------------------
def _naca_upper(t: float, c: float, ds: float) -> np.ndarray:
    a = 5.0 * t * c * np.array([0.2969, -0.1260, -0.3516, 0.2843, -0.1036])

    def ubd(x):
        u = max(x, 0.0) / c
        return a[0] * math.sqrt(u) + a[1] * u + a[2] * u * u + a[3] * u ** 3 + a[4] * u ** 4

    def root(fn, lo, hi):
        flo = fn(lo)
        for _ in range(80):
            mid = 0.5 * (lo + hi)
            fm = fn(mid)
            if (fm > 0) == (flo > 0):
                lo, flo = mid, fm
            else:
                hi = mid
            if hi - lo < 1e-15 * max(1.0, abs(hi)):
                break
        return 0.5 * (lo + hi)

    x0 = root(lambda x: ubd(x) - ds / 2, 1e-300, ds)
    pts = [(x0, ubd(x0))]
    while True:
        xp, yp = pts[-1]
        if xp > 0.5 * c and yp < ds / 2:
            pts.pop()   # the point that crossed into the trailing-edge gap is dropped
            break
        if xp >= c:
            break
        xn = root(lambda x: (x - xp) ** 2 + (ubd(x) - yp) ** 2 - ds * ds, xp, min(xp + ds, c))
        pts.append((xn, ubd(xn)))
    return np.array(pts)


def naca00(thickness_pct: float = 12.0, ds: float = 0.01, chord: float = 1.0, alpha_deg: float = 0.0,
           xc: float = 0.0, yc: float = 0.0) -> tuple:
    """x, y of a NACA 00XX airfoil (leading edge at (xc, yc) before rotation about it)."""
    t = min(abs(thickness_pct), 100.0) / 100.0
    # the trailing-edge cut moves in steps of about ds as the nominal chord grows: scan nominal
    # chords up to 10% longer and keep the one whose last point lies closest to `chord`
    best = None
    for i in range(101):
        c = chord * (1.0 + 0.001 * i)
        cand = _naca_upper(t, c, ds)
        err = abs(chord - cand[-1, 0])
        if best is None or err < best[0]:
            best = (err, cand)
    up = best[1]
    xs = np.r_[up[::-1, 0], up[:, 0]]
    ys = np.r_[up[::-1, 1], -up[:, 1]]
    al = math.radians(alpha_deg)
    xr = math.cos(al) * xs + math.sin(al) * ys
    yr = -math.sin(al) * xs + math.cos(al) * ys
    return xc + xr, yc + yr


def pitching_motion(x_ref: np.ndarray, y_ref: np.ndarray, t: float, amp_deg: float, freq: float, phase: float = 0.0,
                    pivot=(0.25, 0.0)) -> tuple:
    """A rigid body pitching about `pivot` as alpha(t) = A sin(2 pi f t + phi) (nose up for
    alpha > 0): positions and velocities of its points at time t, in the layout of the
    body-point vectors (x-unknowns then y-unknowns, each holding every point).  Set them as
    IB_VEC_XB, IB_VEC_YB and IB_VEC_UB before each step (the prescribed-motion hooks of
    user.F90:87-174)."""
    w = 2.0 * math.pi * freq
    al = math.radians(amp_deg) * math.sin(w * t + phase)
    ald = math.radians(amp_deg) * w * math.cos(w * t + phase)
    dx, dy = x_ref - pivot[0], y_ref - pivot[1]
    ca, sa = math.cos(al), math.sin(al)
    px = pivot[0] + ca * dx + sa * dy
    py = pivot[1] - sa * dx + ca * dy
    # d/dt of the rotation: (-sa dx + ca dy, -ca dx - sa dy) alpha'
    ux = ald * (-sa * dx + ca * dy)
    uy = ald * (-ca * dx - sa * dy)
    xb = np.r_[px, px]
    yb = np.r_[py, py]
    ub = np.r_[ux, uy]
    return xb, yb, ub


def config_ensemble(nsim: int = 256, seed0: int = 0) -> list:
    """The batched-ensemble workload: nsim independent hinged-plate simulations, simulation s
    drawing from default_rng(seed0 + s): Re uniform in [100, 500], mass ratio log-uniform in
    [0.1, 2] (itheta = mass ratio x length^3 / 3 about the hinge), stiffness log-uniform in
    [1e-4, 1e-2], incidence uniform in [0, 20] degrees, fine grid one of 256x128, 384x192,
    512x256 on [-1,7]x[-2,2], 3 levels, dt 2e-3, GMRES and FSI tolerances 1e-10.  The plate length
    is drawn in [0.75, 1.25] and its points are two grid spacings apart (17 to 41 points by
    grid and length): closer points make the Schur operator singular (tests/
    test_conditioning_cpu.py), so the 50-150 points of a flexible beam's nodes are not used."""
    grids = [(256, 128), (384, 192), (512, 256)]
    runs = []
    for s in range(nsim):
        rng = np.random.default_rng(seed0 + s)
        Re = rng.uniform(100.0, 500.0)
        mass_ratio = math.exp(rng.uniform(math.log(0.1), math.log(2.0)))
        stiffness = math.exp(rng.uniform(math.log(1e-4), math.log(1e-2)))
        incidence = rng.uniform(0.0, 20.0)
        m, n = grids[int(rng.integers(0, 3))]
        length = rng.uniform(0.75, 1.25)
        delta = 8.0 / m
        npts = int(round(length / (2.0 * delta))) + 1
        p = Params(m=m, n=n, mgridlev=3, dt=2e-3, Re=Re, len=8.0, offsetx=1.0, offsety=2.0, fsi_tol=1e-10,
                   atol=1e-10, rtol=1e-10, autotune=False)
        body = torsional_plate(npts, length, -incidence, itheta=mass_ratio * length ** 3 / 3.0, ktheta=stiffness)
        runs.append((p, [body]))
    return runs
