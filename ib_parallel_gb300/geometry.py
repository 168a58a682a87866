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
