"""Shared test helpers: matching oracle / GPU problem setups."""
import numpy as np

import ib_oracle as O
from ib_parallel_gb300 import ibgpu as G
from ib_parallel_gb300 import geometry as GEO


def pair(p_kwargs: dict, bodies):
    """Build an oracle and a GPU simulation of the same problem."""
    po = O.Params(**{k: v for k, v in p_kwargs.items() if k in O.Params.__dataclass_fields__})
    pg = G.Params(**p_kwargs)
    ob = [O.Body(x=b.x.copy(), y=b.y.copy(), fam=b.fam, gamma0_deg=b.gamma0_deg, alpha0_deg=b.alpha0_deg,
                 itheta=b.itheta, ktheta=b.ktheta, ctheta=b.ctheta,
                 nelem=getattr(b, 'nelem', 0)) for b in bodies]
    return O.IBOracle(po, ob), G.Simulation(pg, bodies)


def rel(a, b):
    a = np.asarray(a); b = np.asarray(b)
    d = np.abs(a - b).max() if a.size else 0.0
    s = np.abs(b).max() if b.size else 0.0
    return d / s if s > 0 else d


SMALL = dict(m=64, n=32, mgridlev=3, dt=0.01, Re=100.0, len=8.0, offsetx=2.0, offsety=2.0,
             fsi_tol=1e-9, atol=1e-12, rtol=1e-11, autotune=False)
PLATE = dict(m=64, n=32, mgridlev=3, dt=0.004, Re=100.0, len=4.0, offsetx=1.0, offsety=1.0,
             fsi_tol=1e-9, atol=1e-12, rtol=1e-9, autotune=False)


def small_cylinder():
    return GEO.cylinder(npts=25)


def small_plate():
    return GEO.torsional_plate(npts=17, length=1.0, gamma0_deg=-10.0, itheta=0.5 / 3.0, ktheta=1e-3)
