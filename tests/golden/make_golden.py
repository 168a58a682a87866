"""Regenerate the frozen regression vectors of the oracle (tests/golden/*.npz).

The reference ships no golden outputs, so these vectors freeze the oracle's own
results on small problems; test_golden_cpu.py checks the oracle still produces
them and test_gpu_golden.py checks the CUDA path against them.

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent / "oracle"))
import ib_oracle as O  # noqa: E402

CYL = dict(m=64, n=32, mgridlev=3, dt=0.01, Re=100.0, len=8.0, offsetx=2.0, offsety=2.0,
           fsi_tol=1e-9, atol=1e-12, rtol=1e-11, num_stat=True)
PLATE = dict(m=64, n=32, mgridlev=3, dt=0.004, Re=100.0, len=4.0, offsetx=1.0, offsety=1.0,
             fsi_tol=1e-9, atol=1e-12, rtol=1e-9)


def cylinder_case(steps):
    o = O.IBOracle(O.Params(**CYL), [O.cylinder(npts=25)])
    for _ in range(steps):
        o.advance()
    cx, cy = o.force_coeffs(o.f)
    return dict(omega0=o.omega[0], omega1=o.omega[1], omega2=o.omega[2], s0=o.s[0], qx0=o.qx[0],
                qy0=o.qy[0], f=o.f, f_rdst=o.f_rdst, cx=cx, cy=cy)


def plate_case(steps):
    o = O.IBOracle(O.Params(**PLATE), [O.torsional_plate(npts=17, length=1.0, gamma0_deg=-10.0,
                                                         itheta=0.5 / 3.0, ktheta=1e-3)])
    th, its, fsi = [], [], []
    for _ in range(steps):
        o.advance()
        th.append(o.theta.copy()); its.append(o.ksp_iter); fsi.append(o.fsi_iter)
    cx, cy = o.force_coeffs(o.f)
    return dict(theta=np.array(th), ksp=np.array(its), fsi=np.array(fsi), omega0=o.omega[0], f=o.f,
                xb=o.xb, cx=cx, cy=cy)


if __name__ == "__main__":
    np.savez_compressed(HERE / "cylinder64x32_direct_1step.npz", **cylinder_case(1))
    np.savez_compressed(HERE / "cylinder64x32_direct_10steps.npz", **cylinder_case(10))
    np.savez_compressed(HERE / "plate64x32_gmres_3steps.npz", **plate_case(3))
    print("written", sorted(p.name for p in HERE.glob("*.npz")))
