"""CPU oracle for the IB_Parallel time step -- TEST INFRASTRUCTURE ONLY.

This module is a plain numpy/scipy restatement of the reference Fortran
(nirmaljp6/IB_Parallel, ``src/*.F90``) for one rank.  It is the checker for the
GPU path: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it.  The product library never calls it.

Parity status: the reference cannot be compiled here (no Fortran compiler,
PETSc, FFTW or MPI) and ships no golden vectors, known-answer tests or result
files, so this restatement is *parity unpinned* against the reference's own
outputs.  It is pinned instead by mathematical identities that the reference's
algorithm must satisfy (DST-I involution, Poisson inversion, rot/curl and
reg/regT adjointness, delta-function moments, uniform flow staying uniform)
and by frozen regression vectors (``tests/golden``).

Array layout (x fastest, C order, shape = (rows=y, cols=x)):
  vertex fields (omega, s, rhs):  (n-1, m-1), [J-2, I-2] <-> grid point (I, J)
  u-face fluxes qx:               (n, m+1),   [j-1, i-1]
  v-face fluxes qy:               (n+1, m),   [j-1, i-1]
  boundary ring (nbc=2(m+1)+2(n+1)): left[n+1], right[n+1], bottom[m+1], top[m+1]
  force-like vectors (nf=2*nb): per body, x-unknowns then y-unknowns
  (``grid.F90:403-433`` collect_bodies).

Third-party arithmetic restated here (absent from the reference tree):
  * FFTW 3.3.8 ``FFTW_RODFT00`` (``myfft.F90:119``) = unnormalised DST-I,
    restated with ``scipy.fft.dstn(type=1)``.
  * PETSc 3.11.1 KSPGMRES (``variables.F90:565-574``): restart 30, classical
    Gram-Schmidt without refinement, unpreconditioned norm, nonzero initial
    guess, default convergence test ``rnorm <= max(rtol*||b||, atol)``.
  * Elemental Cholesky (``variables.F90:554-562``): dense Cholesky of the upper
    triangle, restated with numpy.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np
import scipy.fft as sfft

PI = 4.0 * math.atan(1.0)  # parameters.F90:61


def _f32(v: float) -> float:
    """A default-REAL (single precision) Fortran literal promoted to double."""
    return float(np.float32(v))


# ---------------------------------------------------------------------------
# Smoothed 6-point delta function, grid.F90:955-1003.  Literals written without
# a ``d`` exponent in the Fortran source are default REAL (single precision) and
# are rounded to float32 here exactly as the compiled reference does.
# ---------------------------------------------------------------------------
_D1 = dict(c4=0.4166666667e-1, a=_f32(-.1388888889), b=0.3472222222e-1,
           c=-0.7121664902e-1, d=0.5208333333e-1, e=_f32(0.2405626122),
           f=_f32(.2405626122), g=_f32(.3792313933), h=_f32(.1012731481),
           i=0.8018753741e-1, j=0.4195601852e-1, k=_f32(.6485698427))
_D2 = dict(c4=-0.6250000000e-1, a=_f32(.4861111111), b=0.1736111111e-1,
           c=_f32(-1.143175026), d=0.7812500000e-1, e=_f32(.1202813061),
           f=_f32(.8751991178), g=_f32(.3608439183), h=_f32(.1548032407),
           i=_f32(.2806563809), j=0.822848104e-2, k=_f32(.1150173611))
_D3 = dict(c4=0.2083333333e-1, a=0.3472222222e-2, b=_f32(.2638888889),
           c=_f32(1.214391675), d=0.2604166667e-1, e=0.2405626122e-1,
           f=_f32(.1202813061), g=_f32(2.449273192), h=0.7262731481e-1,
           i=_f32(.1523563211), j=_f32(1.843201677), k=0.7306134259e-1)


def deltafnc(x1: float, x2: float, dr: float) -> float:
    """grid.F90:955-1003 (scalar, same operation order as the source)."""
    r = abs(x1 - x2)
    r1 = r / dr
    r2 = r1 * r1
    r3 = r2 * r1
    r4 = r3 * r1
    s3 = math.sqrt(3.0)
    if r1 <= 1.0:
        c = _D1
        a5 = math.asin((1.0 / 2.0) * s3 * (2.0 * r1 - 1.0))
        a8 = math.sqrt(1.0 - 12.0 * r2 + 12.0 * r1)
        v = (c['c4'] * r4 + (c['a'] + c['b'] * a8) * r3
             + (c['c'] - c['d'] * a8 + c['e'] * a5) * r2
             + (-c['f'] * a5 - c['g'] + c['h'] * a8) * r1
             + c['i'] * a5 - c['j'] * a8 + c['k'])
    elif r1 <= 2.0:
        c = _D2
        a6 = math.asin((1.0 / 2.0) * s3 * (-3.0 + 2.0 * r1))
        a9 = math.sqrt(-23.0 + 36.0 * r1 - 12.0 * r2)
        v = (c['c4'] * r4 + (c['a'] - c['b'] * a9) * r3
             + (c['c'] + c['d'] * a9 - c['e'] * a6) * r2
             + (c['f'] + c['g'] * a6 - c['h'] * a9) * r1
             - c['i'] * a6 + c['j'] + c['k'] * a9)
    elif r1 <= 3.0:
        c = _D3
        a1 = math.asin((1.0 / 2.0 * (2.0 * r1 - 5.0)) * s3)
        a7 = math.sqrt(-71.0 - 12.0 * r2 + 60.0 * r1)
        v = (c['c4'] * r4 + (c['a'] * a7 - c['b']) * r3
             + (c['c'] - c['d'] * a7 + c['e'] * a1) * r2
             + (-c['f'] * a1 - c['g'] + c['h'] * a7) * r1
             + c['i'] * a1 + c['j'] - c['k'] * a7)
    else:
        v = 0.0
    return v / dr


def deltafnc_vec(x1, x2, dr):
    """Elementwise grid.F90:955-1003 (same branches, literals and operation order)."""
    x1, x2 = np.broadcast_arrays(np.asarray(x1, dtype=np.float64), np.asarray(x2, dtype=np.float64))
    r = np.abs(x1 - x2)
    r1 = r / dr
    r2 = r1 * r1
    r3 = r2 * r1
    r4 = r3 * r1
    s3 = math.sqrt(3.0)
    out = np.zeros_like(r1)
    with np.errstate(invalid='ignore'):
        c = _D1
        a5 = np.arcsin((1.0 / 2.0) * s3 * (2.0 * r1 - 1.0))
        a8 = np.sqrt(1.0 - 12.0 * r2 + 12.0 * r1)
        v1 = (c['c4'] * r4 + (c['a'] + c['b'] * a8) * r3
              + (c['c'] - c['d'] * a8 + c['e'] * a5) * r2
              + (-c['f'] * a5 - c['g'] + c['h'] * a8) * r1
              + c['i'] * a5 - c['j'] * a8 + c['k'])
        c = _D2
        a6 = np.arcsin((1.0 / 2.0) * s3 * (-3.0 + 2.0 * r1))
        a9 = np.sqrt(-23.0 + 36.0 * r1 - 12.0 * r2)
        v2 = (c['c4'] * r4 + (c['a'] - c['b'] * a9) * r3
              + (c['c'] + c['d'] * a9 - c['e'] * a6) * r2
              + (c['f'] + c['g'] * a6 - c['h'] * a9) * r1
              - c['i'] * a6 + c['j'] + c['k'] * a9)
        c = _D3
        a1 = np.arcsin((1.0 / 2.0 * (2.0 * r1 - 5.0)) * s3)
        a7 = np.sqrt(-71.0 - 12.0 * r2 + 60.0 * r1)
        v3 = (c['c4'] * r4 + (c['a'] * a7 - c['b']) * r3
              + (c['c'] - c['d'] * a7 + c['e'] * a1) * r2
              + (-c['f'] * a1 - c['g'] + c['h'] * a7) * r1
              + c['i'] * a1 + c['j'] - c['k'] * a7)
    out = np.where(r1 <= 1.0, v1, np.where(r1 <= 2.0, v2, np.where(r1 <= 3.0, v3, 0.0)))
    return out / dr


# ---------------------------------------------------------------------------
# Problem description
# ---------------------------------------------------------------------------
@dataclass
class Body:
    """One ``input/body.NNN.inp`` (grid.F90:252-288)."""
    x: np.ndarray
    y: np.ndarray
    fam: int = 1                 # 1 rigid, 2 torsional, 3 Euler-Bernoulli beam (a stub in the reference)
    gamma0_deg: float = 0.0
    alpha0_deg: float = 0.0
    itheta: float = 0.0          # fam 3: mass per unit length
    ktheta: float = 0.0          # fam 3: bending stiffness EI
    ctheta: float = 0.0
    nelem: int = 0               # fam 3: finite elements (0: (npts - 1) / 2)

    @property
    def npts(self) -> int:
        return len(self.x)


@dataclass
class Params:
    """Namelist ``read_parameters`` (parameters.F90:55-59)."""
    m: int
    n: int
    mgridlev: int
    dt: float
    Re: float
    len: float
    offsetx: float
    offsety: float
    fsi_tol: float = 1e-10
    atol: float = 1e-10
    rtol: float = 1e-10
    num_stat: bool = False
    # motion_grid (user.F90:13-31): frame velocity (u, v), angular velocity, centre
    motion: tuple = (-1.0, 0.0, 0.0, 0.0, 0.0)
    gmres_restart: int = 30
    gmres_max_it: int = 10000


# ---------------------------------------------------------------------------
# The solver
# ---------------------------------------------------------------------------
class IBOracle:
    def __init__(self, p: Params, bodies: List[Body]):
        self.p = p
        m, n, L = p.m, p.n, p.mgridlev
        if m % 4 or n % 4:
            raise ValueError("grid must be divisible by 4")          # grid.F90:135-139
        self.m, self.n, self.L = m, n, L
        self.delta = p.len / float(m)                                  # grid.F90:131
        self.nbc = 2 * (m + 1) + 2 * (n + 1)                           # grid.F90:224-228
        self.left, self.right = 0, n + 1
        self.bottom, self.top = 2 * (n + 1), 2 * (n + 1) + m + 1
        self._setup_fft()
        self._setup_bodies(bodies)
        # state (variables.F90:262-295 initial_condition)
        self.omega = [np.zeros((n - 1, m - 1)) for _ in range(L)]
        self.s = [np.zeros((n - 1, m - 1)) for _ in range(L)]
        self.qx = [np.zeros((n, m + 1)) for _ in range(L)]
        self.qy = [np.zeros((n + 1, m)) for _ in range(L)]
        self.rhs_old = [np.zeros((n - 1, m - 1)) for _ in range(L)]
        self.q0x, self.q0y = self.frame_flux(0)
        self.f = np.zeros(self.nf)
        self.f_rdst = np.zeros(self.nf)
        # velocity u_B of prescribed rigid-body motion (compute_rhs_prescribed, user.F90:137-174;
        # its body is commented out in the reference: a host sets it with the positions)
        self.ub = np.zeros(self.nf)
        self.itime = 0
        self.ksp_iter = 0
        self.fsi_iter = 0
        self.cholM = None
        self.sd = None   # ib_subdomain.SubDomain: the sub-domain method (sub_domain = T)

    # ----------------------------------------------------------- myfft.F90
    def _setup_fft(self):
        """setup_fft, myfft.F90:96-157."""
        p, m, n = self.p, self.m, self.n
        self.normalize = 4.0 * float(m * n)
        del2 = self.delta * self.delta
        I = np.arange(2, m + 1, dtype=np.float64)[None, :]
        J = np.arange(2, n + 1, dtype=np.float64)[:, None]
        lam = -2.0 * (np.cos(PI * (I - 1) / float(m)) + np.cos(PI * (J - 1) / float(n)) - 2.0)
        self.lam = lam
        self.laminv = 1.0 / lam / self.normalize
        self.vfac, self.con1, self.con2, self.lam1, self.lam1i = [], [], [], [], []
        for k in range(1, self.L + 1):
            del22 = del2 * 4.0 ** (k - 1)
            self.vfac.append(0.5 * p.dt / p.Re / del22 / self.normalize)
            self.con1.append(1.5 * p.dt / del22 / self.normalize)
            self.con2.append(-0.5 * p.dt / del22 / self.normalize)
            self.lam1.append((1.0 - 0.5 * p.dt * lam / del22 / p.Re) / self.normalize)
            self.lam1i.append(1.0 / (1.0 + 0.5 * p.dt * lam / del22 / p.Re))

    @staticmethod
    def dst(x):
        """FFTW RODFT00 x RODFT00 (myfft.F90:207-216): unnormalised 2-D DST-I."""
        return sfft.dstn(x, type=1)

    def ctci(self, vort):
        """myfft.F90:177-188."""
        return self.dst(self.laminv * self.dst(vort))

    def ainv(self, vort):
        """myfft.F90:161-173."""
        return self.dst(self.lam1i[0] * self.dst(vort) / self.normalize)

    # ------------------------------------------------ operators_fluid.F90
    def ghost_vertex(self, f, ring):
        """Ghosted vertex field with its edges overwritten by a boundary ring in
        the order left, right, bottom, top (operators_fluid.F90:448-451, 563-566)."""
        m, n = self.m, self.n
        g = np.zeros((n + 1, m + 1))
        g[1:n, 1:m] = f
        g[:, 0] = ring[self.left:self.left + n + 1]
        g[:, m] = ring[self.right:self.right + n + 1]
        g[0, :] = ring[self.bottom:self.bottom + m + 1]
        g[n, :] = ring[self.top:self.top + m + 1]
        return g

    def nonlinear(self, omega, qx, qy, bc):
        """operators_fluid.F90:553-587.  Ghost fluxes outside the physical grid are
        zero (DM_BOUNDARY_GHOSTED local vectors are never filled there)."""
        m, n = self.m, self.n
        W = self.ghost_vertex(omega, bc)
        QX = np.zeros((n + 2, m + 1))
        QX[1:n + 1] = qx
        QY = np.zeros((n + 1, m + 2))
        QY[:, 1:m + 1] = qy
        U = 0.5 * (QX[1:n + 2] + QX[0:n + 1])           # uavg(i,j), i=1..m+1, j=1..n+1
        V = 0.5 * (QY[:, 1:m + 2] + QY[:, 0:m + 1])     # vavg(i,j)
        nlx = 0.5 * (V[1:n + 1] * W[1:n + 1] + V[0:n] * W[0:n])
        nly = -0.5 * (U[:, 1:m + 1] * W[:, 1:m + 1] + U[:, 0:m] * W[:, 0:m])
        return nlx, nly

    def rot(self, hx, hy):
        """rot_int + rot_bc, operators_fluid.F90:203-233 (curl transpose)."""
        m, n = self.m, self.n
        return hy[1:n, 1:m] - hy[1:n, 0:m - 1] - hx[1:n, 1:m] + hx[0:n - 1, 1:m]

    def curl(self, s, sbc):
        """curl_int + curl_bc, operators_fluid.F90:423-471."""
        m, n = self.m, self.n
        S = self.ghost_vertex(s, sbc)
        velx = S[1:n + 1, :] - S[0:n, :]
        vely = S[:, 0:m] - S[:, 1:m + 1]
        return velx, vely

    def coarsify(self, fine, coarse):
        """operators_fluid.F90:381-419 with index set grid.F90:1061-1087.  The
        full-weighting sum of the fine field at odd fine points overwrites the
        centre of the coarse field (in place)."""
        m, n = self.m, self.n
        F = fine
        cI = slice(1, m - 2, 2)
        cJ = slice(1, n - 2, 2)
        pI = slice(2, m - 1, 2)
        mI = slice(0, m - 3, 2)
        pJ = slice(2, n - 1, 2)
        mJ = slice(0, n - 3, 2)
        a = F[cJ, pI]; b = F[pJ, cI]; c = F[cJ, mI]; d = F[mJ, cI]
        e = F[pJ, pI]; f = F[mJ, pI]; g = F[mJ, mI]; h = F[pJ, mI]
        val = F[cJ, cI] + 0.5 * (a + b + c + d) + 0.25 * (e + f + g + h)
        coarse[n // 4: 3 * n // 4 - 1, m // 4: 3 * m // 4 - 1] = val
        return coarse

    def get_bc(self, s, fac):
        """operators_fluid.F90:475-535 (indices grid.F90:1091-1140): values of a
        coarse field on the fine grid's boundary, coincident points copied and
        midpoints averaged, times fac."""
        m, n = self.m, self.n
        ring = np.zeros(self.nbc)

        def sv(i, j):
            return s[j - 2, i - 2]

        i0, i1 = m // 4 + 1, 3 * m // 4 + 1
        j0, j1 = n // 4 + 1, 3 * n // 4 + 1
        ii = np.arange(i0, i1 + 1)
        jj = np.arange(j0, j1 + 1)
        for base, jrow in ((self.bottom, j0), (self.top, j1)):
            line = s[jrow - 2, ii - 2]
            ring[base + 2 * (ii - 1 - m // 4)] = line
            ring[base + 2 * (ii[:-1] - 1 - m // 4) + 1] = 0.5 * (line[:-1] + line[1:])
        for base, icol in ((self.left, i0), (self.right, i1)):
            line = s[jj - 2, icol - 2]
            ring[base + 2 * (jj - 1 - n // 4)] = line
            ring[base + 2 * (jj[:-1] - 1 - n // 4) + 1] = 0.5 * (line[:-1] + line[1:])
        return ring * fac

    def apply_bc(self, vort, ring, fac):
        """operators_fluid.F90:539-549 (in place): left, right, bottom, top."""
        m, n = self.m, self.n
        vort[:, 0] = vort[:, 0] + fac * ring[self.left + 1:self.left + n]
        vort[:, m - 2] = vort[:, m - 2] + fac * ring[self.right + 1:self.right + n]
        vort[0, :] = vort[0, :] + fac * ring[self.bottom + 1:self.bottom + m]
        vort[n - 2, :] = vort[n - 2, :] + fac * ring[self.top + 1:self.top + m]
        return vort

    def vort2flux(self, omega, L=None):
        """operators_fluid.F90:237-377.  Coarsifies omega in place (levels 2..L),
        then solves the Poisson problem coarse to fine.  Returns (s, qx, qy)."""
        L = self.L if L is None else L
        for k in range(1, L):
            self.coarsify(omega[k - 1], omega[k])
        vort2 = [w.copy() for w in omega]
        s = [None] * L
        qx = [None] * L
        qy = [None] * L
        sbc = np.zeros(self.nbc)
        s[L - 1] = self.ctci(vort2[L - 1])
        qx[L - 1], qy[L - 1] = self.curl(s[L - 1], sbc)
        if L > 1:
            sbc = self.get_bc(s[L - 1], 1.0)
        for k in range(L - 2, -1, -1):
            self.apply_bc(vort2[k], sbc, 1.0)
            s[k] = self.ctci(vort2[k])
            qx[k], qy[k] = self.curl(s[k], sbc)
            if k > 0:
                sbc = self.get_bc(s[k], 1.0)
        return s, qx, qy

    def fluid_predictor(self, omega, rhs, rhs_old, rhsbc, k):
        """operators_fluid.F90:649-663."""
        inner = self.dst(self.con1[k] * rhs + self.con2[k] * rhs_old + rhsbc)
        return self.dst(self.lam1i[k] * (inner + self.lam1[k] * self.dst(omega)))

    def frame_flux(self, it):
        """motion_potential + motion_rotation (variables.F90:299-360)."""
        m, n = self.m, self.n
        uv = self.p.motion
        q0x, q0y = [], []
        for k in range(1, self.L + 1):
            fac = self.delta * 2.0 ** (k - 1)
            qpx = np.full((n, m + 1), -fac * uv[0])
            qpy = np.full((n + 1, m), -fac * uv[1])
            omb = uv[2]
            rox, roy = uv[3], uv[4]
            i = np.arange(1, m + 2, dtype=np.float64)[None, :]
            j = np.arange(1, n + 1, dtype=np.float64)[:, None]
            yy = (j - 0.5 - n // 2) * self.delta * (2 ** (k - 1)) + n // 2 * self.delta - self.p.offsety
            qrx = fac * (0.0 + omb * (yy - roy)) * np.ones_like(i)
            i2 = np.arange(1, m + 1, dtype=np.float64)[None, :]
            xx = (i2 - 0.5 - m // 2) * self.delta * (2 ** (k - 1)) + m // 2 * self.delta - self.p.offsetx
            qry = fac * (0.0 - omb * (xx - rox)) * np.ones((n + 1, 1))
            q0x.append(qpx + qrx)
            q0y.append(qpy + qry)
        return q0x, q0y

    # ------------------------------------------------------- bodies / E
    def _setup_bodies(self, bodies: List[Body]):
        """setup_geometry + collect_bodies (grid.F90:239-433)."""
        # rigid bodies must come first (grid.F90:1226,1244)
        seen_nonrigid = False
        for b in bodies:
            if b.fam != 1:
                seen_nonrigid = True
            elif seen_nonrigid:
                raise ValueError("rigid bodies must be numbered before non-rigid ones")
            if b.fam not in (1, 2, 3):
                raise ValueError("body families are 1 (rigid), 2 (torsional) and 3 (beam)")
        self.bodies = bodies
        self.nb = sum(b.npts for b in bodies)
        self.nf = 2 * self.nb
        xb = np.zeros(self.nf)
        yb = np.zeros(self.nf)
        comp = np.zeros(self.nf, dtype=np.int64)   # codeb(:,3): 1 = x, 2 = y
        bid = np.zeros(self.nf, dtype=np.int64)    # codeb(:,1): body number (0-based)
        self.body_off = []
        off = 0
        for ib, b in enumerate(bodies):
            np_ = b.npts
            self.body_off.append(off)
            xb[off:off + np_] = b.x; yb[off:off + np_] = b.y
            xb[off + np_:off + 2 * np_] = b.x; yb[off + np_:off + 2 * np_] = b.y
            comp[off:off + np_] = 1; comp[off + np_:off + 2 * np_] = 2
            bid[off:off + 2 * np_] = ib
            off += 2 * np_
        self.xb, self.yb, self.comp, self.bid = xb, yb, comp, bid
        # torsional bodies (family 2) in file order = rank_body order for one rank
        self.tors = [i for i, b in enumerate(bodies) if b.fam == 2]
        nt = len(self.tors)
        self.theta = np.zeros(nt); self.thetad = np.zeros(nt); self.thetadd = np.zeros(nt)
        self.theta0 = np.zeros(nt); self.thetad0 = np.zeros(nt); self.thetadd0 = np.zeros(nt)
        self.beams = [beam_setup(bodies[i], self.body_off[i], self.p.dt) for i, b in enumerate(bodies) if b.fam == 3]
        self.tb = []
        for i in self.tors:
            b = bodies[i]
            self.tb.append(dict(
                gamma0=b.gamma0_deg * PI / 180, itheta=b.itheta, ktheta=b.ktheta,
                ctheta=b.ctheta, npts=b.npts, off=self.body_off[i],
                deltas=math.sqrt((b.x[1] - b.x[0]) ** 2 + (b.y[1] - b.y[0]) ** 2),
                xbf0=float(b.x[0]), ybf0=float(b.y[0])))
        self.setup_reg()

    def reg_weights(self, xb, yb, comp):
        """grid.F90:459-528 (and setup_pre_reg_subdomain, grid.F90:627-693, for the sub-domain
        points): stencil face indices and weights of points at (xb, yb) with components comp
        (1 = x on u-faces, 2 = y on v-faces).  weight = delta*delta*d(x)*d(y), l (y offset)
        outer, p (x offset) inner, exactly as the source loops."""
        d, ox, oy, m = self.delta, self.p.offsetx, self.p.offsety, self.m
        d2 = 0.5 * d
        ix = ((xb + ox) / d).astype(np.int64) + 1      # Fortran INT truncation
        iy = ((yb + oy) / d).astype(np.int64) + 1
        off = np.arange(-3, 4)
        xs = (comp == 1)[:, None]
        # grid coordinates of the 7 stencil columns / rows for each unknown
        gx = d * (ix[:, None] - 1 + off[None, :]) - ox
        gx = np.where(xs, gx, gx + d2)
        gy = d * (iy[:, None] - 1 + off[None, :]) - oy
        gy = np.where(xs, gy + d2, gy)
        dxv = deltafnc_vec(gx, xb[:, None], d)          # (nf, 7) over p
        dyv = deltafnc_vec(gy, yb[:, None], d)          # (nf, 7) over l
        w = (d * d * dxv[:, None, :]) * dyv[:, :, None]      # (nf, l, p)
        fi = ix[:, None, None] + off[None, None, :]           # face i
        fj = iy[:, None, None] + off[None, :, None]           # face j
        idx = np.where(xs[:, :, None], (m + 1) * (fj - 1) + (fi - 1), m * (fj - 1) + (fi - 1))
        return idx.reshape(len(xb), 49), w.reshape(len(xb), 49)

    def setup_reg(self):
        """grid.F90:459-528: stencil indices and weights of E for the current body positions."""
        self.reg_idx, self.reg_w = self.reg_weights(self.xb, self.yb, self.comp)

    def reg_with(self, idx, w, comp, h0):
        """fsinterface.F90:14-47 (reg_sd_sparse, fsinterface.F90:84-126, with the sub-domain's
        weights): E^T, scatter-add in unknown order."""
        m, n = self.m, self.n
        hx = np.zeros((n, m + 1)).ravel()
        hy = np.zeros((n + 1, m)).ravel()
        xs = comp == 1
        vals = w * h0[:, None]
        np.add.at(hx, idx[xs].ravel(), vals[xs].ravel())
        np.add.at(hy, idx[~xs].ravel(), vals[~xs].ravel())
        return hx.reshape(n, m + 1), hy.reshape(n + 1, m)

    def regT_with(self, idx, w, comp, hx, hy, h0=None):
        """fsinterface.F90:51-80 (regT_sd_sparse, fsinterface.F90:130-161, with the
        sub-domain's weights): E, gathered and accumulated into h0 in stencil order (slot by
        slot, so each unknown sees the source's summation order)."""
        h0 = np.zeros(len(comp)) if h0 is None else h0.copy()
        fx, fy = hx.ravel(), hy.ravel()
        xs = comp == 1
        acc = h0
        for t in range(49):
            ix = idx[:, t]
            src = np.where(xs, fx[np.where(xs, ix, 0)], fy[np.where(xs, 0, ix)])
            acc = acc + w[:, t] * src
        return acc

    def reg(self, h0):
        """fsinterface.F90:14-47: E^T, scatter-add in body-point order."""
        return self.reg_with(self.reg_idx, self.reg_w, self.comp, h0)

    def regT(self, hx, hy, h0=None):
        """fsinterface.F90:51-80: E, gathered in stencil order."""
        return self.regT_with(self.reg_idx, self.reg_w, self.comp, hx, hy, h0)

    def redistribute(self, f):
        """operators_struct.F90:735-834."""
        wx, wy = self.reg(np.ones(self.nf))
        fx, fy = self.reg(f)
        ix = np.zeros_like(wx); iy = np.zeros_like(wy)
        mx = wx > 1e-10; my = wy > 1e-10
        ix[mx] = 1.0 / wx[mx] * fx[mx]
        iy[my] = 1.0 / wy[my] * fy[my]
        return self.regT(ix, iy)

    def force_coeffs(self, f):
        """write_force2, operators_struct.F90:711-731: per body (Cx, Cy)."""
        nbod = len(self.bodies)
        fx = np.zeros(nbod); fy = np.zeros(nbod)
        for k in range(self.nf):
            if self.comp[k] == 1:
                fx[self.bid[k]] += f[k] / self.p.dt
            else:
                fy[self.bid[k]] += f[k] / self.p.dt
        return 2 * self.delta * fx, 2 * self.delta * fy

    # ------------------------------------------------ operators_struct.F90
    def _BR(self, t, th):
        """BR_build, operators_struct.F90:319-338."""
        b = self.tb[t]
        np_ = b['npts']
        j = np.arange(np_, dtype=np.float64)
        out = np.empty(2 * np_)
        out[:np_] = j * b['deltas'] * math.sin(b['gamma0'] - th)
        out[np_:] = -j * b['deltas'] * math.cos(b['gamma0'] - th)
        return out

    def _keff(self, t):
        b = self.tb[t]
        dt = self.p.dt
        return 4.0 / dt ** 2 * b['itheta'] + 2.0 / dt * b['ctheta'] + b['ktheta']

    def b_times(self, x):
        """b_times2, operators_struct.F90:14-127: rank-one torsional block,
        y = BR (BR . x) / K_eff * (delta^2/ds/dt)(2 ds/dt) on each torsional body."""
        y = np.zeros(self.nf)
        dt = self.p.dt
        for t, b in enumerate(self.tb):
            o, np_ = b['off'], b['npts']
            br = self._BR(t, self.theta[t])
            xb_ = x[o:o + 2 * np_]
            y[o:o + 2 * np_] = br * (br @ xb_) / self._keff(t) * \
                ((self.delta ** 2 / b['deltas'] / dt) * (2 * b['deltas'] / dt))
        for bm in self.beams:
            o, n2 = bm.off, 2 * bm.npts
            y[o:o + n2] = bm.B @ x[o:o + n2] * (2.0 * self.delta * self.delta / (dt * dt))
        return y

    def compute_rhs(self):
        """operators_struct.F90:342-398 (gravity and pseudo-forces are zero)."""
        y = np.zeros(self.nf)
        dt = self.p.dt
        for t, b in enumerate(self.tb):
            I, C, K = b['itheta'], b['ctheta'], b['ktheta']
            th, th0, thd, thd0, thdd0 = self.theta[t], self.theta0[t], self.thetad[t], self.thetad0[t], self.thetadd0[t]
            rth = thd0 + thd + 2.0 / dt * (th0 - th)
            jr = 2.0 / dt / (4.0 / dt ** 2 * I + 2.0 / dt * C + K) * (
                I * (4.0 / dt ** 2 * th0 + 4.0 / dt * thd0 + thdd0) + C * (thd0 + 2.0 / dt * th0)
                - (4.0 / dt ** 2 * I + 2.0 / dt * C + K) * th + 0.0 + 0.0)
            o, np_ = b['off'], b['npts']
            y[o:o + 2 * np_] = self._BR(t, th) * (self.delta * (rth - jr - thd))
        for bm in self.beams:
            y[bm.off:bm.off + 2 * bm.npts] = bm.rhs(self.delta)
        return y

    def compute_dx(self, f):
        """operators_struct.F90:402-505 + update_xb 600-620.  Returns err_fsi."""
        dt = self.p.dt
        err = 0.0
        for t, b in enumerate(self.tb):
            I, C, K = b['itheta'], b['ctheta'], b['ktheta']
            th, th0, thd0, thdd0 = self.theta[t], self.theta0[t], self.thetad0[t], self.thetadd0[t]
            jr = 1.0 / (4.0 / dt ** 2 * I + 2.0 / dt * C + K) * (
                I * (4.0 / dt ** 2 * th0 + 4.0 / dt * thd0 + thdd0) + C * (thd0 + 2.0 / dt * th0)
                - (4.0 / dt ** 2 * I + 2.0 / dt * C + K) * th + 0.0 + 0.0)
            o, np_ = b['off'], b['npts']
            brf = self._BR(t, th) @ f[o:o + 2 * np_]
            brf = b['deltas'] / (4.0 / dt ** 2 * I + K) * brf * (self.delta / b['deltas'] / dt)
            dth = jr + brf
            err = max(err, abs(dth))
            self.theta[t] = th + dth
            self.thetad[t] = -thd0 + 2.0 / dt * (self.theta[t] - th0)
            self.thetadd[t] = -thdd0 - 4.0 / dt * thd0 + 4.0 / dt ** 2 * (self.theta[t] - th0)
            j = np.arange(np_, dtype=np.float64)
            g = b['gamma0'] - self.theta[t]
            px = b['xbf0'] + j * b['deltas'] * math.cos(g)
            py = b['ybf0'] + j * b['deltas'] * math.sin(g)
            self.xb[o:o + np_] = px; self.xb[o + np_:o + 2 * np_] = px
            self.yb[o:o + np_] = py; self.yb[o + np_:o + 2 * np_] = py
        for bm in self.beams:
            err = max(err, bm.dx(f[bm.off:bm.off + 2 * bm.npts], self.delta))
            px, py = bm.positions()
            o, np_ = bm.off, bm.npts
            self.xb[o:o + np_] = px; self.xb[o + np_:o + 2 * np_] = px
            self.yb[o:o + np_] = py; self.yb[o + np_:o + 2 * np_] = py
        return err

    def initial_acc(self, f):
        """operators_struct.F90:233-294."""
        dt = self.p.dt
        for t, b in enumerate(self.tb):
            o, np_ = b['off'], b['npts']
            brf = self._BR(t, self.theta[t]) @ f[o:o + 2 * np_]
            brf = brf * self.delta / b['deltas'] / dt
            ftint = b['ktheta'] * self.theta[t]
            self.thetadd[t] = 1.0 / b['itheta'] * (-b['ctheta'] * self.thetad[t] - ftint
                                                    + brf * b['deltas'] + 0.0 + 0.0)
        for bm in self.beams:
            bm.initial_acc(f[bm.off:bm.off + 2 * bm.npts], self.delta)

    # -------------------------------------------------------- Schur operator
    def a_times(self, x, with_b=True):
        """a_times2 (operators_fluid.F90:14-120) + ab_times (timestepper.F90:774-782);
        with_b=False gives a_times (operators_fluid.F90:1020-1105)."""
        hx, hy = self.reg(x)
        vort = [np.zeros_like(self.omega[0]) for _ in range(self.L)]
        vort[0] = self.ainv(self.rot(hx, hy))
        _, qx, qy = self.vort2flux(vort)
        y1 = self.regT(qx[0], qy[0])
        if not with_b:
            return y1
        return y1 + self.b_times(x)

    def gmres(self, b, x0, op):
        """PETSc 3.11 KSPGMRES as configured in variables.F90:565-574.  Returns
        (x, iterations, reason)."""
        p = self.p
        restart = p.gmres_restart
        x = x0.copy()
        its = 0
        ttol = None
        bnorm = float(np.sqrt(b @ b))
        reason = 0
        while not reason:
            r = b - op(x)
            rnorm = float(np.sqrt(r @ r))
            V = [r * (1.0 / rnorm) if rnorm != 0.0 else r]
            H = np.zeros((restart + 1, restart))
            cs = np.zeros(restart); sn = np.zeros(restart)
            g = np.zeros(restart + 1)
            g[0] = rnorm
            if rnorm == 0.0:
                reason = 2
                break
            if its == 0:
                rnorm0 = bnorm if bnorm != 0.0 else rnorm
                ttol = max(p.rtol * rnorm0, p.atol)
            if rnorm <= ttol:
                reason = 3
                break
            it = 0
            res = rnorm
            while not reason and it < restart and its < p.gmres_max_it:
                w = op(V[it])
                h = np.array([w @ V[j] for j in range(it + 1)])
                for j in range(it + 1):
                    w = w - h[j] * V[j]
                tt = float(np.sqrt(w @ w))
                if tt != 0.0:
                    w = w * (1.0 / tt)
                V.append(w)
                hapbnd = min(abs(tt / g[it]), 1e-30)
                hapend = tt < hapbnd
                col = np.zeros(restart + 1)
                col[:it + 1] = h
                col[it + 1] = tt
                for j in range(it):
                    t0 = col[j]
                    col[j] = cs[j] * t0 + sn[j] * col[j + 1]
                    col[j + 1] = cs[j] * col[j + 1] - sn[j] * t0
                if not hapend:
                    nrm = math.sqrt(col[it] * col[it] + col[it + 1] * col[it + 1])
                    cs[it] = col[it] / nrm
                    sn[it] = col[it + 1] / nrm
                    g[it + 1] = -(sn[it] * g[it])
                    g[it] = cs[it] * g[it]
                    col[it] = cs[it] * col[it] + sn[it] * col[it + 1]
                    res = abs(g[it + 1])
                else:
                    res = 0.0
                H[:, it] = col
                it += 1
                its += 1
                if res <= ttol:
                    reason = 2
                elif hapend:
                    reason = -3
            # KSPGMRESBuildSoln: back substitution on the rotated Hessenberg matrix
            k = it - 1
            if k >= 0:
                y = np.zeros(it)
                y[k] = g[k] / H[k, k]
                for i in range(k - 1, -1, -1):
                    tt = g[i]
                    for j in range(i + 1, k + 1):
                        tt = tt - H[i, j] * y[j]
                    y[i] = tt / H[i, i]
                upd = np.zeros_like(x)
                for j in range(it):
                    upd = upd + y[j] * V[j]
                x = x + upd
            if its >= p.gmres_max_it and not reason:
                reason = -3
        return x, its, reason

    # -------------------------------------------------- operators_pressure.F90
    # Pressure on every level (cell centres, (n, m) arrays, [j-1, i-1] <-> cell (i, j)) from the
    # state after a step: D D^T P = D N(q) - D E^T f/dt solved coarse to fine, then the
    # dynamic part removed and the result scaled to a pressure coefficient.
    def ddti(self, rhs):
        """myfft.F90:192-203: S[laminv_ddti * S[rhs]], S = RODFT00 x RODFT00 on (n, m),
        laminv_ddti = 1 / lam_ddti / (4 (m+1)(n+1)) (myfft.F90:147-152)."""
        m, n = self.m, self.n
        i = np.arange(1, m + 1, dtype=np.float64)[None, :]
        j = np.arange(1, n + 1, dtype=np.float64)[:, None]
        lam = 2.0 * (np.cos(PI * i / float(m + 1)) + np.cos(PI * j / float(n + 1)) - 2.0)
        laminv = 1.0 / lam / (4.0 * float((m + 1) * (n + 1)))
        return self.dst(laminv * self.dst(rhs))

    @staticmethod
    def divergence(qx, qy):
        """operators_pressure.F90:505-516: cell (i,j) gets qx(i+1,j)-qx(i,j)+qy(i,j+1)-qy(i,j)."""
        return qx[:, 1:] - qx[:, :-1] + qy[1:, :] - qy[:-1, :]

    def nonlinear_corner(self, omega, qx, qy):
        """operators_pressure.F90:441-455: omega times the vertex-averaged flux."""
        m, n = self.m, self.n
        oqx = 0.5 * (qy[1:n, 1:m] + qy[1:n, 0:m - 1]) * omega
        oqy = -0.5 * (qx[1:n, 1:m] + qx[0:n - 1, 1:m]) * omega
        return oqx, oqy

    def nonlinear_corner2edge(self, oqx, oqy, ubc, vbc):
        """operators_pressure.F90:459-501: the vertex products ghosted by their rings, averaged
        onto the faces."""
        m, n = self.m, self.n
        wx = self.ghost_vertex(oqx, ubc)
        wy = self.ghost_vertex(oqy, vbc)
        return 0.5 * (wx[1:n + 1, :] + wx[0:n, :]), 0.5 * (wy[:, 1:m + 1] + wy[:, 0:m])

    def coarsify_pressure(self, fine):
        """operators_pressure.F90:529-563 (index set :567-608, one rank): the full-weighting
        sums at even cells, interpolated to the centres of 2x2 blocks, into coarse cells
        (m/4+i/2+1, n/4+j/2+1); the coarse field is zero elsewhere."""
        m, n = self.m, self.n
        P = fine                                     # [j-1, i-1]
        I = np.arange(2, m - 1, 2)                   # even i = 2..m-2
        J = np.arange(2, n - 1, 2)
        jj, ii = np.meshgrid(J - 1, I - 1, indexing="ij")
        temp = (P[jj, ii] + 0.5 * (P[jj, ii + 1] + P[jj + 1, ii] + P[jj, ii - 1] + P[jj - 1, ii])
                + 0.25 * (P[jj + 1, ii + 1] + P[jj - 1, ii + 1] + P[jj - 1, ii - 1] + P[jj + 1, ii - 1]))
        coarse = np.zeros((n, m))
        a = temp[:-1, :-1]; b = temp[:-1, 1:]; c = temp[1:, :-1]; d = temp[1:, 1:]
        yy = (a + 3.0 * b + 3.0 * c + 9.0 * d) / 16.0   # i, j = 2..m-4, n-4 step 2
        i2 = np.arange(2, m - 3, 2); j2 = np.arange(2, n - 3, 2)
        coarse[np.ix_(n // 4 + j2 // 2, m // 4 + i2 // 2)] = yy
        return coarse

    def _qsq(self, qx, qy, fac):
        """fac ((qx(i+1,j)+qx(i,j))^2 + (qy(i,j+1)+qy(i,j))^2) at every cell."""
        a = qx[:, 1:] + qx[:, :-1]
        b = qy[1:, :] + qy[:-1, :]
        return fac * (a * a + b * b)

    def get_bc_phi1(self, qx, qy, fac):
        """operators_pressure.F90:731-767: the coarsest level's ring (left[n], right[n],
        bottom[m], top[m]) from the velocity of its boundary cells."""
        m, n = self.m, self.n
        v = self._qsq(qx, qy, fac)
        return np.concatenate([v[:, 0], v[:, m - 1], v[0, :], v[n - 1, :]])

    def get_bc_phi2(self, p):
        """operators_pressure.F90:771-817: a finer level's ring from the coarse cells around
        its footprint (two ring entries per coarse cell)."""
        m, n = self.m, self.n
        P = lambda i, j: p[j - 1, i - 1]
        ring = np.zeros(2 * m + 2 * n)
        L, R, B, T = 0, n, 2 * n, 2 * n + m
        for i in range(m // 4 + 1, 3 * m // 4 + 1):
            j = n // 4
            ring[B + 2 * (i - 1 - m // 4)] = 0.25 * (2 * P(i, j) + P(i, j + 1) + P(i - 1, j))
            ring[B + 2 * (i - 1 - m // 4) + 1] = 0.25 * (2 * P(i, j) + P(i, j + 1) + P(i + 1, j))
            j = 3 * n // 4 + 1
            ring[T + 2 * (i - 1 - m // 4)] = 0.25 * (2 * P(i, j) + P(i, j - 1) + P(i - 1, j))
            ring[T + 2 * (i - 1 - m // 4) + 1] = 0.25 * (2 * P(i, j) + P(i, j - 1) + P(i + 1, j))
        for j in range(n // 4 + 1, 3 * n // 4 + 1):
            i = m // 4
            ring[L + 2 * (j - 1 - n // 4)] = 0.25 * (2 * P(i, j) + P(i + 1, j) + P(i, j - 1))
            ring[L + 2 * (j - 1 - n // 4) + 1] = 0.25 * (2 * P(i, j) + P(i + 1, j) + P(i, j + 1))
            i = 3 * m // 4 + 1
            ring[R + 2 * (j - 1 - n // 4)] = 0.25 * (2 * P(i, j) + P(i - 1, j) + P(i, j - 1))
            ring[R + 2 * (j - 1 - n // 4) + 1] = 0.25 * (2 * P(i, j) + P(i - 1, j) + P(i, j + 1))
        return ring

    def apply_bc_phi(self, rhs, ring):
        """operators_pressure.F90:821-838 (in place): left, right, bottom, top subtracted."""
        m, n = self.m, self.n
        rhs[:, 0] = rhs[:, 0] - ring[0:n]
        rhs[:, m - 1] = rhs[:, m - 1] - ring[n:2 * n]
        rhs[0, :] = rhs[0, :] - ring[2 * n:2 * n + m]
        rhs[n - 1, :] = rhs[n - 1, :] - ring[2 * n + m:2 * n + 2 * m]
        return rhs

    def calculate_pressure(self):
        """operators_pressure.F90:110-437 (no sub-domain, zero user forcing): pressure
        coefficient 2 (P - |u|^2/2) on every level, coarsest to finest solve."""
        L, m, n = self.L, self.m, self.n
        nlq = [None] * L
        oq = [None] * L
        for k in range(L - 1, -1, -1):
            if k == L - 1:
                ubc = np.zeros(self.nbc); vbc = np.zeros(self.nbc)
            else:
                ubc = self.get_bc(oq[k + 1][0], 1.0); vbc = self.get_bc(oq[k + 1][1], 1.0)
            qx = self.qx[k] + self.q0x[k]; qy = self.qy[k] + self.q0y[k]
            oq[k] = self.nonlinear_corner(self.omega[k], qx, qy)
            nx, ny = self.nonlinear_corner2edge(oq[k][0], oq[k][1], ubc, vbc)
            d = self.delta * float(2 ** k)
            nlq[k] = (nx / (d * d), ny / (d * d))
        rhs = [np.zeros((n, m)) for _ in range(L)]
        if self.nf:
            hx, hy = self.reg(self.f / self.p.dt)
            rhs[0] = -self.divergence(hx, hy)
        for k in range(1, L):
            rhs[k] = self.coarsify_pressure(rhs[k - 1])
        for k in range(L):
            rhs[k] = rhs[k] + self.divergence(*nlq[k])
        p = [None] * L
        for k in range(L - 1, -1, -1):
            if k == L - 1:
                fac = 0.125 / (self.delta * 2.0 ** k) ** 2
                ring = self.get_bc_phi1(self.qx[k] + self.q0x[k], self.qy[k] + self.q0y[k], fac)
            else:
                ring = self.get_bc_phi2(p[k + 1])
            p[k] = self.ddti(self.apply_bc_phi(rhs[k], ring))
        for k in range(L):
            fac = 0.125 / (self.delta * 2.0 ** k) ** 2
            p[k] = 2.0 * (p[k] - self._qsq(self.qx[k] + self.q0x[k], self.qy[k] + self.q0y[k], fac))
        return p

    # ------------------------------------------------------------ stepping
    def preprocess(self):
        """timestepper.F90:560-598: dense Schur matrix, column i = a_times(e_i),
        factored by Cholesky of its upper triangle."""
        nf = self.nf
        M = np.zeros((nf, nf))
        for i in range(nf):
            e = np.zeros(nf); e[i] = 1.0
            M[:, i] = self.a_times(e, with_b=False)
        U = np.triu(M)
        Msym = U + np.triu(U, 1).T
        self.cholM = M
        self.cholL = np.linalg.cholesky(Msym)

    def chol_solve(self, b):
        import scipy.linalg as sla
        y = sla.solve_triangular(self.cholL, b, lower=True)
        return sla.solve_triangular(self.cholL.T, y, lower=False)

    def advance(self):
        """timestepper.F90:18-556: one time step."""
        p, L = self.p, self.L
        self.itime += 1
        it = self.itime
        self.q0x, self.q0y = self.frame_flux(it - 1)
        if it == 1 and p.num_stat:
            self.preprocess()
        # lastbc from the previous step's coarse vorticity (timestepper.F90:103-117)
        lastbc = [self.get_bc(self.omega[k + 1], 0.25) for k in range(L - 1)] + [np.zeros(self.nbc)]
        for k in range(L - 1, -1, -1):
            if k < L - 1:
                omegabc = self.get_bc(self.omega[k + 1], 0.25)
            else:
                omegabc = np.zeros(self.nbc)
            nlx, nly = self.nonlinear(self.omega[k], self.qx[k] + self.q0x[k],
                                      self.qy[k] + self.q0y[k], lastbc[k])
            rhsbc = np.zeros_like(self.omega[k])
            self.apply_bc(rhsbc, lastbc[k], self.vfac[k])
            self.apply_bc(rhsbc, omegabc, self.vfac[k])
            rhs = self.rot(nlx, nly)
            if it == 1:
                self.rhs_old[k] = rhs.copy()
            self.omega[k] = self.fluid_predictor(self.omega[k], rhs, self.rhs_old[k], rhsbc, k)
            self.rhs_old[k] = rhs
        self.s, self.qx, self.qy = self.vort2flux(self.omega)
        qhx = self.qx[0] + self.q0x[0]
        qhy = self.qy[0] + self.q0y[0]
        if self.nf == 0:
            pass
        elif not p.num_stat:
            fsi_count = 0
            err = 10.0
            self.ksp_iter = 0
            if it == 1:
                self.initial_acc(self.f)
            self.theta0 = self.theta.copy(); self.thetad0 = self.thetad.copy()
            self.thetadd0 = self.thetadd.copy()
            for bm in self.beams:
                bm.save()
            if self.sd is not None and self.sd.cols is None:
                self.sd.precompute()   # preprocess_sd at the first step (timestepper.F90:79-97)
            while err >= p.fsi_tol and fsi_count <= 1000:
                fsi_count += 1
                if self.sd is not None:
                    # timestepper.F90:368-405: lumat = body_mat + P B^T P^T, rhsf + P E_o q
                    pidx, pw = self.sd.interp()
                    rhsf = self.sd.rhs_add(self.compute_rhs() - self.delta * self.ub, qhx, qhy, pidx, pw)
                    lu = self.sd.lumat(pidx, pw)
                    self.f, its, _ = self.gmres(rhsf, self.f, lambda x, lu=lu: lu @ x)
                    self.ksp_iter += its
                    self.f_rdst = self.redistribute(self.f)
                    err = self.compute_dx(self.f)
                    self.setup_reg()
                    continue
                # compute_rhs, then rhsf - delta u_B (timestepper.F90:323-331), then E q on top
                rhsf = self.regT(qhx, qhy, self.compute_rhs() - self.delta * self.ub)
                self.f, its, _ = self.gmres(rhsf, self.f, self.a_times)
                self.ksp_iter += its
                self.f_rdst = self.redistribute(self.f)
                err = self.compute_dx(self.f)
                self.setup_reg()
            self.fsi_iter = fsi_count
        else:
            rhsf = self.regT(qhx, qhy, 0.0 - self.delta * self.ub)
            self.f = self.chol_solve(rhsf)
            self.f_rdst = self.redistribute(self.f)
        if self.sd is not None and self.nf and not p.num_stat:
            pidx, pw = self.sd.interp()
            hx, hy = self.sd.spread(self.f, pidx, pw)   # timestepper.F90:500-516
        else:
            hx, hy = self.reg(self.f) if self.nf else (np.zeros_like(self.qx[0]), np.zeros_like(self.qy[0]))
        vort = self.ainv(self.rot(hx, hy))
        self.omega[0] = self.omega[0] - vort
        self.s, self.qx, self.qy = self.vort2flux(self.omega)
        return it


# ---------------------------------------------------------------------------
# Euler-Bernoulli beam (body family 3).  The reference declares this family and leaves every
# routine empty (operators_struct.F90:104-106, 146-148, 171-174, 285-288, 378-381, 472-474):
# this is the library's own formulation, written from the standard finite-element mathematics
# and coupled the way the reference couples its torsional body (operators_struct.F90:14-505),
# with matrices in place of the hinge's scalars.  Parity against the reference is unpinned.
#   * A linear (small-deflection) beam clamped at its first point, lying along the line from its
#     first to its last point; transverse deflection w(s); nel Hermite-cubic elements of length
#     h with DOFs (w, dw/ds) at the nodes, the clamped node's removed: ndof = 2 nel.
#   * Element stiffness EI/h^3 [12 6h -12 6h; 6h 4h^2 -6h 2h^2; -12 -6h 12 -6h; 6h 2h^2 -6h 4h^2],
#     consistent mass rho h/420 [156 22h 54 -13h; 22h 4h^2 13h -3h^2; 54 13h 156 -22h;
#     -13h -3h^2 -22h 4h^2] (rho: mass per unit length).
#   * Body point j (arc length j ds) has deflection Phi_j q; with the unit normal
#     (-sin g, cos g) of the beam's direction g, its x and y unknowns move by W q,
#     W = [-sin g Phi; cos g Phi] (the role of BR).  The point forces f act on the DOFs as
#     F = (delta/dt) W^T f (the torque (BR . f) delta/dt of compute_dx).
#   * Newmark (trapezoidal) with K_eff = 4/dt^2 M + K, as compute_dx does for theta:
#     dq = K_eff^-1 (M (4/dt^2 q0 + 4/dt qd0 + qdd0) - K_eff q) + K_eff^-1 F,
#     qd = -qd0 + 2/dt (q - q0), qdd = -qdd0 - 4/dt qd0 + 4/dt^2 (q - q0), error max |dq|;
#     compute_rhs: delta W (r - jr - qd), r = qd0 + qd + 2/dt (q0 - q),
#     jr = 2/dt K_eff^-1 (M a - K_eff q); b_times: (2 delta^2/dt^2) W K_eff^-1 W^T x;
#     initial_acc: qdd = M^-1 (F - K q).
# ---------------------------------------------------------------------------
class BeamBody:
    def __init__(self, b: "Body", off: int, dt: float):
        x = np.asarray(b.x, dtype=np.float64); y = np.asarray(b.y, dtype=np.float64)
        npts = len(x)
        nel = int(b.nelem) if b.nelem else (npts - 1) // 2
        if nel < 1 or npts < 2:
            raise ValueError("a beam needs at least 2 points and 1 element")
        dx, dy = x[-1] - x[0], y[-1] - y[0]
        length = math.sqrt(dx * dx + dy * dy)
        self.cg, self.sg = dx / length, dy / length          # cos, sin of the beam's direction
        self.off, self.npts, self.nel, self.ndof, self.dt = off, npts, nel, 2 * nel, dt
        self.x0, self.y0 = x.copy(), y.copy()
        h = length / nel
        rho, EI = float(b.itheta), float(b.ktheta)
        kc = EI / (h * h * h)
        ke = kc * np.array([[12.0, 6.0 * h, -12.0, 6.0 * h], [6.0 * h, 4.0 * h * h, -6.0 * h, 2.0 * h * h],
                            [-12.0, -6.0 * h, 12.0, -6.0 * h], [6.0 * h, 2.0 * h * h, -6.0 * h, 4.0 * h * h]])
        mc = rho * h / 420.0
        me = mc * np.array([[156.0, 22.0 * h, 54.0, -13.0 * h], [22.0 * h, 4.0 * h * h, 13.0 * h, -3.0 * h * h],
                            [54.0, 13.0 * h, 156.0, -22.0 * h], [-13.0 * h, -3.0 * h * h, -22.0 * h, 4.0 * h * h]])
        nd = 2 * (nel + 1)
        K = np.zeros((nd, nd)); M = np.zeros((nd, nd))
        for e in range(nel):
            for a in range(4):
                for c in range(4):
                    K[2 * e + a, 2 * e + c] += ke[a, c]
                    M[2 * e + a, 2 * e + c] += me[a, c]
        self.K, self.M = K[2:, 2:].copy(), M[2:, 2:].copy()
        # deflection of body point j: element e = j nel div (npts-1), xi from the remainder
        phi = np.zeros((npts, self.ndof))
        for j in range(npts):
            e = min(j * nel // (npts - 1), nel - 1)
            xi = (j * nel - e * (npts - 1)) / float(npts - 1)
            xi2, xi3 = xi * xi, xi * xi * xi
            nvals = (1.0 - 3.0 * xi2 + 2.0 * xi3, h * (xi - 2.0 * xi2 + xi3), 3.0 * xi2 - 2.0 * xi3, h * (xi3 - xi2))
            for a in range(4):
                dof = 2 * e + a - 2
                if dof >= 0:
                    phi[j, dof] = nvals[a]
        self.phi = phi
        self.W = np.vstack([-self.sg * phi, self.cg * phi])
        self.Keff = 4.0 / (dt * dt) * self.M + self.K
        self.Ki = np.linalg.inv(self.Keff)
        self.Mi = np.linalg.inv(self.M)
        self.B = self.W @ self.Ki @ self.W.T
        z = lambda: np.zeros(self.ndof)
        self.q, self.qd, self.qdd, self.q0, self.qd0, self.qdd0 = z(), z(), z(), z(), z(), z()

    def _a(self):
        dt = self.dt
        return 4.0 / (dt * dt) * self.q0 + 4.0 / dt * self.qd0 + self.qdd0

    def save(self):
        self.q0, self.qd0, self.qdd0 = self.q.copy(), self.qd.copy(), self.qdd.copy()

    def rhs(self, delta):
        dt = self.dt
        r = self.qd0 + self.qd + 2.0 / dt * (self.q0 - self.q)
        jr = 2.0 / dt * (self.Ki @ (self.M @ self._a() - self.Keff @ self.q))
        return self.W @ (delta * (r - jr - self.qd))

    def dx(self, f, delta):
        dt = self.dt
        F = delta / dt * (self.W.T @ f)
        dq = self.Ki @ (self.M @ self._a() - self.Keff @ self.q) + self.Ki @ F
        self.q = self.q + dq
        self.qd = -self.qd0 + 2.0 / dt * (self.q - self.q0)
        self.qdd = -self.qdd0 - 4.0 / dt * self.qd0 + 4.0 / (dt * dt) * (self.q - self.q0)
        return float(np.abs(dq).max())

    def initial_acc(self, f, delta):
        F = delta / self.dt * (self.W.T @ f)
        self.qdd = self.Mi @ (F - self.K @ self.q)

    def positions(self):
        d = self.phi @ self.q
        return self.x0 + (-self.sg) * d, self.y0 + self.cg * d


def beam_setup(b, off, dt):
    return BeamBody(b, off, dt)


# ---------------------------------------------------------------------------
# Restart file output/dataRR_IIIIIII.var (variables.F90:709-913), a Fortran unformatted
# sequential stream as output/getdata.m reads it: each WRITE is one record framed by its byte
# length (4-byte integer) before and after; integers are 4 bytes, reals 8.
# ---------------------------------------------------------------------------
def _rec(buf: bytearray, arr) -> None:
    b = np.ascontiguousarray(arr).tobytes()
    n = np.int32(len(b)).tobytes()
    buf += n + b + n


def write_variables(o: "IBOracle", path) -> None:
    """write_variables (variables.F90:709-803) of a one-rank run."""
    m, n, L, nf = o.m, o.n, o.L, o.nf
    i4 = lambda *v: np.array(v, dtype="<i4")
    f8 = lambda *v: np.array(v, dtype="<f8")
    buf = bytearray()
    _rec(buf, i4(m, n, L, o.nb))
    _rec(buf, f8(o.p.Re, o.p.dt, o.p.len, o.p.offsetx, o.p.offsety))
    _rec(buf, i4(2, m, m - 1, 2, n, n - 1))
    _rec(buf, i4(1, m + 1, m + 1, 1, n, n))
    _rec(buf, i4(1, m, m, 1, n + 1, n + 1))
    uv = o.p.motion
    for k in range(L):
        fac = o.delta * 2.0 ** k
        px = np.full(o.q0x[k].shape, -fac * uv[0])
        py = np.full(o.q0y[k].shape, -fac * uv[1])
        for a in (o.omega[k], o.s[k], o.qx[k], px, o.q0x[k] - px, o.qy[k], py, o.q0y[k] - py):
            _rec(buf, np.asarray(a, dtype="<f8"))
    _rec(buf, np.stack(o.rhs_old).astype("<f8"))
    _rec(buf, f8(uv[2] * o.p.dt * o.itime, uv[3], uv[4]))
    _rec(buf, i4(nf, 1, nf))
    for a in (o.f, o.xb, o.yb):
        _rec(buf, np.asarray(a, dtype="<f8"))
    _rec(buf, i4(len(o.tors)))
    if o.tors:
        _rec(buf, np.concatenate([o.theta, o.thetad, o.thetadd]).astype("<f8"))
    _rec(buf, np.asarray(o.f_rdst, dtype="<f8"))
    with open(path, "wb") as fh:
        fh.write(bytes(buf))


def read_records(path) -> list:
    """The records of a Fortran unformatted sequential file, as raw bytes."""
    data = open(path, "rb").read()
    out, pos = [], 0
    while pos < len(data):
        (nb,) = np.frombuffer(data, "<i4", 1, pos)
        body = data[pos + 4:pos + 4 + nb]
        (ne,) = np.frombuffer(data, "<i4", 1, pos + 4 + nb)
        if ne != nb or len(body) != nb:
            raise ValueError(f"bad record framing at byte {pos}")
        out.append(body)
        pos += 8 + nb
    return out


def read_variables(path) -> dict:
    """Parse a restart file the way output/getdata.m does (one rank)."""
    r = read_records(path)
    i4 = lambda b: np.frombuffer(b, "<i4")
    f8 = lambda b: np.frombuffer(b, "<f8")
    m, n, L, nb = (int(v) for v in i4(r[0]))
    d = dict(m=m, n=n, mgridlev=L, nb=nb)
    d["Re"], d["dt"], d["len"], d["offsetx"], d["offsety"] = (float(v) for v in f8(r[1]))
    d["ranges"] = [tuple(int(v) for v in i4(r[q])) for q in (2, 3, 4)]
    names = ("omega", "s", "qx", "q0px", "q0rx", "qy", "q0py", "q0ry")
    shapes = dict(omega=(n - 1, m - 1), s=(n - 1, m - 1), qx=(n, m + 1), q0px=(n, m + 1), q0rx=(n, m + 1),
                  qy=(n + 1, m), q0py=(n + 1, m), q0ry=(n + 1, m))
    i = 5
    for nm in names:
        d[nm] = []
    for k in range(L):
        for nm in names:
            d[nm].append(f8(r[i]).reshape(shapes[nm]).copy())
            i += 1
    d["rhs_old"] = list(f8(r[i]).reshape(L, n - 1, m - 1).copy()); i += 1
    d["rot_angle"], d["rox"], d["roy"] = (float(v) for v in f8(r[i])); i += 1
    d["xfm"], d["xfi"], d["xfe"] = (int(v) for v in i4(r[i])); i += 1
    d["f"] = f8(r[i]).copy(); d["xb"] = f8(r[i + 1]).copy(); d["yb"] = f8(r[i + 2]).copy(); i += 3
    d["mt_body"] = int(i4(r[i])[0]); i += 1
    if d["mt_body"] > 0:
        t = f8(r[i]).reshape(3, d["mt_body"]); i += 1
        d["theta"], d["thetad"], d["thetadd"] = t[0].copy(), t[1].copy(), t[2].copy()
    d["f_rdst"] = f8(r[i]).copy() if i < len(r) else None
    d["nrecords"] = len(r)
    return d


def restore(o: "IBOracle", d: dict, itime: int) -> None:
    """read_variables (variables.F90:807-913) into an oracle of the same grid and bodies:
    q0 = q0p + q0r, E rebuilt at the positions read, step counter istart = itime."""
    if (d["m"], d["n"], d["mgridlev"], d["nb"]) != (o.m, o.n, o.L, o.nb):
        raise ValueError("grid or bodies differ")
    for k in range(o.L):
        o.omega[k] = d["omega"][k].copy(); o.s[k] = d["s"][k].copy()
        o.qx[k] = d["qx"][k].copy(); o.qy[k] = d["qy"][k].copy()
        o.q0x[k] = d["q0px"][k] + d["q0rx"][k]; o.q0y[k] = d["q0py"][k] + d["q0ry"][k]
        o.rhs_old[k] = d["rhs_old"][k].copy()
    o.f = d["f"].copy(); o.xb = d["xb"].copy(); o.yb = d["yb"].copy()
    if o.tors:
        o.theta = d["theta"].copy(); o.thetad = d["thetad"].copy(); o.thetadd = d["thetadd"].copy()
    o.itime = itime
    if o.nf:
        o.setup_reg()


# ---------------------------------------------------------------------------
# Seeded geometry generators for the configurations (the reference builds
# bodies with MATLAB scripts; these restate the shapes).
# ---------------------------------------------------------------------------
def cylinder(npts=157, diameter=1.0, xc=0.0, yc=0.0):
    th = 2.0 * PI * np.arange(npts) / npts
    return Body(x=xc + 0.5 * diameter * np.cos(th), y=yc + 0.5 * diameter * np.sin(th), fam=1)


def torsional_plate(npts=201, length=1.0, gamma0_deg=-10.0, itheta=0.5 / 3.0,
                    ktheta=1e-3, ctheta=0.0, x0=0.0, y0=0.0):
    g = gamma0_deg * PI / 180
    j = np.arange(npts, dtype=np.float64)
    ds = length / (npts - 1)
    return Body(x=x0 + j * ds * math.cos(g), y=y0 + j * ds * math.sin(g), fam=2,
                gamma0_deg=gamma0_deg, itheta=itheta, ktheta=ktheta, ctheta=ctheta)
