"""CPU oracle of the discrete adjoint of the time step -- TEST INFRASTRUCTURE ONLY.

The reference has no adjoint; this restates, for the oracle's own step (ib_oracle.IBOracle
.advance, i.e. timestepper.F90:18-556 with stationary rigid bodies), the exact
transpose of every linear map the step applies, so that the gradient of any function of the
per-step force coefficients with respect to the step's inputs follows by reverse accumulation.
The kinematics enter through the moving frame's flux (motion_potential + motion_rotation,
variables.F90:299-360), which is linear in the frame velocity (u, v) and angular velocity W at a
fixed centre: q0 = u Bu + v Bv + W BW on every level.  A pitching or plunging body held fixed in
its own frame (the reference's user.F90 motion_grid) takes a coefficient triple per step.

Transposes used (each is the exact adjoint of the oracle's forward arithmetic):
  * DST-I and the spectral solves ctci, ainv and the predictor's are symmetric;
  * rot^T = curl with a zero ring, curl^T = rot plus the ring's edge gathers (operators_fluid.F90:
    203-233, 423-471), ghost_vertex^T gathers the edges it overwrote;
  * nonlinear (operators_fluid.F90:553-587) is bilinear in (omega, q + q0) and linear in its
    ghost ring: each argument's transpose;
  * get_bc^T scatters the ring back onto the coarse grid, apply_bc^T gathers the boundary rows,
    coarsify^T spreads the full-weighting stencil (operators_fluid.F90:381-549);
  * reg and regT are each other's transposes (fsinterface.F90:14-80); the Cholesky solve of the
    symmetrised Schur matrix is symmetric (timestepper.F90:560-598).  Without num_stat the
    reference solves the Schur system by GMRES (timestepper.F90:363-366); here the forward solves
    it exactly with the dense Schur matrix (a_times on unit vectors; the bodies do not move, so it
    is formed once) and the reverse solves with its transpose: the adjoint of the exact solve,
    which a converged Krylov solve approaches.  With the sub-domain method the matrix is lumat,
    E is P E_o and E^T is E_o^T P^T (each the other's transpose).
The step's state between steps is (omega, q, rhs_old) on every level.
"""
from __future__ import annotations

import numpy as np


class Adjoint:
    def __init__(self, o):
        if any(b.fam != 1 for b in o.bodies):
            raise ValueError("the adjoint covers stationary rigid bodies")
        self.o = o
        self.S = None             # the dense Schur matrix without num_stat
        # frame bases: the flux of a unit u, v and W about the frame's centre (motion[3:5])
        saved = o.p.motion
        bases = []
        for uvw in ((1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0)):
            o.p.motion = (uvw[0], uvw[1], uvw[2], saved[3], saved[4])
            bases.append(o.frame_flux(0))
        o.p.motion = saved
        self.bases = bases        # [u, v, W] -> (q0x levels, q0y levels)

    def schur(self):
        """The Schur matrix a_times (operators_fluid.F90:14-120) column by column, or with the
        sub-domain method lumat = body + P B^T P^T (operators_struct.F90:840-905)."""
        if self.S is None:
            o = self.o
            if o.sd is not None:
                if o.sd.cols is None:
                    o.sd.precompute()
                self.S = o.sd.lumat(*o.sd.interp())
            else:
                eye = np.eye(o.nf)
                self.S = np.stack([o.a_times(eye[l]) for l in range(o.nf)], axis=1)
        return self.S

    # the transfers of the Schur system: E (q + q0) into its right-hand side and E^T f out of its
    # solution; with the sub-domain method P E_o and E_o^T P^T (timestepper.F90:380-397, 500-516)
    def E(self, qx, qy):
        o = self.o
        if o.sd is not None:
            return o.sd.rhs_add(np.zeros(o.nf), qx, qy, *o.sd.interp())
        return o.regT(qx, qy)

    def ET(self, f):
        o = self.o
        if o.sd is not None:
            return o.sd.spread(f, *o.sd.interp())
        return o.reg(f)

    def frame(self, c):
        qx = [c[0] * self.bases[0][0][k] + c[1] * self.bases[1][0][k] + c[2] * self.bases[2][0][k]
              for k in range(self.o.L)]
        qy = [c[0] * self.bases[0][1][k] + c[1] * self.bases[1][1][k] + c[2] * self.bases[2][1][k]
              for k in range(self.o.L)]
        return qx, qy

    # ------------------------------------------------------------- forward
    def step(self, c):
        """One step (IBOracle.advance with the frame flux of coefficients c); returns the force
        coefficients (nbody, 2) and the tape of what the reverse step reads."""
        o = self.o
        L = o.L
        if o.p.num_stat and o.itime == 0 and o.cholM is None:
            o.preprocess()
        o.itime += 1
        it = o.itime
        q0x, q0y = self.frame(c)
        tape = dict(it=it, omega=[w.copy() for w in o.omega], qx=[q.copy() for q in o.qx],
                    qy=[q.copy() for q in o.qy], q0x=q0x, q0y=q0y)
        zero_ring = np.zeros(o.nbc)
        lastbc = [o.get_bc(o.omega[k + 1], 0.25) for k in range(L - 1)] + [zero_ring]
        tape["lastbc"] = lastbc
        ostar = [None] * L
        for k in range(L - 1, -1, -1):
            omegabc = o.get_bc(ostar[k + 1], 0.25) if k < L - 1 else zero_ring
            nlx, nly = o.nonlinear(o.omega[k], o.qx[k] + q0x[k], o.qy[k] + q0y[k], lastbc[k])
            rhsbc = np.zeros_like(o.omega[k])
            o.apply_bc(rhsbc, lastbc[k], o.vfac[k])
            o.apply_bc(rhsbc, omegabc, o.vfac[k])
            rhs = o.rot(nlx, nly)
            rhs_old = rhs if it == 1 else o.rhs_old[k]
            ostar[k] = o.fluid_predictor(o.omega[k], rhs, rhs_old, rhsbc, k)
            o.rhs_old[k] = rhs
        s, qx, qy = o.vort2flux(ostar)          # coarsifies ostar in place
        tape["ostar_c"] = [w.copy() for w in ostar]
        rhsf = self.E(qx[0] + q0x[0], qy[0] + q0y[0]) + (0.0 - o.delta * o.ub)
        f = o.chol_solve(rhsf) if o.p.num_stat else np.linalg.solve(self.schur(), rhsf)
        hx, hy = self.ET(f)
        ostar[0] = ostar[0] - o.ainv(o.rot(hx, hy))
        o.omega = ostar
        o.s, o.qx, o.qy = o.vort2flux(o.omega)
        o.f = f
        o.f_rdst = o.redistribute(f)
        cx, cy = o.force_coeffs(f)
        return np.stack([cx, cy], axis=1), tape

    def forward(self, coefs):
        """Steps with per-step frame coefficients coefs (N, 3); forces (N, nbody, 2)."""
        self.tapes = []
        out = []
        for c in coefs:
            fc, tape = self.step(c)
            self.tapes.append(tape)
            out.append(fc)
        return np.array(out)

    # ------------------------------------------------------------ transposes
    def ghost_T(self, g):
        o = self.o
        m, n = o.m, o.n
        ring = np.zeros(o.nbc)
        ring[o.left + 1:o.left + n] += g[1:n, 0]
        ring[o.right + 1:o.right + n] += g[1:n, m]
        ring[o.bottom:o.bottom + m + 1] += g[0, :]
        ring[o.top:o.top + m + 1] += g[n, :]
        return g[1:n, 1:m].copy(), ring

    def curl_T(self, lx, ly):
        """(s, ring) adjoint of curl(s, ring)."""
        o = self.o
        m, n = o.m, o.n
        G = np.zeros((n + 1, m + 1))
        G[1:n + 1, :] += lx
        G[0:n, :] -= lx
        G[:, 0:m] += ly
        G[:, 1:m + 1] -= ly
        return self.ghost_T(G)

    def rot_T(self, lam):
        o = self.o
        m, n = o.m, o.n
        hx = np.zeros((n, m + 1))
        hy = np.zeros((n + 1, m))
        hy[1:n, 1:m] += lam
        hy[1:n, 0:m - 1] -= lam
        hx[1:n, 1:m] -= lam
        hx[0:n - 1, 1:m] += lam
        return hx, hy

    def nonlinear_T(self, omega, ux, uy, bc, lx, ly):
        """Adjoints (omega, ux, uy, bc) of nonlinear(omega, ux, uy, bc) at (lx, ly)."""
        o = self.o
        m, n = o.m, o.n
        W = o.ghost_vertex(omega, bc)
        QX = np.zeros((n + 2, m + 1)); QX[1:n + 1] = ux
        QY = np.zeros((n + 1, m + 2)); QY[:, 1:m + 1] = uy
        U = 0.5 * (QX[1:n + 2] + QX[0:n + 1])
        V = 0.5 * (QY[:, 1:m + 2] + QY[:, 0:m + 1])
        lW = np.zeros_like(W); lU = np.zeros_like(U); lV = np.zeros_like(V)
        lV[1:n + 1] += 0.5 * lx * W[1:n + 1]
        lV[0:n] += 0.5 * lx * W[0:n]
        lW[1:n + 1] += 0.5 * lx * V[1:n + 1]
        lW[0:n] += 0.5 * lx * V[0:n]
        lU[:, 1:m + 1] += -0.5 * ly * W[:, 1:m + 1]
        lU[:, 0:m] += -0.5 * ly * W[:, 0:m]
        lW[:, 1:m + 1] += -0.5 * ly * U[:, 1:m + 1]
        lW[:, 0:m] += -0.5 * ly * U[:, 0:m]
        lQX = np.zeros_like(QX); lQY = np.zeros_like(QY)
        lQX[1:n + 2] += 0.5 * lU
        lQX[0:n + 1] += 0.5 * lU
        lQY[:, 1:m + 2] += 0.5 * lV
        lQY[:, 0:m + 1] += 0.5 * lV
        lom, lbc = self.ghost_T(lW)
        return lom, lQX[1:n + 1].copy(), lQY[:, 1:m + 1].copy(), lbc

    def get_bc_T(self, ring, fac):
        o = self.o
        m, n = o.m, o.n
        r = ring * fac
        ls = np.zeros((n - 1, m - 1))
        i0, i1 = m // 4 + 1, 3 * m // 4 + 1
        j0, j1 = n // 4 + 1, 3 * n // 4 + 1
        ii = np.arange(i0, i1 + 1)
        jj = np.arange(j0, j1 + 1)
        for base, jrow in ((o.bottom, j0), (o.top, j1)):
            lline = np.zeros(len(ii))
            lline += r[base + 2 * (ii - 1 - m // 4)]
            mid = r[base + 2 * (ii[:-1] - 1 - m // 4) + 1]
            lline[:-1] += 0.5 * mid
            lline[1:] += 0.5 * mid
            ls[jrow - 2, ii - 2] += lline
        for base, icol in ((o.left, i0), (o.right, i1)):
            lline = np.zeros(len(jj))
            lline += r[base + 2 * (jj - 1 - n // 4)]
            mid = r[base + 2 * (jj[:-1] - 1 - n // 4) + 1]
            lline[:-1] += 0.5 * mid
            lline[1:] += 0.5 * mid
            ls[jj - 2, icol - 2] += lline
        return ls

    def apply_bc_T(self, lvort, fac):
        o = self.o
        m, n = o.m, o.n
        ring = np.zeros(o.nbc)
        ring[o.left + 1:o.left + n] += fac * lvort[:, 0]
        ring[o.right + 1:o.right + n] += fac * lvort[:, m - 2]
        ring[o.bottom + 1:o.bottom + m] += fac * lvort[0, :]
        ring[o.top + 1:o.top + m] += fac * lvort[n - 2, :]
        return ring

    def coarsify_T(self, lfine, lcoarse):
        """In place: the coarse centre's adjoint spread onto the fine field, then cleared."""
        o = self.o
        m, n = o.m, o.n
        lv = lcoarse[n // 4: 3 * n // 4 - 1, m // 4: 3 * m // 4 - 1].copy()
        lcoarse[n // 4: 3 * n // 4 - 1, m // 4: 3 * m // 4 - 1] = 0.0
        cI = slice(1, m - 2, 2); cJ = slice(1, n - 2, 2)
        pI = slice(2, m - 1, 2); mI = slice(0, m - 3, 2)
        pJ = slice(2, n - 1, 2); mJ = slice(0, n - 3, 2)
        lfine[cJ, cI] += lv
        for (J, I) in ((cJ, pI), (pJ, cI), (cJ, mI), (mJ, cI)):
            lfine[J, I] += 0.5 * lv
        for (J, I) in ((pJ, pI), (mJ, pI), (mJ, mI), (pJ, mI)):
            lfine[J, I] += 0.25 * lv

    def coarsify_chain_T(self, lam):
        for k in range(self.o.L - 1, 0, -1):
            self.coarsify_T(lam[k - 1], lam[k])

    def vsolve_T(self, lqx, lqy):
        """Adjoint of vort2flux's solves (after its coarsify): (qx, qy) levels -> omega levels."""
        o = self.o
        L = o.L
        lom = [None] * L
        lsbc_from_finer = None     # adjoint of the ring level k-1 read (get_bc of s_k)
        for k in range(L):
            ls, lring_curl = self.curl_T(lqx[k], lqy[k])
            if k > 0:
                ls = ls + self.get_bc_T(lsbc_from_finer, 1.0)
            lv2 = o.ctci(ls)
            lom[k] = lv2
            if k < L - 1:
                lsbc_from_finer = self.apply_bc_T(lv2, 1.0) + lring_curl
        return lom

    def fluid_predictor_T(self, lam, k):
        """Adjoints (omega, rhs, rhs_old, rhsbc) of fluid_predictor at level k."""
        o = self.o
        linner = o.lam1i[k] * o.dst(lam)
        lsum = o.dst(linner)
        return o.dst(o.lam1[k] * linner), o.con1[k] * lsum, o.con2[k] * lsum, lsum

    # ------------------------------------------------------------- reverse
    def step_T(self, tape, lom, lqx, lqy, lro, lforce):
        """Reverse of one step: the adjoints of its outputs (omega, qx, qy, rhs_old levels; the
        force coefficients (nbody, 2)) -> the adjoints of its inputs and of its frame
        coefficients (3)."""
        o = self.o
        L = o.L
        it = tape["it"]
        # final vort2flux: coarsify, then the solves
        lw = [a.copy() for a in lom]
        extra = self.vsolve_T(lqx, lqy)
        for k in range(L):
            lw[k] = lw[k] + extra[k]
        self.coarsify_chain_T(lw)
        # correction: omega_0 - ainv(rot(reg f))
        lf = np.zeros(o.nf)
        g = o.ainv(lw[0])
        hx, hy = self.rot_T(g)
        lf -= self.E(hx, hy)
        scale = 2.0 * o.delta / o.p.dt
        for kf in range(o.nf):
            lf[kf] += scale * lforce[o.bid[kf], 0 if o.comp[kf] == 1 else 1]
        lrhsf = o.chol_solve(lf) if o.p.num_stat else np.linalg.solve(self.schur().T, lf)
        # rhsf = regT(q*_0 + q0_0): the adjoint fluxes on level 0
        ax, ay = self.ET(lrhsf)
        lq0x = [np.zeros_like(b) for b in tape["q0x"]]
        lq0y = [np.zeros_like(b) for b in tape["q0y"]]
        lq0x[0] += ax
        lq0y[0] += ay
        zx = [np.zeros_like(q) for q in tape["qx"]]
        zy = [np.zeros_like(q) for q in tape["qy"]]
        zx[0] = ax
        zy[0] = ay
        lostar = self.vsolve_T(zx, zy)
        for k in range(L):
            lostar[k] = lostar[k] + lw[k]
        self.coarsify_chain_T(lostar)
        # predictor, level k after its coarser neighbour in the forward: reverse fine to coarse
        lomega = [np.zeros_like(w) for w in tape["omega"]]
        lqx_in = [np.zeros_like(q) for q in tape["qx"]]
        lqy_in = [np.zeros_like(q) for q in tape["qy"]]
        lro_in = [np.zeros_like(r) for r in lro]
        for k in range(L):
            lo, lrhs, lrold, lrb = self.fluid_predictor_T(lostar[k], k)
            lomega[k] += lo
            lrhs = lrhs + lro[k]
            if it == 1:
                lrhs = lrhs + lrold
            else:
                lro_in[k] += lrold
            lbc_last = self.apply_bc_T(lrb, o.vfac[k])
            lbc_omega = self.apply_bc_T(lrb, o.vfac[k])
            if k < L - 1:
                lostar[k + 1] += self.get_bc_T(lbc_omega, 0.25)
            lnx, lny = o.curl(lrhs, np.zeros(o.nbc))
            om, lux, luy, lbc_nl = self.nonlinear_T(tape["omega"][k], tape["qx"][k] + tape["q0x"][k],
                                                    tape["qy"][k] + tape["q0y"][k], tape["lastbc"][k], lnx, lny)
            lomega[k] += om
            lqx_in[k] += lux
            lqy_in[k] += luy
            lq0x[k] += lux
            lq0y[k] += luy
            if k < L - 1:
                lomega[k + 1] += self.get_bc_T(lbc_last + lbc_nl, 0.25)
        lc = np.zeros(3)
        for i in range(3):
            for k in range(L):
                lc[i] += np.sum(lq0x[k] * self.bases[i][0][k]) + np.sum(lq0y[k] * self.bases[i][1][k])
        return lomega, lqx_in, lqy_in, lro_in, lc

    def backward(self, lforces):
        """Adjoints of the per-step frame coefficients (N, 3) for force adjoints (N, nbody, 2)."""
        o = self.o
        L = o.L
        lom = [np.zeros_like(w) for w in o.omega]
        lqx = [np.zeros_like(q) for q in o.qx]
        lqy = [np.zeros_like(q) for q in o.qy]
        lro = [np.zeros_like(r) for r in o.rhs_old]
        out = np.zeros((len(self.tapes), 3))
        for n in range(len(self.tapes) - 1, -1, -1):
            lom, lqx, lqy, lro, out[n] = self.step_T(self.tapes[n], lom, lqx, lqy, lro, lforces[n])
        return out
