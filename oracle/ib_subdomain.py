"""CPU oracle of the sub-domain precomputed-Schur method -- TEST INFRASTRUCTURE ONLY.

Restates, for one rank, the reference's ``sub_domain = T`` path (Nair & Goza's accelerator):

* the point cloud (grid.F90:320-352): with ``sub_domain_full_rectangular = F`` the points of the
  stationary rigid bodies first, then the rectangle [sdxi, sdxe] x [sdyi, sdye] at spacing
  delta_sd, x fastest; nb_sd points, nf_sd = 2 nb_sd unknowns (x components, then y;
  collect_subdomain, grid.F90:437-455);
* E_o, the delta-function weights of those unknowns (setup_pre_reg_subdomain, grid.F90:627-693);
* the sparsity of E E^T with a 21 x 21 support (get_sparsity_EEt, variables.F90:528-607;
  setup_subdomain_sparsity, grid.F90:697-753): column j of B is evaluated on the unknowns whose
  21 x 21 face blocks overlap j's, x components then y components;
* B, column by column: a_times_sd (operators_fluid.F90:124-199) of the unit vector, then the drop
  tolerance |B_ij| > droptol B_jj, droptol the single-precision literal 7.0e-3 (grid.F90:14;
  preprocess_sd, timestepper.F90:602-770), written to / read from ``sd_precomputed.chd``;
* P, bilinear interpolation (interp_points = 4, grid.F90:13) from the sub-domain unknowns to the
  body unknowns with the 2-point hat function deltafnc2 (grid.F90:1007-1029), exact for the
  points of a stationary rigid body that are themselves sub-domain points
  (setup_reg_subdomain_indices, grid.F90:777-951);
* each FSI iteration: lumat = body_mat + P B^T P^T (compute_operator, operators_struct.F90:840-
  905; body_mat, operators_struct.F90:909-980), the right-hand side P E_o q added to the
  structure's (timestepper.F90:368-405), GMRES on lumat; the correction spreads E_o^T P^T f
  (timestepper.F90:500-516).

The reference assumes one stationary rigid body when its points lead the cloud (its exact
mapping takes the body point's force index for its point index, grid.F90:836-848); here rigid
point p of the bodies in file order maps to sub-domain point p, which is the same for one body.
The E E^T sparsity is formed from linear face indices without bounds (grid.F90:724-731), so the
library and this oracle require every point's 21 x 21 block inside the grid.
"""
from __future__ import annotations

import math
import struct

import numpy as np

DROPTOL = float(np.float32(7.0e-3))   # grid.F90:14 (default REAL literal)
SUPPORT_NZ = 10                        # variables.F90:537
INTERP_POINTS = 4                      # grid.F90:13


def _nint(v: float) -> int:
    """Fortran NINT (round half away from zero)."""
    return int(math.floor(v + 0.5)) if v >= 0 else -int(math.floor(-v + 0.5))


def deltafnc2(x1, x2, dr):
    """grid.F90:1007-1029: the 2-point hat function, same operation order."""
    r = np.abs(np.asarray(x1, dtype=np.float64) - np.asarray(x2, dtype=np.float64))
    r1 = r / dr
    d = np.where(r1 <= 1.0, 1.0 - r1, 0.0)
    return d / dr


class SubDomain:
    def __init__(self, o, full_rectangular, sdxi, sdxe, sdyi, sdye, delta_sd):
        self.o = o
        self.full_rectangular = bool(full_rectangular)
        self.sdxi, self.sdxe, self.sdyi, self.sdye, self.dsd = sdxi, sdxe, sdyi, sdye, delta_sd
        self.nx = _nint((sdxe - sdxi) / delta_sd + 1)
        self.ny = _nint((sdye - sdyi) / delta_sd + 1)
        xs, ys = [], []
        # rigid body points first (grid.F90:329-338); rigid[k] = sub-domain point of body unknown k
        self.rigid_pt = np.full(o.nf, -1, dtype=np.int64)
        if not self.full_rectangular:
            pt = 0
            for ib, b in enumerate(o.bodies):
                if b.fam != 1:
                    continue
                off = o.body_off[ib]
                for i in range(b.npts):
                    xs.append(float(b.x[i])); ys.append(float(b.y[i]))
                    self.rigid_pt[off + i] = pt
                    self.rigid_pt[off + b.npts + i] = pt
                    pt += 1
        self.nr_sd = len(xs)
        for j in range(1, self.ny + 1):
            for i in range(1, self.nx + 1):
                xs.append(sdxi + (i - 1) * delta_sd)
                ys.append(sdyi + (j - 1) * delta_sd)
        self.px = np.array(xs); self.py = np.array(ys)
        self.nb_sd = len(xs)
        self.nf_sd = 2 * self.nb_sd
        self.ux = np.concatenate([self.px, self.px])
        self.uy = np.concatenate([self.py, self.py])
        self.ucomp = np.concatenate([np.ones(self.nb_sd, np.int64), np.full(self.nb_sd, 2, np.int64)])
        self.idx, self.w = o.reg_weights(self.ux, self.uy, self.ucomp)
        d, ox, oy = o.delta, o.p.offsetx, o.p.offsety
        self.gix = ((self.px + ox) / d).astype(np.int64) + 1
        self.giy = ((self.py + oy) / d).astype(np.int64) + 1
        if (self.gix.min() < SUPPORT_NZ + 1 or self.gix.max() > o.m - SUPPORT_NZ or
                self.giy.min() < SUPPORT_NZ + 1 or self.giy.max() > o.n - SUPPORT_NZ):
            raise ValueError("sub-domain points too close to the domain boundary")
        # candidate rows per point: every point whose 21 x 21 block meets this one's
        self.cand = []
        for k in range(self.nb_sd):
            sel = np.nonzero((np.abs(self.gix - self.gix[k]) <= 2 * SUPPORT_NZ) &
                             (np.abs(self.giy - self.giy[k]) <= 2 * SUPPORT_NZ))[0]
            self.cand.append(sel)
        self.cols = None   # per unknown j: (rows, values) of column j of B after the drop

    def rows_of(self, j):
        """Candidate rows of column j (0-based unknowns): x components, then y components."""
        c = self.cand[j % self.nb_sd]
        return np.concatenate([c, c + self.nb_sd])

    # -------------------------------------------------------------- precompute
    def column(self, j):
        """a_times_sd (operators_fluid.F90:124-199) of the unit vector e_j, on every unknown."""
        o = self.o
        e = np.zeros(self.nf_sd)
        e[j] = 1.0
        hx, hy = o.reg_with(self.idx, self.w, self.ucomp, e)
        vort = [np.zeros_like(o.omega[0]) for _ in range(o.L)]
        vort[0] = o.ainv(o.rot(hx, hy))
        _, qx, qy = o.vort2flux(vort)
        return o.regT_with(self.idx, self.w, self.ucomp, qx[0], qy[0])

    def precompute(self, columns=None):
        """preprocess_sd (timestepper.F90:608-737): every column on its candidate rows, then the
        drop tolerance against the diagonal.  columns: evaluate only these (the others None)."""
        self.cols = [None] * self.nf_sd
        for j in (range(self.nf_sd) if columns is None else columns):
            self.cols[j] = self.drop(j, self.column(j))

    def drop(self, j, full):
        rows = self.rows_of(j)
        vals = full[rows]
        keep = np.abs(vals) > DROPTOL * full[j]
        return rows[keep], vals[keep]

    def write_chd(self, path):
        """The sd_precomputed.chd records of timestepper.F90:691-695, 753-756: per column one
        record with its count, one with its values then its 1-based row indices (PetscInt,
        32-bit); Fortran unformatted sequential (4-byte length markers)."""
        out = bytearray()
        for rows, vals in self.cols:
            rec = struct.pack("<i", len(rows))
            out += struct.pack("<i", len(rec)) + rec + struct.pack("<i", len(rec))
            rec = vals.astype("<f8").tobytes() + (rows + 1).astype("<i4").tobytes()
            out += struct.pack("<i", len(rec)) + rec + struct.pack("<i", len(rec))
        with open(path, "wb") as fh:
            fh.write(bytes(out))

    def read_chd(self, path):
        """The reader of timestepper.F90:740-757."""
        data = open(path, "rb").read()
        pos = 0
        cols = []

        def record():
            nonlocal pos
            n = struct.unpack_from("<i", data, pos)[0]
            body = data[pos + 4:pos + 4 + n]
            if struct.unpack_from("<i", data, pos + 4 + n)[0] != n:
                raise ValueError("bad record marker")
            pos += 8 + n
            return body

        for _ in range(self.nf_sd):
            nz = struct.unpack("<i", record())[0]
            body = record()
            vals = np.frombuffer(body[:8 * nz], dtype="<f8").copy()
            rows = np.frombuffer(body[8 * nz:12 * nz], dtype="<i4").astype(np.int64) - 1
            cols.append((rows, vals))
        self.cols = cols

    def dense(self):
        """B as a dense nf_sd x nf_sd matrix (zero where dropped or outside the pattern)."""
        B = np.zeros((self.nf_sd, self.nf_sd))
        for j, (rows, vals) in enumerate(self.cols):
            B[rows, j] = vals
        return B

    # ---------------------------------------------------------- interpolation
    def interp(self):
        """setup_reg_subdomain_indices (grid.F90:777-873) at the current body positions: the 4
        sub-domain unknowns (0-based) and weights of each body unknown."""
        o = self.o
        nf = o.nf
        idx = np.zeros((nf, INTERP_POINTS), dtype=np.int64)
        wts = np.zeros((nf, INTERP_POINTS))
        dsd = self.dsd
        for k in range(nf):
            xb, yb = float(o.xb[k]), float(o.yb[k])
            isx = o.comp[k] == 1
            if self.rigid_pt[k] >= 0:
                p0 = int(self.rigid_pt[k])
                nn = [p0, p0 + 1, p0 + 1, p0 + 1]   # the body point itself, then dummies
                dist = [0.0, 1.0, 1.0, 1.0]
            else:
                fx = (xb - self.sdxi) / dsd + 1
                fy = (yb - self.sdyi) / dsd + 1
                ll = [int(fx), int(fx) + 1]
                pp = [int(fy), int(fy) + 1]
                nn, dist = [], []
                for l in range(2):
                    for p in range(2):
                        if ll[l] < 1 or ll[l] > self.nx or pp[p] < 1 or pp[p] > self.ny:
                            raise ValueError("body has left the sub-domain")
                        q = self.nr_sd + (pp[p] - 1) * self.nx + ll[l] - 1
                        dx = xb - self.px[q]
                        dy = yb - self.py[q]
                        nn.append(q)
                        dist.append(math.sqrt(dx ** 2 + dy ** 2))
            w = [0.0] * 4
            mk = [True] * 4
            for i in range(4):
                q = nn[i]
                w[i] = float(dsd * dsd * deltafnc2(self.px[q], xb, dsd) * deltafnc2(self.py[q], yb, dsd))
                if dist[i] == 0.0:
                    w[i] = 1.0
                    mk[i] = False
            if not all(mk):
                w = [0.0 if mk[i] else w[i] for i in range(4)]
            idx[k] = [q if isx else q + self.nb_sd for q in nn]
            wts[k] = w
        return idx, wts

    # ------------------------------------------------------- FSI iteration
    def lumat(self, idx, wts):
        """compute_operator (operators_struct.F90:840-905): body_mat + P B^T P^T, where
        lumat(k, i) = body + sum_a P(k,a) sum_b P(i,b) B(b, a), each dot product in order; B's
        columns are read from their kept rows (zero elsewhere)."""
        o = self.o
        nf = o.nf
        body = np.zeros((nf, nf))
        for l in range(nf):
            e = np.zeros(nf); e[l] = 1.0
            body[:, l] = o.b_times(e)
        cols = {}
        for a in np.unique(idx):
            rows, vals = self.cols[a]
            cols[int(a)] = dict(zip(rows.tolist(), vals.tolist()))
        inter = {}   # inter[a][i] = sum_r B(b_r(i), a) P(i, r)
        for a, col in cols.items():
            v = np.zeros(nf)
            for i in range(nf):
                acc = 0.0
                for r in range(4):
                    acc = acc + col.get(int(idx[i, r]), 0.0) * wts[i, r]
                v[i] = acc
            inter[a] = v
        M = np.zeros((nf, nf))
        for k in range(nf):
            acc = np.zeros(nf)
            for q in range(4):
                acc = acc + wts[k, q] * inter[int(idx[k, q])]
            M[k] = body[k] + acc
        return M

    def rhs_add(self, rhsf, qhx, qhy, idx, wts):
        """timestepper.F90:380-397: rhsf(j) = P_j . (E_o (q + q0)) + rhsf(j)."""
        o = self.o
        e = o.regT_with(self.idx, self.w, self.ucomp, qhx, qhy)
        dot = np.zeros(o.nf)
        for q in range(4):
            dot = dot + wts[:, q] * e[idx[:, q]]
        return dot + rhsf

    def spread(self, f, idx, wts):
        """timestepper.F90:500-516: E_o^T (P^T f); P^T f summed over the body unknowns in order."""
        o = self.o
        fsd = np.zeros(self.nf_sd)
        for k in range(o.nf):
            for q in range(4):
                fsd[idx[k, q]] += wts[k, q] * f[k]
        return o.reg_with(self.idx, self.w, self.ucomp, fsd)
