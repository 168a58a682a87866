// Device bodies shared by the per-stage kernels of the FSI iteration (structure update,
// delta-function weights, influence patches) and the device FSI loop's fused kernel, so that
// both evaluate the same arithmetic.
#pragma once
#include "kernels.cuh"

namespace ib {

// Smoothed 6-point delta function.  Literals without a d exponent in the Fortran
// source are default REAL, i.e. single precision: they appear as float literals.
__device__ inline double deltafnc_dev(double x1, double x2, double dr) {
  double r = fabs(x1 - x2);
  double r1 = r / dr;
  double r2 = r1 * r1;
  double r3 = r2 * r1;
  double r4 = r3 * r1;
  const double s3 = sqrt(3.0);
  double v;
  if (r1 <= 1.0) {
    double a5 = asin((1.0 / 2.0) * s3 * (2.0 * r1 - 1.0));
    double a8 = sqrt(1.0 - 12.0 * r2 + 12.0 * r1);
    v = 0.4166666667e-1 * r4 + ((double)(-.1388888889f) + 0.3472222222e-1 * a8) * r3 +
        (-0.7121664902e-1 - 0.5208333333e-1 * a8 + (double)(0.2405626122f) * a5) * r2 +
        (-(double)(.2405626122f) * a5 - (double)(.3792313933f) + (double)(.1012731481f) * a8) * r1 +
        0.8018753741e-1 * a5 - 0.4195601852e-1 * a8 + (double)(.6485698427f);
  } else if (r1 <= 2.0) {
    double a6 = asin((1.0 / 2.0) * s3 * (-3.0 + 2.0 * r1));
    double a9 = sqrt(-23.0 + 36.0 * r1 - 12.0 * r2);
    v = -0.6250000000e-1 * r4 + ((double)(.4861111111f) - 0.1736111111e-1 * a9) * r3 +
        ((double)(-1.143175026f) + 0.7812500000e-1 * a9 - (double)(.1202813061f) * a6) * r2 +
        ((double)(.8751991178f) + (double)(.3608439183f) * a6 - (double)(.1548032407f) * a9) * r1 -
        (double)(.2806563809f) * a6 + 0.822848104e-2 + (double)(.1150173611f) * a9;
  } else if (r1 <= 3.0) {
    double a1 = asin((1.0 / 2.0 * (2.0 * r1 - 5.0)) * s3);
    double a7 = sqrt(-71.0 - 12.0 * r2 + 60.0 * r1);
    v = 0.2083333333e-1 * r4 + (0.3472222222e-2 * a7 - (double)(.2638888889f)) * r3 +
        ((double)(1.214391675f) - 0.2604166667e-1 * a7 + 0.2405626122e-1 * a1) * r2 +
        (-(double)(.1202813061f) * a1 - (double)(2.449273192f) + 0.7262731481e-1 * a7) * r1 +
        (double)(.1523563211f) * a1 + (double)(1.843201677f) - 0.7306134259e-1 * a7;
  } else {
    v = 0.0;
  }
  return v / dr;
}

// compute_dx + update_xb (operators_struct.F90:402-505, 600-620) of torsional body t, the
// scalar part, on one whole warp: BR . f from lane-strided partials joined by an xor tree and
// the Newmark update of theta (with the body's step constants); g = gamma0 - theta_new, whose
// sin and cos the caller evaluates.  Every lane returns the same.
struct TorsDx {
  double thn, dth, g;
};
__device__ __forceinline__ TorsDx tors_dx_warp(const TorsBody& b, const TorsState& s, int t,
                                               const double* __restrict__ f) {
  const int lane = threadIdx.x & 31;
  const double th = s.theta[t], th0 = s.theta0[t], thd0 = s.thetad0[t], thdd0 = s.thetadd0[t];
  const double I = b.itheta, C = b.ctheta;
  const double sn0 = s.sinv[t], cs0 = s.cosv[t];
  double part = 0.0;
  for (int j = lane; j < 2 * b.npts; j += 32) part += br_val(b, sn0, cs0, j) * f[b.off + j];
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  double brf = 0.0 + part;
  const double jr = b.keff_inv * (I * (b.a44 * th0 + b.a4 * thd0 + thdd0) + C * (thd0 + b.a2 * th0) - b.keff * th);
  brf = b.bq * brf * b.bs;
  TorsDx u;
  u.dth = jr + brf;
  u.thn = th + u.dth;
  u.g = b.gamma0 - u.thn;
  return u;
}
// The new velocity and acceleration of the Newmark update.
__device__ __forceinline__ void tors_rates(const TorsBody& b, double thn, double th0, double thd0, double thdd0,
                                           double* thd, double* thdd) {
  *thd = -thd0 + b.a2 * (thn - th0);
  *thdd = -thdd0 - b.a4 * thd0 + b.a44 * (thn - th0);
}
// Position of unknown idx (0..2 npts-1) of a torsional body at sin, cos (gamma0 - theta).
// Each product and the sum are rounded separately, as update_xb writes them
// (operators_struct.F90:600-620): the positions decide which side of a stencil edge a grid
// point falls on.
__device__ __forceinline__ double2 tors_point(const TorsBody& b, int idx, double sg, double cg) {
  const int j = idx < b.npts ? idx : idx - b.npts;
  const double r = __dmul_rn((double)j, b.deltas);
  return make_double2(__dadd_rn(b.xbf0, __dmul_rn(r, cg)), __dadd_rn(b.ybf0, __dmul_rn(r, sg)));
}

// Stencil origins and the 49 weights (l outer, p inner) of the 8 unknowns k0..k0+7 on one CTA
// of 4 warps, from their positions pos[u] = (x, y).  With phi the fractional position of a
// point in its cell, the 7 stencil offsets q sit at distances |q - 3 - phi| (in cells), so
// offsets {3,4}, {2,5} and {1,6} fall in the first, second and third piece of the delta
// function and offset 0 at its edge.  Warp w evaluates one offset pair for the x and y factors
// of all 8 unknowns, so its lanes take one branch of the FP64-latency-bound evaluation instead
// of all three; the factors meet in shared memory for the products.  Writes the weights to w
// (and wsm[u][.] when given), the origins to ix, iy (and org[u][.]); stale |= 1 when an origin
// moved; err = IB_ERR_DOMAIN when a stencil leaves the grid.  Ends with a CTA barrier.
__device__ __forceinline__ void reg_weights_cta(const GridDims& g, int nf, int k0, const double (*pos)[2], double d,
                                                double ox, double oy, const int* __restrict__ comp, int* ix, int* iy,
                                                double* w, int* stale, int* err, double (*fac)[7],
                                                double (*wsm)[49], int (*org)[2]) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double d2 = 0.5 * d;
  int pi, q;
  if (warp < 3) {
    pi = lane >> 1;
    const int lo = 3 - warp, hi = 4 + warp;   // {3,4}, {2,5}, {1,6}
    q = (lane & 1) ? hi : lo;
  } else {
    pi = lane;
    q = 0;
  }
  const int u = pi >> 1, k = k0 + u, axis = pi & 1;
  if (pi < 16 && k < nf) {
    const double xk = pos[u][0], yk = pos[u][1];
    const int cx = (int)((xk + ox) / d) + 1;   // Fortran INT truncates toward zero
    const int cy = (int)((yk + oy) / d) + 1;
    const bool isx = comp[k] == 1;
    const int off = q - 3;
    double fv;
    // The grid coordinate is rounded after the product and again after the sum, as the
    // reference's expression delta*(indexx-1+p)-offsetx is (grid.F90:459-528): the delta
    // function is discontinuous at 3 cells (its single-precision constants leave about 1e-8
    // there), so a point on a grid line (e.g. x = 0 with offsetx = 1, delta = 0.02) must see
    // the same side of that edge, which a fused multiply-add could change by one rounding.
    if (axis == 0) {
      double x = __dsub_rn(__dmul_rn(d, (double)(cx - 1 + off)), ox);
      if (!isx) x = __dadd_rn(x, d2);
      fv = deltafnc_dev(x, xk, d);
    } else {
      double y = __dsub_rn(__dmul_rn(d, (double)(cy - 1 + off)), oy);
      if (isx) y = __dadd_rn(y, d2);
      fv = deltafnc_dev(y, yk, d);
    }
    fac[pi][q] = fv;
    if (warp == 3 && axis == 0) {
      // the contribution lists depend on the stencil origins only: rebuild them when one moved
      if (ix[k] != cx || iy[k] != cy) atomicOr(stale, 1);
      ix[k] = cx;
      iy[k] = cy;
      if (org) {
        org[u][0] = cx;
        org[u][1] = cy;
      }
      // faces touched: u-face i in [1,m+1], j in [1,n]; v-face i in [1,m], j in [1,n+1]
      const int imax = isx ? g.m + 1 : g.m, jmax = isx ? g.n : g.n + 1;
      if (cx - 3 < 1 || cx + 3 > imax || cy - 3 < 1 || cy + 3 > jmax) atomicExch(err, IB_ERR_DOMAIN);
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < 8 * 49; t += blockDim.x) {
    const int uu = t / 49, sl = t - uu * 49;
    if (k0 + uu >= nf) break;
    const int l = sl / 7, p = sl - l * 7;
    const double wv = d * d * fac[2 * uu][p] * fac[2 * uu + 1][l];
    w[(size_t)(k0 + uu) * 49 + sl] = wv;
    if (wsm) wsm[uu][sl] = wv;
  }
  __syncthreads();
}

// Entry q (of 64) of unknown k's influence patch: rot(E^T e_k) on the vertices
// I in [cx-3, cx+4], J in [cy-3, cy+4], with the vertex's index in the band (tiles of
// tile x tile vertices).  flag |= 1 when the vertex lies outside the band, |= 2 when it is
// not an interior vertex (its streamfunction would come from the boundary ring).
__device__ __forceinline__ void patch_entry(const GridDims& g, int k, int q, bool isx, int cx, int cy,
                                            const double* wk, const int* __restrict__ tile_of, int ntx, int tile,
                                            double* __restrict__ pval, int* __restrict__ pidx, int* __restrict__ used,
                                            int* __restrict__ flag) {
  const int di = q & 7, dj = q >> 3;
  auto W = [&](int p, int l) -> double {
    return (p >= -3 && p <= 3 && l >= -3 && l <= 3) ? wk[(l + 3) * 7 + (p + 3)] : 0.0;
  };
  const int p = di - 3, l = dj - 3;
  // rot (operators_fluid.F90:203-233) of the spread unit force: a u-face (i,j) adds -1 to
  // vertex (i,j) and +1 to (i,j+1); a v-face adds +1 to (i,j) and -1 to (i+1,j)
  double v = isx ? W(p, l - 1) - W(p, l) : W(p, l) - W(p - 1, l);
  const int a = cx - 3 + di - 2, b = cy - 3 + dj - 2;   // 0-based interior vertex
  int idx = -1, fl = 0;
  if (a < 0 || a >= g.nsx || b < 0 || b >= g.nsy) {
    fl = 2;
  } else if (!tile_of) {
    fl = 1;
  } else {
    const int t = tile_of[(b / tile) * ntx + a / tile];
    if (t < 0) fl = 1;
    else idx = t * 64 + (b % tile) * tile + (a % tile);
  }
  if (idx < 0) v = 0.0;
  pval[(size_t)k * 64 + q] = v;
  pidx[(size_t)k * 64 + q] = idx;
  if (idx >= 0) used[idx] = 1;
  if (fl) atomicOr(flag, fl);
}

}  // namespace ib
