// The sub-domain precomputed-Schur method (sub_domain = T; Nair & Goza's accelerator):
// grid.F90:320-352 (the point cloud), 572-951 (E_o, E E^T's sparsity, P), timestepper.F90:79-97,
// 368-405, 500-516, 602-770 (precompute, FSI iteration, correction), operators_struct.F90:840-
// 980 (compute_operator, body_mat), operators_fluid.F90:124-199 (a_times_sd).
//
//   * Points: the stationary rigid bodies' points first when the cloud is not fully rectangular
//     (rigid point p of the bodies in file order is sub-domain point p: the reference assumes
//     one such body, for which the two agree), then the rectangle [sdxi, sdxe] x [sdyi, sdye] at
//     spacing dsd, x fastest.  Unknowns: every point's x component, then every y component.
//   * B = E_o curl G rot E_o^T between the unknowns (the fluid part of the Schur operator, G the
//     vorticity-to-streamfunction map), column j evaluated on the unknowns whose 21 x 21 face
//     blocks meet j's (E E^T's sparsity with support 10), then thinned: row i is kept when
//     |B_ij| > droptol B_jj, droptol the single-precision literal 7.0e-3.  Each column is one
//     application of the fluid part to the spread unit force of unknown j: the band build's
//     truncated multi-level solve on a scratch set, then E_o (curl s) on the candidate rows;
//     the columns run on the band build's concurrent sets, each set's columns as one captured
//     while-loop graph.
//   * P: bilinear interpolation (4 points, the 2-point hat function deltafnc2) from the
//     sub-domain unknowns to each body unknown at its current position; exact for a stationary
//     rigid body's points.  Every FSI iteration: lumat = body + P B^T P^T into the solver's
//     column-major operator, rhsf = P E_o (q + q0) + rhsf, GMRES on lumat; the correction
//     spreads E_o^T P^T f.
// The arithmetic the reference writes without fused multiply-adds (the hat weights, the dot
// products of P) is rounded step by step here too.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.cuh"

namespace ib {

namespace {

constexpr int kSupportNz = 10;   // get_sparsity_EEt's support (variables.F90:537)
constexpr int kInterp = 4;       // interp_points (grid.F90:13): bilinear
constexpr int kPatch = 64;       // vertices of rot E^T of one unknown (8 x 8)
const double kDropTol = (double)7.0e-3f;   // droptol (grid.F90:14), a default-REAL literal

int fortran_nint(double v) { return v >= 0 ? (int)std::floor(v + 0.5) : -(int)std::floor(-v + 0.5); }

// ------------------------------------------------------------------------- precompute
__global__ void k_sd_col_init(int* col, int c0) {
  IB_GRID_DEP_WAIT();
  if (threadIdx.x == 0) *col = c0;
}

__global__ void k_sd_col_next(int* col, int stride, int ncol, cudaGraphConditionalHandle h) {
  IB_GRID_DEP_WAIT();
  if (threadIdx.x != 0) return;
  const int c = *col + stride;
  *col = c;
  cudaGraphSetConditional(h, c < ncol ? 1u : 0u);
}

// The vorticity of unknown *col's spread unit force, rot E_o^T e_j (a u-face (i,j) adds -1 to
// vertex (i,j) and +1 to (i,j+1); a v-face +1 to (i,j) and -1 to (i+1,j)), after the previous
// column's patch is cleared (64 threads); and the row ranges of the multi-level solve: the
// forward transform's input rows, ainv's response within R rows of them, and on each coarser
// level the rows coarsify fills from those.
__global__ void k_sd_source(const int* col, const int* __restrict__ comp, const int* __restrict__ ix,
                            const int* __restrict__ iy, const double* __restrict__ w, GridDims g, double* vort,
                            int* prev, int* rr_in, int* rr_lv, int* box, int* strip, int L, int R) {
  IB_GRID_DEP_WAIT();
  const int q = threadIdx.x;
  const int u = *col;
  const int pv = prev[q];
  if (pv >= 0) vort[pv] = 0.0;
  __syncthreads();
  const bool isx = comp[u] == 1;
  const int cx = ix[u], cy = iy[u];
  const double* wk = w + (size_t)u * 49;
  const int di = q & 7, dj = q >> 3;
  const int p = di - 3, l = dj - 3;
  auto W = [&](int pp, int ll) -> double {
    return (pp >= -3 && pp <= 3 && ll >= -3 && ll <= 3) ? wk[(ll + 3) * 7 + (pp + 3)] : 0.0;
  };
  const double v = isx ? W(p, l - 1) - W(p, l) : W(p, l) - W(p - 1, l);
  const int a = cx - 5 + di, b = cy - 5 + dj;   // 0-based interior vertex
  int o = -1;
  if (a >= 0 && a < g.nsx && b >= 0 && b < g.nsy) {
    o = b * g.nsx + a;
    vort[o] = v;
  }
  prev[q] = o;
  if (q != 0) return;
  strip[0] = cx - 5;   // the patch's first vertex and the rows of the previous column's strip
  strip[1] = cy - 5;
  strip[2] = rr_lv[0];
  strip[3] = rr_lv[1];
  const int b0 = max(0, cy - 5), b1 = min(g.nsy, cy + 3);
  rr_in[0] = b0;
  rr_in[1] = b1;
  rr_in[2] = ROW_ZERO;
  int lo = max(0, b0 - R), hi = min(g.nsy, b1 + R);
  rr_lv[0] = lo; rr_lv[1] = hi; rr_lv[2] = ROW_ZERO;
  box[0] = max(0, cx - 5 - R);
  box[1] = min(g.nsx - 1, cx + 2 + R);
  box[2] = lo;
  box[3] = hi - 1;
  for (int lv = 1; lv < L; ++lv) {
    int r0 = max(1, lo - 1), r1 = min(g.n - 3, hi);
    if ((r0 & 1) == 0) r0 += 1;
    if ((r1 & 1) == 0) r1 -= 1;
    if (lo >= hi || r0 > r1) { lo = 0; hi = 0; }
    else { lo = g.n / 4 + (r0 - 1) / 2; hi = g.n / 4 + (r1 - 1) / 2 + 1; }
    rr_lv[3 * lv] = lo; rr_lv[3 * lv + 1] = hi;
    rr_lv[3 * lv + 2] = lv == L - 1 ? ROW_ZERO : ROW_EDGES;
  }
}

// The forward x transform of the column's patch rows, D[dj][k] = sum_di vort[b][a] W[a][k]
// (a = strip[0] + di, b = strip[1] + dj, in order of di; zero for rows outside the grid).
__global__ void k_sd_patch_modes(const int* __restrict__ strip, GridDims g, const double* __restrict__ vort,
                                 const double* __restrict__ W, double* __restrict__ D) {
  IB_GRID_DEP_WAIT();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.nsx) return;
  const int dj = blockIdx.y, b = strip[1] + dj;
  double v = 0.0;
  if (b >= 0 && b < g.nsy)
    for (int di = 0; di < 8; ++di) {
      const int a = strip[0] + di;
      if (a >= 0 && a < g.nsx) v = fma(vort[(size_t)b * g.nsx + a], W[(size_t)a * g.nsx + k], v);
    }
  D[(size_t)dj * g.nsx + k] = v;
}

// ainv's modes of the patch: per patch row b (in order), D[b] times the tabulated response A_b to
// a unit row, on the strip's rows within trunc_rows of b; the previous strip's rows outside this
// one cleared.  Grid: x over the modes, y over 2 (2R + 8) row slots (new strip, then old one).
__global__ void k_sd_strip(const int* __restrict__ strip, const int* __restrict__ rr_lv, GridDims g,
                           const double* __restrict__ D, const double* __restrict__ A, int r0, int R,
                           double* __restrict__ specY) {
  IB_GRID_DEP_WAIT();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.nsx) return;
  const int lo = rr_lv[0], hi = rr_lv[1];
  const int sl = blockIdx.y, ws = 2 * R + 8, w = 2 * R + 1;
  if (sl < ws) {
    const int y = lo + sl;
    if (y >= hi) return;
    double v = 0.0;
    for (int dj = 0; dj < 8; ++dj) {
      const int b = strip[1] + dj;
      if (b < 0 || b >= g.nsy || y < b - R || y > b + R) continue;
      const double* Ab = A + ((size_t)(b - r0) * w + (y - (b - R))) * g.nsx;
      v = fma(D[(size_t)dj * g.nsx + k], Ab[k], v);
    }
    specY[(size_t)y * g.nsx + k] = v;
  } else {
    const int y = strip[2] + (sl - ws);
    if (y < 0 || y >= strip[3] || (y >= lo && y < hi)) return;
    specY[(size_t)y * g.nsx + k] = 0.0;
  }
}

// Candidate row i of column *col (one warp each): E_o (curl s) at that unknown
// (regT_sd_sparse of a_times_sd's fluxes).
__global__ void k_sd_entries(const int* col, int nb_sd, const int* __restrict__ cptr, const int* __restrict__ cidx,
                             GridDims g, const double* __restrict__ s, const double* __restrict__ ring,
                             const int* __restrict__ comp, const int* __restrict__ ix, const int* __restrict__ iy,
                             const double* __restrict__ w, double* __restrict__ out) {
  IB_GRID_DEP_WAIT();
  const int i = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  const int u = *col;
  const int pt = u < nb_sd ? u : u - nb_sd;
  const int c0 = cptr[pt], n = cptr[pt + 1] - c0;
  if (i >= 2 * n) return;
  const int r = i < n ? cidx[c0 + i] : cidx[c0 + i - n] + nb_sd;
  const bool isx = comp[r] == 1;
  const int nxf = isx ? g.nux : g.nvx, nyf = isx ? g.nuy : g.nvy;
  const int cx = ix[r], cy = iy[r];
  const double* wr = w + (size_t)r * 49;
  double acc = 0.0;
  for (int sl = lane; sl < 49; sl += 32) {
    const int fi = cx + sl % 7 - 3, fj = cy + sl / 7 - 3;
    if (fi >= 1 && fi <= nxf && fj >= 1 && fj <= nyf) {
      const double qf = isx ? ghost_vertex(s, ring, g, fi, fj + 1) - ghost_vertex(s, ring, g, fi, fj)
                            : ghost_vertex(s, ring, g, fi, fj) - ghost_vertex(s, ring, g, fi + 1, fj);
      acc = fma(wr[sl], qf, acc);
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) out[i] = acc;
}

// The drop tolerance on column *col (one CTA): rows with |B_ij| > droptol B_jj kept, in order,
// from colptr[j]; nz[j] their count.
__global__ void k_sd_drop(const int* col, int nb_sd, const int* __restrict__ cptr, const int* __restrict__ cidx,
                          const int* __restrict__ cself, const double* __restrict__ buf,
                          const long long* __restrict__ colptr, int* __restrict__ rows, double* __restrict__ vals,
                          int* __restrict__ nz, double droptol) {
  IB_GRID_DEP_WAIT();
  __shared__ int wsum[32];
  __shared__ int base_s, tot_s;
  const int u = *col;
  const int pt = u < nb_sd ? u : u - nb_sd;
  const int c0 = cptr[pt], n = cptr[pt + 1] - c0, total = 2 * n;
  const double thr = droptol * buf[(u < nb_sd ? 0 : n) + cself[pt]];
  const long long base = colptr[u];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (threadIdx.x == 0) base_s = 0;
  __syncthreads();
  for (int start = 0; start < total; start += blockDim.x) {
    const int i = start + threadIdx.x;
    const bool keep = i < total && fabs(buf[i]) > thr;
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    const int wpos = __popc(m & ((1u << lane) - 1u));
    if (lane == 0) wsum[wid] = __popc(m);
    __syncthreads();
    if (wid == 0) {
      const int v = lane < nw ? wsum[lane] : 0;
      int inc = v;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
      }
      wsum[lane] = inc - v;
      if (lane == 31) tot_s = inc;
    }
    __syncthreads();
    if (keep) {
      const long long at = base + base_s + wsum[wid] + wpos;
      rows[at] = i < n ? cidx[c0 + i] : cidx[c0 + i - n] + nb_sd;
      vals[at] = buf[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) base_s += tot_s;
    __syncthreads();
  }
  if (threadIdx.x == 0) nz[u] = base_s;
}

// Clears a set's last patch (the scratch vorticity is all zero between builds).
__global__ void k_sd_clear(double* vort, int* prev) {
  IB_GRID_DEP_WAIT();
  const int pv = prev[threadIdx.x];
  if (pv >= 0) vort[pv] = 0.0;
  prev[threadIdx.x] = -1;
}

__global__ void k_sd_compact(const long long* __restrict__ from, const int* __restrict__ nz,
                             const long long* __restrict__ to, const int* __restrict__ rows_in,
                             const double* __restrict__ vals_in, int* __restrict__ rows_out,
                             double* __restrict__ vals_out) {
  const int c = blockIdx.x;
  for (int i = threadIdx.x; i < nz[c]; i += blockDim.x) {
    rows_out[to[c] + i] = rows_in[from[c] + i];
    vals_out[to[c] + i] = vals_in[from[c] + i];
  }
}

// --------------------------------------------------------------------- FSI iteration
struct InterpArgs {
  int nf, nr_sd, nx, ny, nb_sd;
  double sdxi, sdyi, dsd;
  const double* xb;
  const double* yb;
  const int* comp;
  const int* rigid;
  int* pidx;
  double* pw;
  int* err;
};

// deltafnc2 (grid.F90:1007-1029), the 2-point hat, in the source's order
__device__ __forceinline__ double hat2(double x1, double x2, double dr) {
  const double r1 = __ddiv_rn(fabs(__dsub_rn(x1, x2)), dr);
  const double d = r1 <= 1.0 ? __dsub_rn(1.0, r1) : 0.0;
  return __ddiv_rn(d, dr);
}

// setup_reg_subdomain_indices (grid.F90:819-873) for each body unknown: the 4 sub-domain
// unknowns (x outer, y inner) and weights delta_sd^2 hat(x) hat(y); a point on a sub-domain
// point takes it with weight 1 alone.  A point outside the cloud sets IB_ERR_DOMAIN (the
// reference stops) and takes the nearest cell.
__global__ void k_sd_interp(InterpArgs a) {
  IB_GRID_DEP_WAIT();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.nf) return;
  const bool isx = a.comp[k] == 1;
  const int yoff = isx ? 0 : a.nb_sd;
  const int rp = a.rigid[k];
  if (rp >= 0) {   // the body point is sub-domain point rp (the others are weightless dummies)
    const int dummy = min(rp + 1, a.nb_sd - 1);
    a.pidx[4 * k] = rp + yoff;
    a.pw[4 * k] = 1.0;
    for (int i = 1; i < 4; ++i) {
      a.pidx[4 * k + i] = dummy + yoff;
      a.pw[4 * k + i] = 0.0;
    }
    return;
  }
  const double xb = a.xb[k], yb = a.yb[k], d = a.dsd;
  const double fx = __dadd_rn(__ddiv_rn(__dsub_rn(xb, a.sdxi), d), 1.0);
  const double fy = __dadd_rn(__ddiv_rn(__dsub_rn(yb, a.sdyi), d), 1.0);
  int l0 = (int)fx, p0 = (int)fy;   // Fortran INT (toward zero)
  if (l0 < 1 || l0 + 1 > a.nx || p0 < 1 || p0 + 1 > a.ny) {
    atomicExch(a.err, IB_ERR_DOMAIN);
    l0 = min(max(l0, 1), a.nx - 1);
    p0 = min(max(p0, 1), a.ny - 1);
  }
  int nn[4];
  double w[4];
  bool exact[4];
  bool any = false;
  const double d2 = __dmul_rn(d, d);
  for (int l = 0; l < 2; ++l) {
    for (int p = 0; p < 2; ++p) {
      const int i = 2 * l + p;
      const int ll = l0 + l, pp = p0 + p;
      nn[i] = a.nr_sd + (pp - 1) * a.nx + (ll - 1);
      const double sx = __dadd_rn(a.sdxi, __dmul_rn((double)(ll - 1), d));
      const double sy = __dadd_rn(a.sdyi, __dmul_rn((double)(pp - 1), d));
      const double dx = __dsub_rn(xb, sx), dy = __dsub_rn(yb, sy);
      exact[i] = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)) == 0.0;
      any = any || exact[i];
      w[i] = __dmul_rn(__dmul_rn(d2, hat2(sx, xb, d)), hat2(sy, yb, d));
    }
  }
  for (int i = 0; i < 4; ++i) {
    a.pidx[4 * k + i] = nn[i] + yoff;
    a.pw[4 * k + i] = exact[i] ? 1.0 : (any ? 0.0 : w[i]);
  }
}

// B(b, a): row b of column a, zero where dropped (binary search over the column's rows)
__device__ __forceinline__ double b_at(const long long* __restrict__ colptr, const int* __restrict__ nz,
                                       const int* __restrict__ rows, const double* __restrict__ vals, int b, int a) {
  long long lo = colptr[a], hi = lo + nz[a];
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    const int r = rows[mid];
    if (r == b) return vals[mid];
    if (r < b) lo = mid + 1;
    else hi = mid;
  }
  return 0.0;
}

// compute_operator (operators_struct.F90:840-905): lumat(k, l) = body(k, l) + sum_q P(k,q)
// inter(l, a_q(k)), inter(l, a) = sum_r B(b_r(l), a) P(l, r), each dot product in order; written
// into the solver's column-major operator St[l][k].  body: b_times2's matrix (body_mat).  A CTA
// takes 32 entries l of column k: its threads find the 16 B entries of each (binary searches in
// the columns, the latency) and their products, then one warp sums each entry in the order above.
constexpr int kLumatRows = 32;
__global__ void __launch_bounds__(256) k_sd_lumat(int nf, const int* __restrict__ pidx, const double* __restrict__ pw,
                                                  const long long* __restrict__ colptr, const int* __restrict__ nz,
                                                  const int* __restrict__ rows, const double* __restrict__ vals,
                                                  const double* __restrict__ brv, const double* __restrict__ bco,
                                                  const int* __restrict__ bod, double* __restrict__ St) {
  IB_GRID_DEP_WAIT();
  __shared__ double prod[kLumatRows][17];
  const int k = blockIdx.y, l0 = blockIdx.x * kLumatRows;
  for (int t = threadIdx.x; t < kLumatRows * 16; t += blockDim.x) {
    const int e = t >> 4, sub = t & 15, q = sub >> 2, r = sub & 3, l = l0 + e;
    if (l < nf)
      prod[e][sub] = __dmul_rn(b_at(colptr, nz, rows, vals, pidx[4 * l + r], pidx[4 * k + q]), pw[4 * l + r]);
  }
  __syncthreads();
  const int l = l0 + (int)threadIdx.x;
  if (threadIdx.x >= kLumatRows || l >= nf) return;
  const double* v = prod[threadIdx.x];
  double dot = 0.0;
#pragma unroll
  for (int qq = 0; qq < 4; ++qq) {
    double inter = 0.0;
#pragma unroll
    for (int rr = 0; rr < 4; ++rr) inter = __dadd_rn(inter, v[4 * qq + rr]);
    dot = __dadd_rn(dot, __dmul_rn(pw[4 * k + qq], inter));
  }
  const int bk = bod[k];
  const double body = (bk >= 0 && bod[l] == bk) ? brv[k] * brv[l] * bco[k] : 0.0;
  St[(size_t)l * nf + k] = __dadd_rn(body, dot);
}

// timestepper.F90:371-395: rhsf(j) = P_j . (E_o (q + q0)) + rhsf(j).  E_o (q + q0) is needed only
// at the four sub-domain unknowns P_j reads, so each CTA (one body unknown, four warps) forms
// those four with regT's arithmetic (k_regT: one warp per unknown, lanes over the 49 stencil
// slots, a xor tree), then thread 0 takes the dot product in order.
__global__ void __launch_bounds__(128) k_sd_rhs(GridDims g, const int* __restrict__ pidx,
                                                const double* __restrict__ pw, const double* __restrict__ qx,
                                                const double* __restrict__ qx0, const double* __restrict__ qy,
                                                const double* __restrict__ qy0, RegDev r, double* __restrict__ rhsf) {
  IB_GRID_DEP_WAIT();
  __shared__ double eq[4];
  const int k = blockIdx.x, q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int a = pidx[4 * k + q];
  const bool isx = r.comp[a] == 1;
  const double* fq = isx ? qx : qy;
  const double* fq0 = isx ? qx0 : qy0;
  const int ld = isx ? g.nux : g.nvx, ny = isx ? g.nuy : g.nvy;
  const int cx = r.ix[a], cy = r.iy[a];
  const double* wk = r.w + (size_t)a * 49;
  double acc = 0.0;
  for (int sl = lane; sl < 49; sl += 32) {
    const int fi = cx + sl % 7 - 3, fj = cy + sl / 7 - 3;
    if (fi >= 1 && fi <= ld && fj >= 1 && fj <= ny) {
      const int idx = (fj - 1) * ld + (fi - 1);
      acc = fma(wk[sl], fq0 ? fq[idx] + fq0[idx] : fq[idx], acc);
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) eq[q] = 0.0 + acc;
  __syncthreads();
  if (threadIdx.x != 0) return;
  double dot = 0.0;
  for (int qq = 0; qq < 4; ++qq) dot = __dadd_rn(dot, __dmul_rn(pw[4 * k + qq], eq[qq]));
  rhsf[k] = __dadd_rn(dot, rhsf[k]);
}

// P^T f (timestepper.F90:502: matmul over the body unknowns in order) on every sub-domain unknown.
// The entries (k, q) of P pass through shared memory in chunks, each with its product
// P(k,q) f(k); every thread scans them in order for its own cloud unknown.
__global__ void __launch_bounds__(128) k_sd_ptf(int nf, int nf_sd, const int* __restrict__ pidx,
                                                const double* __restrict__ pw, const double* __restrict__ f,
                                                double* __restrict__ fsd) {
  constexpr int kChunk = 1024;
  __shared__ int sidx[kChunk];
  __shared__ double sprod[kChunk];
  IB_GRID_DEP_WAIT();
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  double acc = 0.0;
  for (int e0 = 0; e0 < 4 * nf; e0 += kChunk) {
    const int ne = min(kChunk, 4 * nf - e0);
    __syncthreads();
    for (int e = threadIdx.x; e < ne; e += blockDim.x) {
      sidx[e] = pidx[e0 + e];
      sprod[e] = __dmul_rn(pw[e0 + e], f[(e0 + e) >> 2]);
    }
    __syncthreads();
    // the entries of this unknown first (integer work), then their sum in order, so that the
    // FP64 adds are issued for the few entries that match only
    int hit[8];
    int nh = 0;
    for (int e = 0; e < ne; ++e) {
      if (sidx[e] != a) continue;
      if (nh == 8) {   // more than eight: add the ones held, keep collecting
        for (int h = 0; h < 8; ++h) acc = __dadd_rn(acc, sprod[hit[h]]);
        nh = 0;
      }
      hit[nh++] = e;
    }
    for (int h = 0; h < nh; ++h) acc = __dadd_rn(acc, sprod[hit[h]]);
  }
  if (a < nf_sd) fsd[a] = acc;
}

}  // namespace

int launch_sd_interp(Ctx* c, cudaStream_t st) {
  SubDomain& S = c->sd;
  InterpArgs a;
  a.nf = c->nf; a.nr_sd = S.nr_sd; a.nx = S.nx; a.ny = S.ny; a.nb_sd = S.nb_sd;
  a.sdxi = S.sdxi; a.sdyi = S.sdyi; a.dsd = S.dsd;
  a.xb = c->xb; a.yb = c->yb; a.comp = c->comp; a.rigid = S.rigid;
  a.pidx = S.pidx; a.pw = S.pw; a.err = c->d_err;
  count_launch();
  k_sd_interp<<<cdiv(c->nf, 128), 128, 0, st>>>(a);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

void sd_free(Ctx* c) {
  SubDomain& S = c->sd;
  if (S.mem) cudaFree(S.mem);
  if (S.rows) cudaFree(S.rows);
  if (S.vals) cudaFree(S.vals);
  S = SubDomain{};
}

int sd_setup(Ctx* c, int full_rectangular, double sdxi, double sdxe, double sdyi, double sdye, double dsd,
             std::string* msg) {
  const GridDims& g = c->g;
  const IbParams& p = c->p;
  auto bad = [&](int rc, const char* m) {
    *msg = m;
    return rc;
  };
  if (c->itime != 0) return bad(IB_ERR_STATE, "the sub-domain is set up before the first step");
  if (c->sd.on) return bad(IB_ERR_STATE, "the sub-domain is already set up");
  if (p.num_stat) return bad(IB_ERR_ARG, "the sub-domain method needs the GMRES path (num_stat = F)");
  if (c->nf == 0) return bad(IB_ERR_ARG, "the sub-domain method needs a body");
  if (!(dsd > 0.0) || !(sdxe > sdxi) || !(sdye > sdyi)) return bad(IB_ERR_ARG, "bad sub-domain rectangle");
  SubDomain S;
  S.on = true;
  S.full_rect = full_rectangular != 0;
  S.sdxi = sdxi; S.sdxe = sdxe; S.sdyi = sdyi; S.sdye = sdye; S.dsd = dsd;
  S.nx = fortran_nint((sdxe - sdxi) / dsd + 1);   // grid.F90:325
  S.ny = fortran_nint((sdye - sdyi) / dsd + 1);
  if (S.nx < 2 || S.ny < 2) return bad(IB_ERR_ARG, "the sub-domain needs at least 2 x 2 points");
  // the point cloud (grid.F90:320-352) and the rigid map of the body unknowns
  std::vector<double> px, py;
  std::vector<int> rigid(c->nf, -1);
  if (!S.full_rect) {   // the stationary rigid bodies' points, at their positions now
    std::vector<double> xh(c->nf), yh(c->nf);
    if (cudaStreamSynchronize(c->st) != cudaSuccess ||
        cudaMemcpy(xh.data(), c->xb, 8 * (size_t)c->nf, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(yh.data(), c->yb, 8 * (size_t)c->nf, cudaMemcpyDeviceToHost) != cudaSuccess)
      return bad(IB_ERR_CUDA, "cannot read the body positions");
    int off = 0;
    for (const auto& b : c->bodies_h) {
      if (b.fam == 1) {
        for (int i = 0; i < b.npts; ++i) {
          rigid[off + i] = (int)px.size();
          rigid[off + b.npts + i] = (int)px.size();
          px.push_back(xh[off + i]);
          py.push_back(yh[off + i]);
        }
      }
      off += 2 * b.npts;
    }
  }
  S.nr_sd = (int)px.size();
  for (int j = 1; j <= S.ny; ++j)
    for (int i = 1; i <= S.nx; ++i) {
      px.push_back(sdxi + (double)(i - 1) * dsd);
      py.push_back(sdyi + (double)(j - 1) * dsd);
    }
  S.nb_sd = (int)px.size();
  S.nf_sd = 2 * S.nb_sd;
  const int nb = S.nb_sd, nfs = S.nf_sd;
  // grid origins (grid.F90:663-664) and E E^T's sparsity: points whose 21 x 21 face blocks
  // meet; the blocks are indexed without bounds in the reference, so they must lie in the grid
  std::vector<int> gx(nb), gy(nb);
  for (int k = 0; k < nb; ++k) {
    gx[k] = (int)((px[k] + p.offsetx) / c->delta) + 1;
    gy[k] = (int)((py[k] + p.offsety) / c->delta) + 1;
    if (gx[k] < kSupportNz + 1 || gx[k] > g.m - kSupportNz || gy[k] < kSupportNz + 1 || gy[k] > g.n - kSupportNz)
      return bad(IB_ERR_DOMAIN, "a sub-domain point lies within 11 cells of the domain boundary");
  }
  std::vector<std::vector<int>> cell((size_t)(g.m + 2) * (g.n + 2));
  for (int k = 0; k < nb; ++k) cell[(size_t)gy[k] * (g.m + 2) + gx[k]].push_back(k);
  std::vector<int> cptr(nb + 1, 0), cidx, cself(nb, 0);
  const int span = 2 * kSupportNz;
  for (int k = 0; k < nb; ++k) {
    const size_t start = cidx.size();
    for (int y = std::max(0, gy[k] - span); y <= std::min(g.n + 1, gy[k] + span); ++y)
      for (int x = std::max(0, gx[k] - span); x <= std::min(g.m + 1, gx[k] + span); ++x)
        for (int q : cell[(size_t)y * (g.m + 2) + x]) cidx.push_back(q);
    std::sort(cidx.begin() + start, cidx.end());
    cself[k] = (int)(std::lower_bound(cidx.begin() + start, cidx.end(), k) - (cidx.begin() + start));
    cptr[k + 1] = (int)cidx.size();
    S.max_cand = std::max(S.max_cand, cptr[k + 1] - cptr[k]);
  }
  std::vector<long long> colptr(nfs + 1, 0);
  for (int u = 0; u < nfs; ++u) {
    const int pt = u % nb;
    colptr[u + 1] = colptr[u] + 2LL * (cptr[pt + 1] - cptr[pt]);
  }
  S.candidates = colptr[nfs];
  // the fixed-size buffers in one allocation
  const int sets = Influence::kBuildStreams;
  const int max_faces = (g.m + 3) * (g.n + 3) + 1;
  struct Part { size_t bytes; void** at; };
  std::vector<Part> parts;
  auto part = [&](void** at, size_t bytes) { parts.push_back({(bytes + 255) / 256 * 256, at}); };
  part((void**)&S.ux, 8 * (size_t)nfs);
  part((void**)&S.uy, 8 * (size_t)nfs);
  part((void**)&S.ucomp, 4 * (size_t)nfs);
  part((void**)&S.reg.ix, 4 * (size_t)nfs);
  part((void**)&S.reg.iy, 4 * (size_t)nfs);
  part((void**)&S.reg.w, 8 * 49 * (size_t)nfs);
  part((void**)&S.reg.bbox, 4 * 16);
  part((void**)&S.reg.cnt_x, 4 * (size_t)max_faces);
  part((void**)&S.reg.cnt_y, 4 * (size_t)max_faces);
  part((void**)&S.reg.lst_x, 4 * 49 * (size_t)nfs);
  part((void**)&S.reg.lst_y, 4 * 49 * (size_t)nfs);
  part((void**)&S.reg.stale, 4);
  part((void**)&S.cptr, 4 * (size_t)(nb + 1));
  part((void**)&S.cidx, 4 * std::max<size_t>(1, cidx.size()));
  part((void**)&S.cself, 4 * (size_t)nb);
  part((void**)&S.colptr, 8 * (size_t)(nfs + 1));
  part((void**)&S.nz, 4 * (size_t)nfs);
  part((void**)&S.rigid, 4 * (size_t)c->nf);
  part((void**)&S.pidx, 4 * kInterp * (size_t)c->nf);
  part((void**)&S.pw, 8 * kInterp * (size_t)c->nf);
  part((void**)&S.fsd, 8 * (size_t)nfs);
  part((void**)&S.pprev, 4 * kPatch * (size_t)sets);
  part((void**)&S.colbuf, 8 * 2 * (size_t)S.max_cand * sets);
  size_t total = 0;
  for (const Part& q : parts) total += q.bytes;
  size_t freeb = 0, totalb = 0;
  if (cudaMemGetInfo(&freeb, &totalb) != cudaSuccess) return bad(IB_ERR_CUDA, "cudaMemGetInfo failed");
  if (total > freeb / 2) return bad(IB_ERR_NOMEM, "the sub-domain's buffers do not fit in device memory");
  if (cudaMalloc(&S.mem, total) != cudaSuccess) return bad(IB_ERR_NOMEM, "sub-domain allocation failed");
  {
    char* base = (char*)S.mem;
    for (const Part& q : parts) {
      *q.at = base;
      base += q.bytes;
    }
  }
  S.reg.comp = S.ucomp;
  S.reg.max_faces = max_faces;
  S.reg.max_list = 49 * nfs;
  std::vector<double> ux(nfs), uy(nfs);
  std::vector<int> uc(nfs);
  for (int u = 0; u < nfs; ++u) {
    ux[u] = px[u % nb];
    uy[u] = py[u % nb];
    uc[u] = u < nb ? 1 : 2;   // collect_subdomain (grid.F90:437-455)
  }
  cudaStream_t st = c->st;
  // zero: the weights kernel rebuilds the contribution lists only where an origin moved, and
  // no origin of the cloud is 0
  int rc = cudaMemsetAsync(S.mem, 0, total, st) == cudaSuccess ? IB_OK : IB_ERR_CUDA;
  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (rc == IB_OK && bytes && cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
      rc = IB_ERR_CUDA;
  };
  up(S.ux, ux.data(), 8 * ux.size());
  up(S.uy, uy.data(), 8 * uy.size());
  up(S.ucomp, uc.data(), 4 * uc.size());
  up(S.cptr, cptr.data(), 4 * cptr.size());
  up(S.cidx, cidx.data(), 4 * cidx.size());
  up(S.cself, cself.data(), 4 * cself.size());
  up(S.colptr, colptr.data(), 8 * colptr.size());
  up(S.rigid, rigid.data(), 4 * rigid.size());
  if (rc == IB_OK && cudaMemsetAsync(S.pprev, 0xff, 4 * kPatch * (size_t)sets, st) != cudaSuccess) rc = IB_ERR_CUDA;
  if (rc == IB_OK && cudaMemsetAsync(S.reg.stale, 0, 4, st) != cudaSuccess) rc = IB_ERR_CUDA;
  // E_o: the weights and contribution lists of every sub-domain unknown (setup_pre_reg_subdomain)
  if (rc == IB_OK) rc = launch_reg_build(g, nfs, S.ux, S.uy, c->delta, p.offsetx, p.offsety, S.reg, c->d_err, st);
  if (rc == IB_OK && cudaStreamSynchronize(st) != cudaSuccess) rc = IB_ERR_CUDA;
  if (rc == IB_OK) rc = check_err(c);
  if (rc != IB_OK) {
    cudaFree(S.mem);
    return bad(rc, "sub-domain setup failed on the device");
  }
  c->sd = S;
  // the cloud's stencils read the finest fluxes away from the body: the step's first vort2flux
  // forms every row
  c->v2f_partial = false;
  return IB_OK;
}

int sd_precompute(Ctx* c) {
  SubDomain& S = c->sd;
  if (!S.on) return IB_ERR_STATE;
  const GridDims& g = c->g;
  Influence& I = c->inf;
  const auto t0 = std::chrono::steady_clock::now();
  RC(inf_build_scratch(c));
  // the coarse levels' responses for the level-1 vertices the columns reach (coarse.cu)
  bool use_cr = false;
  if (c->L > 1 && I.cr.enabled) {
    std::vector<int> ixh(S.nf_sd), iyh(S.nf_sd);
    IB_CUDA_CHECK(cudaStreamSynchronize(c->st));
    IB_CUDA_CHECK(cudaMemcpy(ixh.data(), S.reg.ix, 4 * (size_t)S.nf_sd, cudaMemcpyDeviceToHost));
    IB_CUDA_CHECK(cudaMemcpy(iyh.data(), S.reg.iy, 4 * (size_t)S.nf_sd, cudaMemcpyDeviceToHost));
    std::vector<unsigned char> mask(g.ns, 0);
    for (int u = 0; u < S.nf_sd; ++u)
      for (int b = std::max(0, iyh[u] - 5); b <= std::min(g.nsy - 1, iyh[u] + 2); ++b)
        for (int a = std::max(0, ixh[u] - 5); a <= std::min(g.nsx - 1, ixh[u] + 2); ++a)
          mask[(size_t)b * g.nsx + a] = 1;
    cr_dilate(g, mask, I.trunc_rows);
    use_cr = cr_prepare(c, mask) == IB_OK;   // else each column runs the coarse chain itself
    cudaGetLastError();
  }
  for (SchurScratch& sc : I.bscr) {
    sc.cr_R1 = use_cr ? I.cr.R[1] : nullptr;
    sc.cr_idx1 = use_cr ? I.cr.idx[1] : nullptr;
  }
  // ainv's modes of each column from the strips of its patch rows (influence.cu)
  bool use_strips = false;
  double* Dmodes = nullptr;
  int strip_lo = 0, strip_hi = -1;
  {
    std::vector<int> iyh(S.nf_sd);
    IB_CUDA_CHECK(cudaStreamSynchronize(c->st));
    IB_CUDA_CHECK(cudaMemcpy(iyh.data(), S.reg.iy, 4 * (size_t)S.nf_sd, cudaMemcpyDeviceToHost));
    strip_lo = g.nsy;
    for (int u = 0; u < S.nf_sd; ++u) {
      strip_lo = std::min(strip_lo, std::max(0, iyh[u] - 5));
      strip_hi = std::max(strip_hi, std::min(g.nsy - 1, iyh[u] + 2));
    }
    if (strip_hi >= strip_lo && inf_strip_alloc(c, strip_hi - strip_lo + 1) &&
        cudaMalloc(&Dmodes, 8 * 8 * (size_t)g.nsx * Influence::kBuildStreams) == cudaSuccess) {
      RC(inf_strip_table(c, strip_lo, strip_hi));
      use_strips = true;
    }
    cudaGetLastError();
  }
  for (SchurScratch& sc : I.bscr) sc.specY_ready = use_strips;
  // the candidate values of every column, before the drop (freed once compacted)
  if (S.rows) cudaFree(S.rows);
  if (S.vals) cudaFree(S.vals);
  S.rows = nullptr;
  S.vals = nullptr;
  int* rows_full = nullptr;
  double* vals_full = nullptr;
  {
    size_t freeb = 0, totalb = 0;
    IB_CUDA_CHECK(cudaMemGetInfo(&freeb, &totalb));
    if ((size_t)S.candidates * 12 > freeb / 2) return IB_ERR_NOMEM;
  }
  IB_CUDA_CHECK(cudaMalloc(&rows_full, 4 * (size_t)std::max(1LL, S.candidates)));
  IB_CUDA_CHECK(cudaMalloc(&vals_full, 8 * (size_t)std::max(1LL, S.candidates)));
  cudaStream_t st = c->st;
  const int nsets = std::min(Influence::kBuildStreams, S.nf_sd);
  cudaEvent_t ev = nullptr;
  IB_CUDA_CHECK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaEventRecord(ev, st);
  for (int i = 0; i < nsets; ++i) cudaStreamWaitEvent(I.bscr[i].st, ev, 0);
  const bool prof = c->prof_on;
  c->prof_on = false;
  int rc = IB_OK;
  long long body_launches = 0;
  std::vector<cudaGraphExec_t> execs(nsets, nullptr);
  cudaStream_t cap = nullptr;
  if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) rc = IB_ERR_CUDA;
  const long long l0 = launch_count();
  const int entry_blocks = cdiv(32LL * 2 * S.max_cand, 128);
  for (int i = 0; i < nsets && rc == IB_OK; ++i) {
    const SchurScratch& sc = I.bscr[i];
    int* col = sc.prev + 4;   // the set's fifth int, as in the band build
    int* pprev = S.pprev + kPatch * i;
    double* buf = S.colbuf + 2 * (size_t)S.max_cand * i;
    cudaGraph_t graph = nullptr;
    do {
      if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeRelaxed) != cudaSuccess) { rc = IB_ERR_CUDA; break; }
      count_launch();
      k_sd_col_init<<<1, 32, 0, cap>>>(col, i);
      cudaGraphConditionalHandle h = 0;
      cudaGraph_t body = nullptr;
      if (cudaGraphConditionalHandleCreate(&h, capture_graph(cap), 1, cudaGraphCondAssignDefault) != cudaSuccess)
        rc = IB_ERR_CUDA;
      if (rc == IB_OK) rc = add_while(cap, h, &body);
      if (rc == IB_OK &&
          cudaStreamBeginCaptureToGraph(sc.st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess)
        rc = IB_ERR_CUDA;
      if (rc == IB_OK) {
        const long long b0 = launch_count();
        count_launch();
        k_sd_source<<<1, kPatch, 0, sc.st>>>(col, S.ucomp, S.reg.ix, S.reg.iy, S.reg.w, g, sc.vort, pprev, sc.rr_in,
                                             sc.rr_lv, sc.box, sc.strip, c->L, I.trunc_rows);
        if (use_strips) {
          double* D = Dmodes + 8 * (size_t)g.nsx * i;
          const int R = I.trunc_rows;
          count_launches(2);
          k_sd_patch_modes<<<dim3(cdiv(g.nsx, 128), 8), 128, 0, sc.st>>>(sc.strip, g, sc.vort, c->wmat, D);
          k_sd_strip<<<dim3(cdiv(g.nsx, 128), 2 * (2 * R + 8)), 128, 0, sc.st>>>(sc.strip, sc.rr_lv, g, D, I.strips,
                                                                                 I.strip_r0, R, sc.specY);
        }
        const double* ring0 = nullptr;
        rc = schur_fluid(c, sc.vort, sc.rr_in, S.reg.bbox + 7, sc.s0, &ring0, &sc);
        count_launches(3);
        k_sd_entries<<<entry_blocks, 128, 0, sc.st>>>(col, S.nb_sd, S.cptr, S.cidx, g, sc.s0, ring0, S.ucomp,
                                                     S.reg.ix, S.reg.iy, S.reg.w, buf);
        k_sd_drop<<<1, 1024, 0, sc.st>>>(col, S.nb_sd, S.cptr, S.cidx, S.cself, buf, S.colptr, rows_full,
                                         vals_full, S.nz, kDropTol);
        k_sd_col_next<<<1, 32, 0, sc.st>>>(col, nsets, S.nf_sd, h);
        body_launches = launch_count() - b0;
        cudaGraph_t tmp;
        if (cudaStreamEndCapture(sc.st, &tmp) != cudaSuccess && rc == IB_OK) rc = IB_ERR_CUDA;
      }
      if (cudaStreamEndCapture(cap, &graph) != cudaSuccess && rc == IB_OK) rc = IB_ERR_CUDA;
      if (rc == IB_OK) make_edges_programmatic(body);
      if (rc == IB_OK && cudaGraphInstantiate(&execs[i], graph, 0) != cudaSuccess) rc = IB_ERR_CUDA;
    } while (false);
    if (graph) cudaGraphDestroy(graph);
  }
  count_launches(-(launch_count() - l0));   // captured, not run
  cudaGetLastError();
  if (rc == IB_OK) {
    for (int i = 0; i < nsets && rc == IB_OK; ++i)
      if (cudaGraphLaunch(execs[i], I.bscr[i].st) != cudaSuccess) rc = IB_ERR_CUDA;
    if (rc == IB_OK) count_launches(nsets + (long long)S.nf_sd * body_launches);
  }
  c->prof_on = prof;
  for (int i = 0; i < nsets; ++i) {
    const SchurScratch& sc = I.bscr[i];
    count_launch();
    k_sd_clear<<<1, kPatch, 0, sc.st>>>(sc.vort, S.pprev + kPatch * i);
    cudaEventRecord(ev, sc.st);
    cudaStreamWaitEvent(st, ev, 0);
  }
  for (int i = 0; i < nsets; ++i) cudaStreamSynchronize(I.bscr[i].st);
  for (cudaGraphExec_t e : execs)
    if (e) cudaGraphExecDestroy(e);
  if (cap) cudaStreamDestroy(cap);
  cudaEventDestroy(ev);
  for (SchurScratch& sc : I.bscr) {
    sc.cr_R1 = nullptr;
    sc.specY_ready = false;
  }
  if (Dmodes) cudaFree(Dmodes);
  if (rc == IB_OK && use_cr) {
    int err = 0;
    if (cudaMemcpy(&err, I.cr.err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) rc = IB_ERR_CUDA;
    else if (err) rc = IB_ERR_STATE;   // a column met a vertex without a response
  }
  // compaction: the kept rows of every column, back to back
  if (rc == IB_OK) {
    std::vector<int> nz(S.nf_sd);
    if (cudaMemcpyAsync(nz.data(), S.nz, 4 * nz.size(), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      rc = IB_ERR_CUDA;
    std::vector<long long> to(S.nf_sd + 1, 0);
    for (int u = 0; u < S.nf_sd && rc == IB_OK; ++u) to[u + 1] = to[u] + nz[u];
    long long* dto = nullptr;
    if (rc == IB_OK && (cudaMalloc(&dto, 8 * to.size()) != cudaSuccess ||
                        cudaMalloc(&S.rows, 4 * (size_t)std::max(1LL, to.back())) != cudaSuccess ||
                        cudaMalloc(&S.vals, 8 * (size_t)std::max(1LL, to.back())) != cudaSuccess))
      rc = IB_ERR_NOMEM;
    if (rc == IB_OK && cudaMemcpyAsync(dto, to.data(), 8 * to.size(), cudaMemcpyHostToDevice, st) != cudaSuccess)
      rc = IB_ERR_CUDA;
    if (rc == IB_OK) {
      count_launch();
      k_sd_compact<<<S.nf_sd, 128, 0, st>>>(S.colptr, S.nz, dto, rows_full, vals_full, S.rows, S.vals);
      if (cudaGetLastError() != cudaSuccess ||
          cudaMemcpyAsync(S.colptr, dto, 8 * to.size(), cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess)
        rc = IB_ERR_CUDA;
    }
    if (dto) cudaFree(dto);
    S.kept = to.back();
  }
  cudaFree(rows_full);
  cudaFree(vals_full);
  RC(rc);
  S.columns += S.nf_sd;
  S.ready = true;
  S.precompute_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return check_err(c);
}

int launch_sd_lumat(Ctx* c, cudaStream_t st) {
  SubDomain& S = c->sd;
  Influence& I = c->inf;
  count_launch();
  k_sd_lumat<<<dim3(cdiv(c->nf, kLumatRows), c->nf), 256, 0, st>>>(c->nf, S.pidx, S.pw, S.colptr, S.nz, S.rows,
                                                                   S.vals, I.brv, I.bco, I.bod, I.St);
  IB_CUDA_CHECK(cudaGetLastError());
  return launch_beam_add_b(c, I.St, st);
}

int sd_assemble(Ctx* c, bool interp) {
  cudaStream_t st = c->st;
  if (interp) RC(launch_sd_interp(c, st));
  RC(inf_assemble_b(c, st));
  return launch_sd_lumat(c, st);
}

int launch_sd_rhs(Ctx* c, double* rhsf, cudaStream_t st, bool interp) {
  SubDomain& S = c->sd;
  const GridDims& g = c->g;
  if (interp) RC(launch_sd_interp(c, st));
  count_launch();
  k_sd_rhs<<<c->nf, 128, 0, st>>>(g, S.pidx, S.pw, c->qx[0], c->q0x[0], c->qy[0], c->q0y[0], S.reg, rhsf);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

int launch_sd_ET(Ctx* c, const double* hx, const double* hy, double* out, cudaStream_t st) {
  SubDomain& S = c->sd;
  IB_CUDA_CHECK(cudaMemsetAsync(out, 0, 8 * (size_t)c->nf, st));
  count_launch();
  k_sd_rhs<<<c->nf, 128, 0, st>>>(c->g, S.pidx, S.pw, hx, nullptr, hy, nullptr, S.reg, out);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

int launch_sd_spread(Ctx* c, const double* f, double* hx, double* hy, cudaStream_t st) {
  SubDomain& S = c->sd;
  RC(launch_sd_interp(c, st));
  count_launch();
  k_sd_ptf<<<cdiv(S.nf_sd, 128), 128, 0, st>>>(c->nf, S.nf_sd, S.pidx, S.pw, f, S.fsd);
  IB_CUDA_CHECK(cudaGetLastError());
  return launch_reg_box(c->g, S.nf_sd, S.fsd, S.reg, hx, hy, st);
}

// ------------------------------------------------------------------ sd_precomputed.chd
// preprocess_sd's file (timestepper.F90:691-695, 753-756; read back at 740-757): per column a
// record holding its count, then one holding its values and its 1-based row indices (PetscInt,
// 32-bit), Fortran unformatted sequential records (4-byte length before and after each).
int sd_write(Ctx* c, const char* path, std::string* msg) {
  SubDomain& S = c->sd;
  if (!S.on || !S.ready) {
    *msg = "no sub-domain matrix to write";
    return IB_ERR_STATE;
  }
  std::vector<long long> colptr(S.nf_sd + 1);
  std::vector<int> nz(S.nf_sd);
  IB_CUDA_CHECK(cudaStreamSynchronize(c->st));
  IB_CUDA_CHECK(cudaMemcpy(colptr.data(), S.colptr, 8 * colptr.size(), cudaMemcpyDeviceToHost));
  IB_CUDA_CHECK(cudaMemcpy(nz.data(), S.nz, 4 * nz.size(), cudaMemcpyDeviceToHost));
  const long long total = colptr[S.nf_sd];
  std::vector<int> rows(std::max(1LL, total));
  std::vector<double> vals(std::max(1LL, total));
  if (total) {
    IB_CUDA_CHECK(cudaMemcpy(rows.data(), S.rows, 4 * (size_t)total, cudaMemcpyDeviceToHost));
    IB_CUDA_CHECK(cudaMemcpy(vals.data(), S.vals, 8 * (size_t)total, cudaMemcpyDeviceToHost));
  }
  FILE* fh = std::fopen(path, "wb");
  if (!fh) {
    *msg = std::string("cannot open ") + path;
    return IB_ERR_ARG;
  }
  bool ok = true;
  auto put = [&](const void* p, size_t n) { ok = ok && std::fwrite(p, 1, n, fh) == n; };
  for (int u = 0; u < S.nf_sd && ok; ++u) {
    const int n = nz[u];
    int32_t len = 4;
    put(&len, 4);
    put(&n, 4);
    put(&len, 4);
    len = 12 * n;
    put(&len, 4);
    put(vals.data() + colptr[u], 8 * (size_t)n);
    for (int i = 0; i < n && ok; ++i) {
      const int32_t r1 = rows[colptr[u] + i] + 1;
      put(&r1, 4);
    }
    put(&len, 4);
  }
  ok = (std::fclose(fh) == 0) && ok;
  if (!ok) {
    *msg = std::string("write failed: ") + path;
    return IB_ERR_ARG;
  }
  return IB_OK;
}

int sd_read(Ctx* c, const char* path, std::string* msg) {
  SubDomain& S = c->sd;
  if (!S.on) {
    *msg = "no sub-domain set up";
    return IB_ERR_STATE;
  }
  FILE* fh = std::fopen(path, "rb");
  if (!fh) {
    *msg = std::string("cannot open ") + path;
    return IB_ERR_ARG;
  }
  std::vector<long long> colptr(S.nf_sd + 1, 0);
  std::vector<int> nz(S.nf_sd), rows;
  std::vector<double> vals;
  bool ok = true;
  auto get = [&](void* p, size_t n) { ok = ok && std::fread(p, 1, n, fh) == n; };
  for (int u = 0; u < S.nf_sd && ok; ++u) {
    int32_t a = 0, b = 0, n = 0;
    get(&a, 4);
    get(&n, 4);
    get(&b, 4);
    ok = ok && a == 4 && b == 4 && n >= 0 && n <= S.nf_sd;
    if (!ok) break;
    get(&a, 4);
    ok = ok && a == 12 * n;
    if (!ok) break;
    const size_t at = vals.size();
    vals.resize(at + n);
    rows.resize(at + n);
    get(vals.data() + at, 8 * (size_t)n);
    for (int i = 0; i < n && ok; ++i) {
      int32_t r1 = 0;
      get(&r1, 4);
      ok = ok && r1 >= 1 && r1 <= S.nf_sd && (i == 0 || r1 - 1 > rows[at + i - 1]);
      rows[at + i] = r1 - 1;
    }
    get(&b, 4);
    ok = ok && b == a;
    nz[u] = n;
    colptr[u + 1] = colptr[u] + n;
  }
  std::fclose(fh);
  if (!ok) {
    *msg = std::string("not a sub-domain matrix of this cloud (ascending rows expected): ") + path;
    return IB_ERR_ARG;
  }
  if (S.rows) cudaFree(S.rows);
  if (S.vals) cudaFree(S.vals);
  S.rows = nullptr;
  S.vals = nullptr;
  const size_t total = std::max<size_t>(1, vals.size());
  IB_CUDA_CHECK(cudaMalloc(&S.rows, 4 * total));
  IB_CUDA_CHECK(cudaMalloc(&S.vals, 8 * total));
  if (!vals.empty()) {
    IB_CUDA_CHECK(cudaMemcpy(S.rows, rows.data(), 4 * rows.size(), cudaMemcpyHostToDevice));
    IB_CUDA_CHECK(cudaMemcpy(S.vals, vals.data(), 8 * vals.size(), cudaMemcpyHostToDevice));
  }
  IB_CUDA_CHECK(cudaMemcpy(S.colptr, colptr.data(), 8 * colptr.size(), cudaMemcpyHostToDevice));
  IB_CUDA_CHECK(cudaMemcpy(S.nz, nz.data(), 4 * nz.size(), cudaMemcpyHostToDevice));
  S.kept = (long long)vals.size();
  S.ready = true;
  return IB_OK;
}

}  // namespace ib
