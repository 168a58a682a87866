// Regularised delta-function transfer between body points and the finest grid:
// E^T (reg, fsinterface.F90:14-47), E (regT, fsinterface.F90:51-80), the weights
// (setup_reg, grid.F90:459-528; deltafnc, grid.F90:955-1003), force
// redistribution (operators_struct.F90:735-834) and force coefficients
// (write_force2, operators_struct.F90:711-731).
//
// reg is a face-major gather: for every face of the stencil bounding box the
// contributing unknowns are listed in ascending order, so each face sums its
// contributions in the same order as the reference's sequential scatter-add.
#include "fsi_dev.cuh"

namespace ib {

// Stencil origins and weights of 8 unknowns per CTA (reg_weights_cta).
__global__ void __launch_bounds__(128) k_reg_weights(GridDims g, int nf, const double* __restrict__ xb,
                                                     const double* __restrict__ yb, double d, double ox,
                                                     double oy, const int* __restrict__ comp, int* ix, int* iy,
                                                     double* w, int* stale, int* err) {
  IB_GRID_DEP_WAIT();
  __shared__ double fac[16][7];    // [2*unknown + axis][offset], axis 0: x factor, 1: y factor
  __shared__ double pos[8][2];
  const int k0 = blockIdx.x * 8;
  if ((int)threadIdx.x < 8 && k0 + (int)threadIdx.x < nf) {
    pos[threadIdx.x][0] = xb[k0 + threadIdx.x];
    pos[threadIdx.x][1] = yb[k0 + threadIdx.x];
  }
  __syncthreads();
  reg_weights_cta(g, nf, k0, pos, d, ox, oy, comp, ix, iy, w, stale, err, fac, nullptr, nullptr);
}

// Bounding box of all stencils (one CTA).  bbox[0..3] = i0, j0, ni, nj of the face box;
// bbox[4..6] and bbox[7..9] = [first, last+1) vertex row (0-based) that rot(E^T f) can touch
// and that E(curl s) reads, followed by the treatment of the other rows (zero / skip).
__global__ void k_reg_bbox(GridDims g, int nf, const int* __restrict__ ix, const int* __restrict__ iy, int* bbox,
                           const int* __restrict__ stale) {
  IB_GRID_DEP_WAIT();
  __shared__ int s[4][32];
  if (!*stale) return;
  int imin = 1 << 30, jmin = 1 << 30, imax = -(1 << 30), jmax = -(1 << 30);
  for (int k = threadIdx.x; k < nf; k += blockDim.x) {
    imin = min(imin, ix[k]); imax = max(imax, ix[k]);
    jmin = min(jmin, iy[k]); jmax = max(jmax, iy[k]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    imin = min(imin, __shfl_xor_sync(0xffffffffu, imin, o));
    imax = max(imax, __shfl_xor_sync(0xffffffffu, imax, o));
    jmin = min(jmin, __shfl_xor_sync(0xffffffffu, jmin, o));
    jmax = max(jmax, __shfl_xor_sync(0xffffffffu, jmax, o));
  }
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { s[0][wid] = imin; s[1][wid] = imax; s[2][wid] = jmin; s[3][wid] = jmax; }
  __syncthreads();
  if (threadIdx.x == 0) {
    int nw = blockDim.x >> 5;
    for (int q = 1; q < nw; ++q) {
      imin = min(imin, s[0][q]); imax = max(imax, s[1][q]);
      jmin = min(jmin, s[2][q]); jmax = max(jmax, s[3][q]);
    }
    if (nf == 0) { imin = imax = jmin = jmax = 4; }
    bbox[0] = imin - 3;
    bbox[1] = jmin - 3;
    bbox[2] = imax - imin + 7;
    bbox[3] = jmax - jmin + 7;
    int rlo = max(0, jmin - 5), rhi = min(g.nsy - 1, jmax + 2) + 1;
    bbox[4] = rlo; bbox[5] = rhi; bbox[6] = 0;   // ROW_ZERO
    bbox[7] = rlo; bbox[8] = rhi; bbox[9] = 3;   // ROW_SKIP
  }
}

// Count (fill=false) or list (fill=true) contributions per box face, ascending k.
template <bool FILL>
__global__ void k_reg_lists(int nf, const int* __restrict__ comp, const int* __restrict__ ix,
                            const int* __restrict__ iy, const int* __restrict__ bbox, int* cnt_x, int* cnt_y,
                            int* lst_x, int* lst_y, int max_faces, const int* __restrict__ stale) {
  IB_GRID_DEP_WAIT();
  if (!*stale) return;
  int i0 = bbox[0], j0 = bbox[1], ni = bbox[2], nj = bbox[3];
  int nface = ni * nj;
  if (nface + 1 > max_faces) return;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 2 * nface; t += gridDim.x * blockDim.x) {
    int c = t < nface ? 1 : 2;
    int fidx = t < nface ? t : t - nface;
    int fi = i0 + fidx % ni, fj = j0 + fidx / ni;
    int* cnt = c == 1 ? cnt_x : cnt_y;
    int* lst = c == 1 ? lst_x : lst_y;
    int pos = FILL ? cnt[fidx] : 0;
    int n = 0;
    for (int k = 0; k < nf; ++k) {
      if (comp[k] != c) continue;
      int p = fi - ix[k], l = fj - iy[k];
      if (p >= -3 && p <= 3 && l >= -3 && l <= 3) {
        if (FILL) lst[pos + n] = k * 49 + (l + 3) * 7 + (p + 3);
        ++n;
      }
    }
    if (!FILL) cnt[fidx] = n;
  }
}

// Exclusive scan of both count arrays (one CTA, 1024 threads): each thread sums a run of
// consecutive faces, the runs are scanned with warp shuffles, then written back.
__global__ void k_reg_scan(const int* __restrict__ bbox, int* cnt_x, int* cnt_y, int max_faces,
                           const int* __restrict__ stale) {
  IB_GRID_DEP_WAIT();
  __shared__ int wsum[32];
  if (!*stale) return;
  const int nface = bbox[2] * bbox[3];
  if (nface + 1 > max_faces) return;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int c = 0; c < 2; ++c) {
    int* cnt = c == 0 ? cnt_x : cnt_y;
    const int per = (nface + blockDim.x - 1) / blockDim.x;
    const int s0 = min(tid * per, nface), s1 = min(s0 + per, nface);
    int sum = 0;
    for (int i = s0; i < s1; ++i) sum += cnt[i];
    int inc = sum;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
      int v = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0, winc = v;
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, winc, o);
        if (lane >= o) winc += y;
      }
      wsum[lane] = winc - v;
      if (lane == 31) cnt[nface] = winc;
    }
    __syncthreads();
    int run = wsum[wid] + inc - sum;
    for (int i = s0; i < s1; ++i) { int v = cnt[i]; cnt[i] = run; run += v; }
    __syncthreads();
  }
}

int launch_reg_weights(const GridDims& g, int nf, const double* xb, const double* yb, double delta, double offx,
                       double offy, RegDev& r, int* d_err, cudaStream_t st) {
  if (nf == 0) return IB_OK;
  // launch_reg_lists skips its work (each kernel returns at once) unless a stencil origin moved
  IB_CUDA_CHECK(cudaMemsetAsync(r.stale, 0, sizeof(int), st));
  count_launch();
  k_reg_weights<<<cdiv(nf, 8), 128, 0, st>>>(g, nf, xb, yb, delta, offx, offy, r.comp, r.ix, r.iy, r.w, r.stale,
                                              d_err);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

int launch_reg_lists(int nf, RegDev& r, const GridDims& g, cudaStream_t st) {
  if (nf == 0) return IB_OK;
  count_launch();
  k_reg_bbox<<<1, 256, 0, st>>>(g, nf, r.ix, r.iy, r.bbox, r.stale);
  count_launch();
  k_reg_lists<false><<<152 * 2, 128, 0, st>>>(nf, r.comp, r.ix, r.iy, r.bbox, r.cnt_x, r.cnt_y, nullptr,
                                              nullptr, r.max_faces, r.stale);
  count_launch();
  k_reg_scan<<<1, 1024, 0, st>>>(r.bbox, r.cnt_x, r.cnt_y, r.max_faces, r.stale);
  count_launch();
  k_reg_lists<true><<<152 * 2, 128, 0, st>>>(nf, r.comp, r.ix, r.iy, r.bbox, r.cnt_x, r.cnt_y, r.lst_x, r.lst_y,
                                             r.max_faces, r.stale);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

int launch_reg_build(const GridDims& g, int nf, const double* xb, const double* yb, double delta, double offx,
                     double offy, RegDev& r, int* d_err, cudaStream_t st) {
  const int rc = launch_reg_weights(g, nf, xb, yb, delta, offx, offy, r, d_err, st);
  return rc != IB_OK ? rc : launch_reg_lists(nf, r, g, st);
}

__global__ void k_reg_snapshot(int nf, const int* __restrict__ ix, const int* __restrict__ iy,
                               const double* __restrict__ w, int* ix_s, int* iy_s, double* w_s) {
  IB_GRID_DEP_WAIT();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 49 * nf; i += gridDim.x * blockDim.x) {
    w_s[i] = w[i];
    if (i < nf) {
      ix_s[i] = ix[i];
      iy_s[i] = iy[i];
    }
  }
}

int launch_reg_snapshot(int nf, const RegDev& r, int* ix_s, int* iy_s, double* w_s, cudaStream_t st) {
  if (nf == 0) return IB_OK;
  count_launch();
  k_reg_snapshot<<<cdiv(49LL * nf, 256), 256, 0, st>>>(nf, r.ix, r.iy, r.w, ix_s, iy_s, w_s);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

// E^T h0: every face of the box gets the ordered sum of weight*h0 over its list.
// zero_empty: faces of the box with no contribution are written as zero (else left as they are).
__global__ void k_reg(GridDims g, const double* __restrict__ h0, const double* __restrict__ w,
                      const int* __restrict__ bbox, const int* __restrict__ cnt_x, const int* __restrict__ cnt_y,
                      const int* __restrict__ lst_x, const int* __restrict__ lst_y, double* hx, double* hy,
                      int max_faces, int zero_empty) {
  IB_GRID_DEP_WAIT();
  int i0 = bbox[0], j0 = bbox[1], ni = bbox[2], nj = bbox[3];
  int nface = ni * nj;
  if (nface + 1 > max_faces) return;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 2 * nface; t += gridDim.x * blockDim.x) {
    bool cx = t < nface;
    int fidx = cx ? t : t - nface;
    int fi = i0 + fidx % ni, fj = j0 + fidx / ni;
    const int* cnt = cx ? cnt_x : cnt_y;
    const int* lst = cx ? lst_x : lst_y;
    int a = cnt[fidx], b = cnt[fidx + 1];
    // faces outside the grid (a body too close to the edge, flagged as IB_ERR_DOMAIN
    // when the weights were built) are skipped rather than written
    if (fi < 1 || fj < 1 || fi > (cx ? g.nux : g.nvx) || fj > (cx ? g.nuy : g.nvy)) continue;
    if (a == b && !zero_empty) continue;
    double acc = 0.0;
    for (int q = a; q < b; ++q) {
      int e = lst[q];
      acc = acc + w[e] * h0[e / 49];
    }
    if (cx) hx[(fj - 1) * g.nux + (fi - 1)] = acc;
    else hy[(fj - 1) * g.nvx + (fi - 1)] = acc;
  }
}

int launch_reg(const GridDims& g, int nf, const double* h0, const RegDev& r, double* hx, double* hy,
               cudaStream_t st) {
  IB_CUDA_CHECK(cudaMemsetAsync(hx, 0, sizeof(double) * g.nu, st));
  IB_CUDA_CHECK(cudaMemsetAsync(hy, 0, sizeof(double) * g.nv, st));
  if (nf == 0) return IB_OK;
  count_launch();
  k_reg<<<152 * 2, 128, 0, st>>>(g, h0, r.w, r.bbox, r.cnt_x, r.cnt_y, r.lst_x, r.lst_y, hx, hy, r.max_faces, 0);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

int launch_reg_box(const GridDims& g, int nf, const double* h0, const RegDev& r, double* hx, double* hy,
                   cudaStream_t st) {
  if (nf == 0) return IB_OK;
  count_launch();
  k_reg<<<152 * 2, 128, 0, st>>>(g, h0, r.w, r.bbox, r.cnt_x, r.cnt_y, r.lst_x, r.lst_y, hx, hy, r.max_faces, 1);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

// E q: h0_out[k] = h0_in[k] + sum_slots w * q(face).  One warp per unknown: the 49 slot
// products are summed by a warp tree, then added to h0_in (fsinterface.F90:51-80 sums the
// slots one by one; the difference is round-off).
__global__ void k_regT(GridDims g, int nf, const double* __restrict__ qx, const double* __restrict__ qx0,
                       const double* __restrict__ qy, const double* __restrict__ qy0, const int* __restrict__ comp,
                       const int* __restrict__ ix, const int* __restrict__ iy, const double* __restrict__ w,
                       const double* __restrict__ h0_in, double* h0_out) {
  IB_GRID_DEP_WAIT();
  int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (k >= nf) return;
  bool isx = comp[k] == 1;
  const double* q = isx ? qx : qy;
  const double* q0 = isx ? qx0 : qy0;
  int ld = isx ? g.nux : g.nvx;
  int ny = isx ? g.nuy : g.nvy;
  int cx = ix[k], cy = iy[k];
  const double* wk = w + (size_t)k * 49;
  double acc = 0.0;
  for (int sl = lane; sl < 49; sl += 32) {
    int fi = cx + sl % 7 - 3, fj = cy + sl / 7 - 3;
    // stencil faces outside the grid (flagged as IB_ERR_DOMAIN) contribute nothing
    if (fi >= 1 && fi <= ld && fj >= 1 && fj <= ny) {
      int idx = (fj - 1) * ld + (fi - 1);
      double v = q0 ? q[idx] + q0[idx] : q[idx];
      acc = fma(wk[sl], v, acc);
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) h0_out[k] = (h0_in ? h0_in[k] : 0.0) + acc;
}

int launch_regT(const GridDims& g, int nf, const double* qx, const double* qx0, const double* qy, const double* qy0,
                const RegDev& r, const double* h0_in, double* h0_out, cudaStream_t st) {
  if (nf == 0) return IB_OK;
  count_launch();
  k_regT<<<cdiv(32LL * nf, 128), 128, 0, st>>>(g, nf, qx, qx0, qy, qy0, r.comp, r.ix, r.iy, r.w, h0_in, h0_out);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

// E curl(s): h0_out[k] = h0_in[k] + sum_slots w * q(face), with q = curl(s) evaluated at the
// stencil faces (operators_fluid.F90:423-471 fused into fsinterface.F90:51-80); s ghosts
// come from the ring.
__global__ void k_regT_s(GridDims g, int nf, const double* __restrict__ s, const double* __restrict__ ring,
                         const int* __restrict__ comp, const int* __restrict__ ix, const int* __restrict__ iy,
                         const double* __restrict__ w, const double* __restrict__ h0_in, double* h0_out) {
  IB_GRID_DEP_WAIT();
  int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (k >= nf) return;
  bool isx = comp[k] == 1;
  int nxf = isx ? g.nux : g.nvx, nyf = isx ? g.nuy : g.nvy;
  int cx = ix[k], cy = iy[k];
  const double* wk = w + (size_t)k * 49;
  double acc = 0.0;
  for (int sl = lane; sl < 49; sl += 32) {
    int fi = cx + sl % 7 - 3, fj = cy + sl / 7 - 3;
    if (fi >= 1 && fi <= nxf && fj >= 1 && fj <= nyf) {
      double q = isx ? ghost_vertex(s, ring, g, fi, fj + 1) - ghost_vertex(s, ring, g, fi, fj)
                     : ghost_vertex(s, ring, g, fi, fj) - ghost_vertex(s, ring, g, fi + 1, fj);
      acc = fma(wk[sl], q, acc);
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) h0_out[k] = (h0_in ? h0_in[k] : 0.0) + acc;
}

int launch_regT_s(const GridDims& g, int nf, const double* s, const double* ring, const RegDev& r,
                  const double* h0_in, double* h0_out, cudaStream_t st) {
  if (nf == 0) return IB_OK;
  count_launch();
  k_regT_s<<<cdiv(32LL * nf, 128), 128, 0, st>>>(g, nf, s, ring, r.comp, r.ix, r.iy, r.w, h0_in, h0_out);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

// finter = (1/E^T 1) * E^T f where E^T 1 > 1e-10, else 0 (redistribute2)
__global__ void k_redist_field(GridDims g, const double* __restrict__ f, const double* __restrict__ w,
                               const int* __restrict__ bbox, const int* __restrict__ cnt_x,
                               const int* __restrict__ cnt_y, const int* __restrict__ lst_x,
                               const int* __restrict__ lst_y, double* fx, double* fy, int max_faces) {
  IB_GRID_DEP_WAIT();
  int i0 = bbox[0], j0 = bbox[1], ni = bbox[2], nj = bbox[3];
  int nface = ni * nj;
  if (nface + 1 > max_faces) return;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 2 * nface; t += gridDim.x * blockDim.x) {
    bool cx = t < nface;
    int fidx = cx ? t : t - nface;
    int fi = i0 + fidx % ni, fj = j0 + fidx / ni;
    const int* cnt = cx ? cnt_x : cnt_y;
    const int* lst = cx ? lst_x : lst_y;
    int a = cnt[fidx], b = cnt[fidx + 1];
    if (a == b) continue;
    if (fi < 1 || fj < 1 || fi > (cx ? g.nux : g.nvx) || fj > (cx ? g.nuy : g.nvy)) continue;
    double ws = 0.0, fs = 0.0;
    for (int q = a; q < b; ++q) {
      int e = lst[q];
      ws = ws + w[e] * 1.0;
      fs = fs + w[e] * f[e / 49];
    }
    double v = ws > 1.0e-10 ? 1.0 / ws * fs : 0.0;
    if (cx) fx[(fj - 1) * g.nux + (fi - 1)] = v;
    else fy[(fj - 1) * g.nvx + (fi - 1)] = v;
  }
}

// Writes the faces of the box that have contributions and leaves the others as they were:
// every face a stencil reads has one (the stencil's own unknown), so E of the result
// (launch_regT with the same weights) reads written faces only.
int launch_redistribute_field(const GridDims& g, int nf, const double* f, const RegDev& r, double* fx,
                              double* fy, cudaStream_t st) {
  if (nf == 0) return IB_OK;
  count_launch();
  // about one box face per thread (a stencil covers 49 faces; the loop strides over the rest)
  const int nblk = std::max(8, std::min(152 * 2, cdiv(49LL * nf, 128)));
  k_redist_field<<<nblk, 128, 0, st>>>(g, f, r.w, r.bbox, r.cnt_x, r.cnt_y, r.lst_x, r.lst_y, fx, fy, r.max_faces);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

// write_force2: out[b] = 2 delta sum_x f/dt, out[nbody+b] = 2 delta sum_y f/dt, each sum in the
// order of the unknowns.  One warp per body: the lanes divide (f/dt, about ten FP64 instructions
// each) a chunk of the unknowns at a time into shared memory, then lane 0 adds the x terms and
// lane 1 the y terms in order.  With mirror set the coefficients, and the nt hinge angles after
// them, are also written there (pinned host memory the device maps).
constexpr int kForceChunk = 1024;
__global__ void k_force_coeffs(int nf, int nbody, const int* __restrict__ comp, const int* __restrict__ bid,
                               const double* __restrict__ f, double dt, double delta, double* out, double* mirror,
                               const double* __restrict__ theta, int nt) {
  IB_GRID_DEP_WAIT();
  __shared__ double q[kForceChunk];
  const int b = blockIdx.x, lane = threadIdx.x;
  double acc = 0.0;   // lane 0: x terms, lane 1: y terms
  for (int k0 = 0; k0 < nf; k0 += kForceChunk) {
    const int n = min(kForceChunk, nf - k0);
    for (int i = lane; i < n; i += 32) q[i] = bid[k0 + i] == b ? f[k0 + i] / dt : 0.0;
    __syncwarp();
    if (lane < 2)
      for (int i = 0; i < n; ++i)
        if (bid[k0 + i] == b && (comp[k0 + i] == 1) == (lane == 0)) acc = acc + q[i];
    __syncwarp();
  }
  if (lane < 2) {
    const double v = 2.0 * delta * acc;
    out[lane * nbody + b] = v;
    if (mirror) mirror[lane * nbody + b] = v;
  }
  if (mirror && b == 0)
    for (int t = lane; t < nt; t += 32) mirror[2 * nbody + t] = theta[t];
}

int launch_force_coeffs(int nf, int nbody, const int* comp, const int* bid, const double* f, double dt,
                        double delta, double* out, cudaStream_t st, double* mirror, const double* theta, int nt) {
  if (nbody == 0) return IB_OK;
  count_launch();
  k_force_coeffs<<<nbody, 32, 0, st>>>(nf, nbody, comp, bid, f, dt, delta, out, mirror, theta, nt);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

}  // namespace ib
