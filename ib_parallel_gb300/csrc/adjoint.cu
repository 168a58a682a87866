// The discrete adjoint of the time step (no reference counterpart; the reference's step is
// timestepper.F90:18-556) for stationary rigid bodies in a moving frame, their Schur system
// solved directly (num_stat) or by the cluster GMRES on the assembled operator: the frame's flux is linear in its velocity (u, v) and angular velocity W about the
// centre motion[3..4] (motion_potential + motion_rotation, variables.F90:299-360), so a
// pitching or plunging body held fixed in its own frame takes one coefficient triple per step,
// q0 = u Bu + v Bv + W BW on every level.
//
// ib_adjoint_forward advances nsteps with the given triples, keeping the state (omega, s, q,
// rhs_old of every level) every K steps and at the end; ib_adjoint_backward runs the steps in
// reverse, each segment of K steps recomputed from its checkpoint with the inputs of every step
// taped, and returns dJ/d(u, v, W) per step for J = sum of dforces . forces.  The reverse of a
// step applies the exact transpose of every linear map of the forward in reverse order:
//   * the spectral solves (ctci, ainv, the predictor's (I - cL)^-1 (I + cL)) are symmetric, and
//     the predictor's transpose is two predictor solves, one on the adjoint as omega and one on
//     it as the boundary right-hand side;
//   * rot^T = curl with a zero ring and curl^T = rot plus the ring's edge gathers;
//   * nonlinear is bilinear in (omega, q + q0) and linear in its ghost ring: k_adj_nl_vertex
//     and k_adj_nl_faces gather each argument's adjoint;
//   * get_bc^T, apply_bc^T and coarsify^T are gathers (each output element sums its own
//     contributions, so no floating-point atomics);
//   * reg and regT are each other's transposes; the Cholesky solve is symmetric, and without
//     num_stat the reverse solves the transposed system, S^T x = b, with the same GMRES on the
//     assembled operator's row-major copy (which, read column-major, is S^T): the adjoint of the
//     exact solve, which the forward's converged Krylov solve approaches (timestepper.F90:363-366).
#include <algorithm>
#include <cmath>
#include <vector>

#include "ctx.cuh"

namespace ib {

namespace {

constexpr int kT = 256;

// out = ((c0 B0) + (c1 B1)) + (c2 B2), rounded step by step
__global__ void k_adj_combine(int n, const double* __restrict__ b0, const double* __restrict__ b1,
                              const double* __restrict__ b2, double c0, double c1, double c2, double* __restrict__ out) {
  IB_GRID_DEP_WAIT();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = __dadd_rn(__dadd_rn(__dmul_rn(c0, b0[i]), __dmul_rn(c1, b1[i])), __dmul_rn(c2, b2[i]));
}

// T[i][j] = M[j][i] (n x n)
__global__ void k_adj_transpose(int n, const double* __restrict__ M, double* __restrict__ T) {
  IB_GRID_DEP_WAIT();
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * n) return;
  const int i = (int)(t / n), j = (int)(t - (long long)i * n);
  T[t] = M[(size_t)j * n + i];
}

// out = a x + b y (y may be null)
__global__ void k_adj_axpby(int n, double a, const double* __restrict__ x, double b, const double* __restrict__ y,
                            double* __restrict__ out) {
  IB_GRID_DEP_WAIT();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = a * x[i];
  out[i] = y ? v + b * y[i] : v;
}

// the ghosted vertex (r, c) (0-based rows and columns of the (n+1) x (m+1) frame) of which the
// ring entry t is the value, or -1 for the left/right corner entries the rows overwrite
__device__ __forceinline__ bool ring_vertex(const GridDims& g, int t, int* r, int* c) {
  if (t < g.right) { *c = 0; *r = t - g.left; return *r >= 1 && *r <= g.n - 1; }
  if (t < g.bottom) { *c = g.m; *r = t - g.right; return *r >= 1 && *r <= g.n - 1; }
  if (t < g.top) { *r = 0; *c = t - g.bottom; return true; }
  *r = g.n; *c = t - g.top;
  return true;
}

// curl^T at the ghosted vertex (r, c): the vertex field's adjoint from (lx, ly)
__device__ __forceinline__ double curl_T_at(const GridDims& g, const double* __restrict__ lx,
                                            const double* __restrict__ ly, int r, int c) {
  double v = 0.0;
  if (r >= 1) v += lx[(r - 1) * g.nux + c];
  if (r <= g.n - 1) v -= lx[r * g.nux + c];
  if (c <= g.m - 1) v += ly[r * g.nvx + c];
  if (c >= 1) v -= ly[r * g.nvx + c - 1];
  return v;
}

// ring += the ring's part of curl^T (the edges of the ghosted frame)
__global__ void k_adj_ring_curl(GridDims g, const double* __restrict__ lx, const double* __restrict__ ly,
                                double* __restrict__ ring) {
  IB_GRID_DEP_WAIT();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.nbc) return;
  int r, c;
  if (ring_vertex(g, t, &r, &c)) ring[t] += curl_T_at(g, lx, ly, r, c);
}

// ring = fac * the boundary rows and columns of v (apply_bc^T; the ring's end entries zero)
__global__ void k_adj_apply_bc(GridDims g, const double* __restrict__ v, double fac, double* __restrict__ ring) {
  IB_GRID_DEP_WAIT();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.nbc) return;
  double out = 0.0;
  if (t < g.right) {
    const int j = t - g.left - 1;
    if (j >= 0 && j <= g.n - 2) out = fac * v[j * g.nsx];
  } else if (t < g.bottom) {
    const int j = t - g.right - 1;
    if (j >= 0 && j <= g.n - 2) out = fac * v[j * g.nsx + g.m - 2];
  } else if (t < g.top) {
    const int i = t - g.bottom - 1;
    if (i >= 0 && i <= g.m - 2) out = fac * v[i];
  } else {
    const int i = t - g.top - 1;
    if (i >= 0 && i <= g.m - 2) out = fac * v[(g.n - 2) * g.nsx + i];
  }
  ring[t] = out;
}

// s += get_bc^T(fac ring): every point of the coarse centre's perimeter gathers the ring
// entries it was copied to and half of each midpoint beside it
__global__ void k_adj_get_bc(GridDims g, const double* __restrict__ ring, double fac, double* __restrict__ s) {
  IB_GRID_DEP_WAIT();
  const int i0 = g.m / 4 + 1, i1 = 3 * g.m / 4 + 1, j0 = g.n / 4 + 1, j1 = 3 * g.n / 4 + 1;
  const int nrow = i1 - i0 + 1, ncol = j1 - j0 - 1;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  int I, J;
  if (t < nrow) { I = i0 + t; J = j0; }
  else if (t < 2 * nrow) { I = i0 + t - nrow; J = j1; }
  else if (t < 2 * nrow + ncol) { I = i0; J = j0 + 1 + (t - 2 * nrow); }
  else if (t < 2 * nrow + 2 * ncol) { I = i1; J = j0 + 1 + (t - 2 * nrow - ncol); }
  else return;
  auto line = [&](int base, int p, int p0, int p1, int q0) -> double {   // p along the line, q0 its start offset
    const int e = base + 2 * (p - 1 - q0);
    double v = fac * ring[e];
    if (p < p1) v += 0.5 * (fac * ring[e + 1]);
    if (p > p0) v += 0.5 * (fac * ring[e - 1]);
    return v;
  };
  double v = 0.0;
  if (J == j0) v += line(g.bottom, I, i0, i1, g.m / 4);
  if (J == j1) v += line(g.top, I, i0, i1, g.m / 4);
  if (I == i0) v += line(g.left, J, j0, j1, g.n / 4);
  if (I == i1) v += line(g.right, J, j0, j1, g.n / 4);
  s[(J - 2) * g.nsx + (I - 2)] += v;
}

// coarsify^T: every fine vertex gathers the full-weighting weights of the coarse centre
// points whose stencil holds it
__global__ void k_adj_coarsify(GridDims g, const double* __restrict__ coarse, double* __restrict__ fine) {
  IB_GRID_DEP_WAIT();
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.ns) return;
  const int J = idx / g.nsx, I = idx % g.nsx;
  const int tmax_j = g.n / 2 - 2, tmax_i = g.m / 2 - 2;
  double v = 0.0;
  for (int dj = 0; dj < 2; ++dj) {
    int tj;
    double wj;
    if (J & 1) { if (dj) break; tj = (J - 1) / 2; wj = 1.0; }
    else { tj = J / 2 - 1 + dj; wj = 0.5; }
    if (tj < 0 || tj > tmax_j) continue;
    for (int di = 0; di < 2; ++di) {
      int ti;
      double wi;
      if (I & 1) { if (di) break; ti = (I - 1) / 2; wi = 1.0; }
      else { ti = I / 2 - 1 + di; wi = 0.5; }
      if (ti < 0 || ti > tmax_i) continue;
      v += (wj * wi) * coarse[(g.n / 4 + tj) * g.nsx + (g.m / 4 + ti)];
    }
  }
  fine[idx] += v;
}

__global__ void k_adj_clear_centre(GridDims g, double* __restrict__ coarse) {
  IB_GRID_DEP_WAIT();
  const int nj = g.n / 2 - 1, ni = g.m / 2 - 1;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nj * ni) return;
  coarse[(g.n / 4 + idx / ni) * g.nsx + (g.m / 4 + idx % ni)] = 0.0;
}

// U (u averaged to vertices) and V at the ghosted vertex (r, c) of nonlinear's flux u = q + q0
__device__ __forceinline__ double u_at(const GridDims& g, const double* qx, const double* q0x, int r, int c) {
  double a = 0.0, b = 0.0;
  if (r <= g.n - 1) a = qx[r * g.nux + c] + q0x[r * g.nux + c];
  if (r >= 1) b = qx[(r - 1) * g.nux + c] + q0x[(r - 1) * g.nux + c];
  return 0.5 * (a + b);
}
__device__ __forceinline__ double v_at(const GridDims& g, const double* qy, const double* q0y, int r, int c) {
  double a = 0.0, b = 0.0;
  if (c <= g.m - 1) a = qy[r * g.nvx + c] + q0y[r * g.nvx + c];
  if (c >= 1) b = qy[r * g.nvx + c - 1] + q0y[r * g.nvx + c - 1];
  return 0.5 * (a + b);
}

// nonlinear^T in its vorticity argument (interior vertices, added to lom) and its ghost ring
// (written to lbc; the corner entries of the left and right columns stay zero)
__global__ void k_adj_nl_vertex(GridDims g, const double* __restrict__ qx, const double* __restrict__ q0x,
                                const double* __restrict__ qy, const double* __restrict__ q0y,
                                const double* __restrict__ lx, const double* __restrict__ ly, double* __restrict__ lom,
                                double* __restrict__ lbc) {
  IB_GRID_DEP_WAIT();
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int nc = g.m + 1;
  if (idx >= (g.n + 1) * nc) return;
  const int r = idx / nc, c = idx % nc;
  const double V = v_at(g, qy, q0y, r, c), U = u_at(g, qx, q0x, r, c);
  double w = 0.0;
  if (r >= 1) w += 0.5 * lx[(r - 1) * g.nux + c] * V;
  if (r <= g.n - 1) w += 0.5 * lx[r * g.nux + c] * V;
  if (c >= 1) w -= 0.5 * ly[r * g.nvx + c - 1] * U;
  if (c <= g.m - 1) w -= 0.5 * ly[r * g.nvx + c] * U;
  if (r >= 1 && r <= g.n - 1 && c >= 1 && c <= g.m - 1) {
    lom[(r - 1) * g.nsx + (c - 1)] += w;
  } else if (r == 0) {
    lbc[g.bottom + c] = w;
  } else if (r == g.n) {
    lbc[g.top + c] = w;
  } else if (c == 0) {
    lbc[g.left + r] = w;
  } else {
    lbc[g.right + r] = w;
  }
}

// nonlinear^T in its flux argument: lux on the u-faces, luy on the v-faces
__global__ void k_adj_nl_faces(GridDims g, const double* __restrict__ om, const double* __restrict__ bc,
                               const double* __restrict__ lx, const double* __restrict__ ly, double* __restrict__ lux,
                               double* __restrict__ luy) {
  IB_GRID_DEP_WAIT();
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.nu + g.nv) return;
  auto W = [&](int r, int c) { return ghost_vertex(om, bc, g, c + 1, r + 1); };
  auto lU = [&](int r, int c) {   // the adjoint of U at vertex (r, c)
    double v = 0.0;
    if (c >= 1) v -= 0.5 * ly[r * g.nvx + c - 1] * W(r, c);
    if (c <= g.m - 1) v -= 0.5 * ly[r * g.nvx + c] * W(r, c);
    return v;
  };
  auto lV = [&](int r, int c) {
    double v = 0.0;
    if (r >= 1) v += 0.5 * lx[(r - 1) * g.nux + c] * W(r, c);
    if (r <= g.n - 1) v += 0.5 * lx[r * g.nux + c] * W(r, c);
    return v;
  };
  if (idx < g.nu) {
    const int j = idx / g.nux, i = idx % g.nux;
    lux[idx] = 0.5 * lU(j + 1, i) + 0.5 * lU(j, i);
  } else {
    const int t = idx - g.nu;
    const int j = t / g.nvx, i = t % g.nvx;
    luy[t] = 0.5 * lV(j, i) + 0.5 * lV(j, i + 1);
  }
}

// lf = scale * dforce(body, component) - t
__global__ void k_adj_force(int nf, int nbody, const int* __restrict__ comp, const int* __restrict__ bid, double scale,
                            const double* __restrict__ dforce, const double* __restrict__ t, double* __restrict__ lf) {
  IB_GRID_DEP_WAIT();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nf) return;
  lf[k] = -t[k] + scale * dforce[2 * bid[k] + (comp[k] == 1 ? 0 : 1)];
}

struct DotArgs {
  const double* lx[kMaxLevels];
  const double* ly[kMaxLevels];
  const double* ax;   // level 0's extra flux adjoint (the Schur right-hand side's)
  const double* ay;
  const double* bases;   // [basis][level][u-faces, v-faces]
  int L, nu, nv;
  double* part;          // 3 x kDotBlocks partial sums
};
constexpr int kDotBlocks = 152;

// part[b][blk] = the block's slice of sum over levels of <lq0, B_b> (fixed-order tree)
__global__ void k_adj_dots(DotArgs a) {
  IB_GRID_DEP_WAIT();
  __shared__ double red[256];
  const int b = blockIdx.y, blk = blockIdx.x;
  const int per = a.nu + a.nv;
  const long long total = (long long)a.L * per;
  double acc = 0.0;
  for (long long t = (long long)blk * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(t / per), i = (int)(t % per);
    double l = i < a.nu ? a.lx[k][i] : a.ly[k][i - a.nu];
    if (k == 0) l += i < a.nu ? a.ax[i] : a.ay[i - a.nu];
    acc = fma(l, a.bases[((size_t)b * a.L + k) * per + i], acc);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) a.part[b * gridDim.x + blk] = red[0];
}

__global__ void k_adj_dots_sum(const double* __restrict__ part, int nblk, double* __restrict__ out) {
  IB_GRID_DEP_WAIT();
  const int b = threadIdx.x;
  if (b >= 3) return;
  double s = 0.0;
  for (int i = 0; i < nblk; ++i) s += part[b * nblk + i];
  out[b] = s;
}

int blocks(long long n) { return (int)cdiv(n, kT); }

}  // namespace

// ---------------------------------------------------------------------------------- host
namespace {

struct Adj {
  Ctx* c;
  AdjointState& A;
  const GridDims& g;
  int L;
  cudaStream_t st;
};

int axpby(cudaStream_t st, int n, double a, const double* x, double b, const double* y, double* out) {
  count_launch();
  k_adj_axpby<<<blocks(n), kT, 0, st>>>(n, a, x, b, y, out);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

int get_bc_T(const GridDims& g, const double* ring, double fac, double* s, cudaStream_t st) {
  const int n = 2 * (g.m / 2 + 1) + 2 * (g.n / 2 - 1);
  count_launch();
  k_adj_get_bc<<<blocks(n), kT, 0, st>>>(g, ring, fac, s);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

int apply_bc_T(const GridDims& g, const double* v, double fac, double* ring, cudaStream_t st) {
  count_launch();
  k_adj_apply_bc<<<blocks(g.nbc), kT, 0, st>>>(g, v, fac, ring);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

// the coarsify chain's transpose (fine to coarse in the forward: coarse to fine here)
int coarsify_chain_T(Adj& a, double* const* lam) {
  for (int k = a.L - 1; k >= 1; --k) {
    count_launches(2);
    k_adj_coarsify<<<blocks(a.g.ns), kT, 0, a.st>>>(a.g, lam[k], lam[k - 1]);
    k_adj_clear_centre<<<blocks((a.g.n / 2 - 1) * (a.g.m / 2 - 1)), kT, 0, a.st>>>(a.g, lam[k]);
  }
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

// vort2flux's solves transposed: flux adjoints (null: zero) of every level -> vorticity
// adjoints added to lw
int vsolve_T(Adj& a, double* const* lqx, double* const* lqy, double* const* lw) {
  AdjointState& A = a.A;
  const GridDims& g = a.g;
  for (int k = 0; k < a.L; ++k) {
    const bool has = lqx[k] != nullptr;
    if (has) RC(launch_rot(g, lqx[k], lqy[k], A.t1, a.st));
    else IB_CUDA_CHECK(cudaMemsetAsync(A.t1, 0, 8 * (size_t)g.ns, a.st));
    if (k > 0) RC(get_bc_T(g, A.ring1, 1.0, A.t1, a.st));
    RC(op_ctci(a.c, A.t1, A.t2, nullptr));
    RC(axpby(a.st, g.ns, 1.0, A.t2, 1.0, lw[k], lw[k]));
    if (k < a.L - 1) {
      RC(apply_bc_T(g, A.t2, 1.0, A.ring1, a.st));
      if (has) {
        count_launch();
        k_adj_ring_curl<<<blocks(g.nbc), kT, 0, a.st>>>(g, lqx[k], lqy[k], A.ring1);
      }
    }
  }
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

// The reverse of forward step n (its inputs taped at slot): the adjoint state in lom/lqx/lqy/lro
// becomes that of the step's inputs, and dframe[3] gets dJ/d(u, v, W) of the step.
int step_T(Adj& a, int slot, int it, const double* frame, const double* dforce_h, double* dframe_d) {
  Ctx* c = a.c;
  AdjointState& A = a.A;
  const GridDims& g = a.g;
  const int L = a.L;
  cudaStream_t st = a.st;
  const size_t per = (size_t)g.ns + g.nu + g.nv;
  double* tp = A.tape + (size_t)slot * L * per;
  auto t_om = [&](int k) { return tp + k * per; };
  auto t_qx = [&](int k) { return tp + k * per + g.ns; };
  auto t_qy = [&](int k) { return tp + k * per + g.ns + g.nu; };
  // the step's frame flux (for nonlinear's transpose) and the force adjoint
  for (int k = 0; k < L; ++k) {
    const double* B[3];
    for (int b = 0; b < 3; ++b) B[b] = A.bases + ((size_t)b * L + k) * (g.nu + g.nv);
    count_launch();
    k_adj_combine<<<blocks(g.nu + g.nv), kT, 0, st>>>(g.nu + g.nv, B[0], B[1], B[2], frame[0], frame[1], frame[2],
                                                       A.q0 + k * (size_t)(g.nu + g.nv));
  }
  IB_CUDA_CHECK(cudaMemcpyAsync(A.dforce, dforce_h, 16 * (size_t)c->nbody, cudaMemcpyHostToDevice, st));
  // final vort2flux: its solves, then its coarsify
  for (int k = 0; k < L; ++k) IB_CUDA_CHECK(cudaMemcpyAsync(A.lw[k], A.lom[k], 8 * (size_t)g.ns, cudaMemcpyDeviceToDevice, st));
  RC(vsolve_T(a, A.lqx.data(), A.lqy.data(), A.lw.data()));
  RC(coarsify_chain_T(a, A.lw.data()));
  // correction omega_0 - ainv(rot(reg f)), the direct solve, the force coefficients
  RC(op_ainv(c, A.lw[0], A.t1));
  RC(launch_curl(g, A.t1, c->zero_ring, A.hx, A.hy, st));
  // the correction spread E^T f (the sub-domain's E_o^T P^T f): its transpose, E (P E_o)
  if (c->sd.on) RC(launch_sd_ET(c, A.hx, A.hy, A.lf, st));
  else RC(launch_regT(g, c->nf, A.hx, nullptr, A.hy, nullptr, c->reg, nullptr, A.lf, st));
  count_launch();
  k_adj_force<<<blocks(c->nf), kT, 0, st>>>(c->nf, c->nbody, c->comp, c->bid, 2.0 * c->delta / c->p.dt, A.dforce,
                                            A.lf, A.lf);
  if (c->p.num_stat) {
    RC(launch_chol_solve(c->nf, c->cholM, A.lf, A.lrhsf, st));
  } else {
    // S^T lrhsf = lf: the band's row-major S (rigid bodies: no structure block), or the
    // sub-domain's lumat transposed, as the column-major operator of the cluster solver, from a
    // zero start
    const IbParams& p = c->p;
    const double* opT = c->inf.S;
    if (c->sd.on) {
      count_launch();
      k_adj_transpose<<<(unsigned)cdiv((long long)c->nf * c->nf, kT), kT, 0, st>>>(c->nf, c->inf.St, A.opT);
      IB_CUDA_CHECK(cudaGetLastError());
      opT = A.opT;
    }
    IB_CUDA_CHECK(cudaMemsetAsync(A.lrhsf, 0, 8 * (size_t)c->nf, st));
    RC(launch_gmres_fused(c->G, &c->fused_plan, opT, A.lf, A.lrhsf, p.rtol, p.atol, p.gmres_max_it, st));
    int ist[2] = {0, 0};
    IB_CUDA_CHECK(cudaMemcpyAsync(ist, c->G.ist, sizeof(ist), cudaMemcpyDeviceToHost, st));
    IB_CUDA_CHECK(cudaStreamSynchronize(st));
    if (ist[1] < 0) return IB_ERR_GMRES;   // the transposed solve stopped without converging
  }
  // rhsf = regT(q*_0 + q0_0): the flux adjoint on level 0, then the first vort2flux transposed
  if (c->sd.on) {   // rhsf = P E_o (q + q0): its transpose is the spread E_o^T P^T
    IB_CUDA_CHECK(cudaMemsetAsync(A.ax, 0, 8 * (size_t)g.nu, st));
    IB_CUDA_CHECK(cudaMemsetAsync(A.ay, 0, 8 * (size_t)g.nv, st));
    RC(launch_sd_spread(c, A.lrhsf, A.ax, A.ay, st));
  } else {
    RC(launch_reg(g, c->nf, A.lrhsf, c->reg, A.ax, A.ay, st));
  }
  for (int k = 0; k < L; ++k) IB_CUDA_CHECK(cudaMemcpyAsync(A.lostar[k], A.lw[k], 8 * (size_t)g.ns, cudaMemcpyDeviceToDevice, st));
  {
    std::vector<double*> zx(L, nullptr), zy(L, nullptr);
    zx[0] = A.ax;
    zy[0] = A.ay;
    RC(vsolve_T(a, zx.data(), zy.data(), A.lostar.data()));
  }
  RC(coarsify_chain_T(a, A.lostar.data()));
  // the predictor, level by level from the finest (each level reads its coarser neighbour)
  for (int k = 0; k < L; ++k) IB_CUDA_CHECK(cudaMemsetAsync(A.lom_n[k], 0, 8 * (size_t)g.ns, st));
  for (int k = 0; k < L; ++k) {
    // t = (I - cL)^-1 lostar_k (the boundary right-hand side's adjoint), om = (I + cL)(I - cL)^-1 lostar_k
    IB_CUDA_CHECK(cudaMemsetAsync(A.t1, 0, 8 * (size_t)g.ns, st));
    RC(op_predictor(c, k, A.t1, A.zero_v, A.zero_v, A.lostar[k]));
    IB_CUDA_CHECK(cudaMemcpyAsync(A.t2, A.lostar[k], 8 * (size_t)g.ns, cudaMemcpyDeviceToDevice, st));
    RC(op_predictor(c, k, A.t2, A.zero_v, A.zero_v, A.zero_v));
    RC(axpby(st, g.ns, 1.0, A.t2, 1.0, A.lom_n[k], A.lom_n[k]));
    // lrhs = con1 t + lro_k (+ con2 t at the first step, where rhs_old is rhs)
    RC(axpby(st, g.ns, c->con1[k], A.t1, 1.0, A.lro[k], A.t3));
    if (it == 1) {
      RC(axpby(st, g.ns, c->con2[k], A.t1, 1.0, A.t3, A.t3));
      IB_CUDA_CHECK(cudaMemsetAsync(A.lro_n[k], 0, 8 * (size_t)g.ns, st));
    } else {
      RC(axpby(st, g.ns, c->con2[k], A.t1, 0.0, nullptr, A.lro_n[k]));
    }
    // rhsbc = apply_bc(lastbc) + apply_bc(omegabc): both rings' adjoint
    RC(apply_bc_T(g, A.t1, c->vfac[k], A.ring2, st));
    if (k < L - 1) RC(get_bc_T(g, A.ring2, 0.25, A.lostar[k + 1], st));
    // rhs = rot(nonlinear(omega_k, q_k + q0_k, lastbc_k))
    RC(launch_curl(g, A.t3, c->zero_ring, A.hx, A.hy, st));
    if (k < L - 1) RC(launch_get_bc(g, t_om(k + 1), 0.25, A.ring3, st));
    else IB_CUDA_CHECK(cudaMemsetAsync(A.ring3, 0, 8 * (size_t)g.nbc, st));
    IB_CUDA_CHECK(cudaMemsetAsync(A.ring1, 0, 8 * (size_t)g.nbc, st));
    const double* q0x = A.q0 + k * (size_t)(g.nu + g.nv);
    const double* q0y = q0x + g.nu;
    count_launches(2);
    k_adj_nl_vertex<<<blocks((long long)(g.n + 1) * (g.m + 1)), kT, 0, st>>>(g, t_qx(k), q0x, t_qy(k), q0y, A.hx,
                                                                             A.hy, A.lom_n[k], A.ring1);
    k_adj_nl_faces<<<blocks(g.nu + g.nv), kT, 0, st>>>(g, t_om(k), A.ring3, A.hx, A.hy, A.lqx_n[k], A.lqy_n[k]);
    IB_CUDA_CHECK(cudaGetLastError());
    if (k < L - 1) {
      RC(axpby(st, g.nbc, 1.0, A.ring2, 1.0, A.ring1, A.ring1));
      RC(get_bc_T(g, A.ring1, 0.25, A.lom_n[k + 1], st));
    }
  }
  // dJ/d(u, v, W): the frame flux's adjoint (nonlinear's on every level, the Schur right-hand
  // side's on level 0) against each basis
  DotArgs d;
  for (int k = 0; k < L; ++k) { d.lx[k] = A.lqx_n[k]; d.ly[k] = A.lqy_n[k]; }
  d.ax = A.ax; d.ay = A.ay; d.bases = A.bases; d.L = L; d.nu = g.nu; d.nv = g.nv; d.part = A.dpart;
  count_launches(2);
  k_adj_dots<<<dim3(kDotBlocks, 3), 256, 0, st>>>(d);
  k_adj_dots_sum<<<1, 32, 0, st>>>(A.dpart, kDotBlocks, dframe_d);
  IB_CUDA_CHECK(cudaGetLastError());
  std::swap(A.lom, A.lom_n);
  std::swap(A.lqx, A.lqx_n);
  std::swap(A.lqy, A.lqy_n);
  std::swap(A.lro, A.lro_n);
  return IB_OK;
}

// the state a step starts from: omega, s, qx, qy, rhs_old of every level
// The state a checkpoint holds: omega, s, qx, qy, rhs_old of every level, and the forces, the
// next step's Krylov starting guess (so that a recomputed segment repeats the forward exactly).
size_t state_doubles(const Ctx* c) {
  const GridDims& g = c->g;
  return (size_t)c->L * (3 * (size_t)g.ns + g.nu + g.nv) + (size_t)c->nf;
}

int save_state(Ctx* c, double* dst) {
  const GridDims& g = c->g;
  double* p = dst;
  for (int k = 0; k < c->L; ++k) {
    for (auto [src, n] : {std::pair<const double*, size_t>{c->omega[k], (size_t)g.ns}, {c->s[k], (size_t)g.ns},
                          {c->qx[k], (size_t)g.nu}, {c->qy[k], (size_t)g.nv}, {c->rhs_old[k], (size_t)g.ns}}) {
      IB_CUDA_CHECK(cudaMemcpyAsync(p, src, 8 * n, cudaMemcpyDeviceToDevice, c->st));
      p += n;
    }
  }
  IB_CUDA_CHECK(cudaMemcpyAsync(p, c->f, 8 * (size_t)c->nf, cudaMemcpyDeviceToDevice, c->st));
  return IB_OK;
}

int load_state(Ctx* c, const double* src) {
  const GridDims& g = c->g;
  const double* p = src;
  for (int k = 0; k < c->L; ++k) {
    for (auto [dst, n] : {std::pair<double*, size_t>{c->omega[k], (size_t)g.ns}, {c->s[k], (size_t)g.ns},
                          {c->qx[k], (size_t)g.nu}, {c->qy[k], (size_t)g.nv}, {c->rhs_old[k], (size_t)g.ns}}) {
      IB_CUDA_CHECK(cudaMemcpyAsync(dst, p, 8 * n, cudaMemcpyDeviceToDevice, c->st));
      p += n;
    }
  }
  IB_CUDA_CHECK(cudaMemcpyAsync(c->f, p, 8 * (size_t)c->nf, cudaMemcpyDeviceToDevice, c->st));
  return IB_OK;
}

int set_frame(Ctx* c, const double* fr) {
  AdjointState& A = c->adj;
  const GridDims& g = c->g;
  for (int k = 0; k < c->L; ++k) {
    const double* B[3];
    for (int b = 0; b < 3; ++b) B[b] = A.bases + ((size_t)b * c->L + k) * (g.nu + g.nv);
    count_launches(2);
    k_adj_combine<<<blocks(g.nu), kT, 0, c->st>>>(g.nu, B[0], B[1], B[2], fr[0], fr[1], fr[2], c->q0x[k]);
    k_adj_combine<<<blocks(g.nv), kT, 0, c->st>>>(g.nv, B[0] + g.nu, B[1] + g.nu, B[2] + g.nu, fr[0], fr[1], fr[2],
                                                   c->q0y[k]);
  }
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

}  // namespace

void adjoint_free(Ctx* c) {
  AdjointState& A = c->adj;
  if (A.mem) cudaFree(A.mem);
  if (A.ckpt) cudaFree(A.ckpt);
  if (A.tape) cudaFree(A.tape);
  A = AdjointState{};
}

std::vector<double> frame_flux_host(Ctx* c, double u, double v, double w, double cx, double cy) {
  const GridDims& g = c->g;
  const IbParams& p = c->p;
  std::vector<double> out((size_t)c->L * (g.nu + g.nv));
  for (int k = 1; k <= c->L; ++k) {
    double* ax = out.data() + (size_t)(k - 1) * (g.nu + g.nv);
    double* ay = ax + g.nu;
    const double fac = c->delta * std::pow(2.0, k - 1);
    for (int j = 1; j <= g.n; ++j)
      for (int i = 1; i <= g.m + 1; ++i) {
        const double yy = ((double)j - 0.5 - g.n / 2) * c->delta * std::pow(2.0, k - 1) + (g.n / 2) * c->delta - p.offsety;
        ax[(size_t)(j - 1) * g.nux + (i - 1)] = -fac * u + fac * (0.0 + w * (yy - cy));
      }
    for (int j = 1; j <= g.n + 1; ++j)
      for (int i = 1; i <= g.m; ++i) {
        const double xx = ((double)i - 0.5 - g.m / 2) * c->delta * std::pow(2.0, k - 1) + (g.m / 2) * c->delta - p.offsetx;
        ay[(size_t)(j - 1) * g.nvx + (i - 1)] = -fac * v + fac * (0.0 - w * (xx - cx));
      }
  }
  return out;
}

static int adjoint_alloc(Ctx* c) {
  AdjointState& A = c->adj;
  if (A.mem) return IB_OK;
  const GridDims& g = c->g;
  const int L = c->L;
  // bases, the adjoint state twice, scratch
  const size_t per_basis = (size_t)L * (g.nu + g.nv);
  const size_t n = 3 * per_basis + per_basis /* q0 */ + 4 * (size_t)L * g.ns /* lom, lro (x2) */ +
                   2 * (size_t)L * (g.nu + g.nv) /* lq (x2) */ + 2 * (size_t)L * g.ns /* lw, lostar */ +
                   4 * (size_t)g.ns /* t1-t3, zero */ + 3 * (size_t)(g.nu + g.nv) /* hx hy, ax ay */ +
                   3 * (size_t)g.nbc + 2 * (size_t)std::max(c->nf, 1) + 2 * (size_t)std::max(c->nbody, 1) +
                   3 * 4096 + 3 * (size_t)kDotBlocks + (size_t)std::max(c->nf, 1) * std::max(c->nf, 1);
  IB_CUDA_CHECK(cudaMalloc(&A.mem, 8 * n));
  IB_CUDA_CHECK(cudaMemset(A.mem, 0, 8 * n));
  double* p = (double*)A.mem;
  auto take = [&](size_t k) { double* r = p; p += k; return r; };
  A.bases = take(3 * per_basis);
  A.q0 = take(per_basis);
  auto lv = [&](std::vector<double*>& v, size_t each) { v.resize(L); for (int k = 0; k < L; ++k) v[k] = take(each); };
  lv(A.lom, g.ns); lv(A.lom_n, g.ns); lv(A.lro, g.ns); lv(A.lro_n, g.ns);
  lv(A.lqx, g.nu); lv(A.lqy, g.nv); lv(A.lqx_n, g.nu); lv(A.lqy_n, g.nv);
  lv(A.lw, g.ns); lv(A.lostar, g.ns);
  A.t1 = take(g.ns); A.t2 = take(g.ns); A.t3 = take(g.ns); A.zero_v = take(g.ns);
  A.hx = take(g.nu); A.hy = take(g.nv); A.ax = take(g.nu); A.ay = take(g.nv);
  take(g.nu + g.nv);
  A.ring1 = take(g.nbc); A.ring2 = take(g.nbc); A.ring3 = take(g.nbc);
  A.lf = take(std::max(c->nf, 1)); A.lrhsf = take(std::max(c->nf, 1));
  A.dforce = take(2 * (size_t)std::max(c->nbody, 1));
  A.dframe = take(3 * 4096);
  A.dpart = take(3 * (size_t)kDotBlocks);
  A.opT = take((size_t)std::max(c->nf, 1) * std::max(c->nf, 1));
  const double cx = c->p.motion[3], cy = c->p.motion[4];
  for (int b = 0; b < 3; ++b) {
    std::vector<double> h = frame_flux_host(c, b == 0, b == 1, b == 2, cx, cy);
    IB_CUDA_CHECK(cudaMemcpy(A.bases + b * per_basis, h.data(), 8 * per_basis, cudaMemcpyHostToDevice));
  }
  return IB_OK;
}

int op_adjoint_forward(Ctx* c, int nsteps, int K, const double* frames, double* forces, std::string* msg) {
  AdjointState& A = c->adj;
  if (c->nt > 0 || c->nbeam > 0 || c->nf == 0) {
    *msg = "the adjoint covers stationary rigid bodies";
    return IB_ERR_ARG;
  }
  if (!c->p.num_stat && (c->p.schur_mode != 0 || !c->use_fused)) {
    *msg = "without num_stat the adjoint needs the assembled operator and the cluster solver (schur_mode 0)";
    return IB_ERR_ARG;
  }
  if (nsteps <= 0 || K <= 0 || nsteps > 4096) {
    *msg = "nsteps in 1..4096 and K >= 1";
    return IB_ERR_ARG;
  }
  RC(adjoint_alloc(c));
  const int nseg = (nsteps + K - 1) / K;
  const size_t sd = state_doubles(c);
  if (A.ckpt) cudaFree(A.ckpt);
  if (A.tape) cudaFree(A.tape);
  A.ckpt = nullptr;
  A.tape = nullptr;
  {
    size_t freeb = 0, totalb = 0;
    IB_CUDA_CHECK(cudaMemGetInfo(&freeb, &totalb));
    const size_t need = 8 * (sd * (nseg + 1) + (size_t)K * c->L * (c->g.ns + c->g.nu + c->g.nv));
    if (need > freeb / 2) {
      *msg = "checkpoints and tape do not fit in device memory (raise K?)";
      return IB_ERR_NOMEM;
    }
  }
  IB_CUDA_CHECK(cudaMalloc(&A.ckpt, 8 * sd * (nseg + 1)));
  IB_CUDA_CHECK(cudaMalloc(&A.tape, 8 * (size_t)K * c->L * (c->g.ns + c->g.nu + c->g.nv)));
  A.nsteps = nsteps;
  A.K = K;
  A.nseg = nseg;
  A.frames.assign(frames, frames + 3 * (size_t)nsteps);
  A.it_ckpt.assign(nseg + 1, 0);
  A.ready = false;
  for (int n = 0; n < nsteps; ++n) {
    if (n % K == 0) {
      RC(save_state(c, A.ckpt + sd * (n / K)));
      A.it_ckpt[n / K] = c->itime;
    }
    RC(set_frame(c, frames + 3 * (size_t)n));
    RC(op_advance(c));
    RC(launch_force_coeffs(c->nf, c->nbody, c->comp, c->bid, c->f, c->p.dt, c->delta, c->forces, c->st));
    std::vector<double> fc(2 * (size_t)c->nbody);
    IB_CUDA_CHECK(cudaMemcpyAsync(fc.data(), c->forces, 16 * (size_t)c->nbody, cudaMemcpyDeviceToHost, c->st));
    IB_CUDA_CHECK(cudaStreamSynchronize(c->st));
    for (int b = 0; b < c->nbody; ++b) {
      forces[((size_t)n * c->nbody + b) * 2] = fc[b];
      forces[((size_t)n * c->nbody + b) * 2 + 1] = fc[c->nbody + b];
    }
  }
  RC(save_state(c, A.ckpt + sd * nseg));
  A.it_ckpt[nseg] = c->itime;
  IB_CUDA_CHECK(cudaStreamSynchronize(c->st));
  A.ready = true;
  return IB_OK;
}

int op_adjoint_backward(Ctx* c, const double* dforces, double* dframes, std::string* msg) {
  AdjointState& A = c->adj;
  if (!A.ready) {
    *msg = "no adjoint forward to reverse";
    return IB_ERR_STATE;
  }
  const GridDims& g = c->g;
  const int L = c->L;
  const size_t sd = state_doubles(c);
  const size_t per = (size_t)g.ns + g.nu + g.nv;
  Adj a{c, A, g, L, c->st};
  // the adjoint state after the last step: zero
  for (int k = 0; k < L; ++k) {
    IB_CUDA_CHECK(cudaMemsetAsync(A.lom[k], 0, 8 * (size_t)g.ns, c->st));
    IB_CUDA_CHECK(cudaMemsetAsync(A.lro[k], 0, 8 * (size_t)g.ns, c->st));
    IB_CUDA_CHECK(cudaMemsetAsync(A.lqx[k], 0, 8 * (size_t)g.nu, c->st));
    IB_CUDA_CHECK(cudaMemsetAsync(A.lqy[k], 0, 8 * (size_t)g.nv, c->st));
  }
  const bool graphs = c->use_whole_step;
  for (int seg = A.nseg - 1; seg >= 0; --seg) {
    const int n0 = seg * A.K, n1 = std::min(A.nsteps, n0 + A.K);
    // recompute the segment from its checkpoint, taping each step's inputs
    RC(load_state(c, A.ckpt + sd * seg));
    c->itime = A.it_ckpt[seg];
    for (int n = n0; n < n1; ++n) {
      double* tp = A.tape + (size_t)(n - n0) * L * per;
      for (int k = 0; k < L; ++k) {
        IB_CUDA_CHECK(cudaMemcpyAsync(tp + k * per, c->omega[k], 8 * (size_t)g.ns, cudaMemcpyDeviceToDevice, c->st));
        IB_CUDA_CHECK(cudaMemcpyAsync(tp + k * per + g.ns, c->qx[k], 8 * (size_t)g.nu, cudaMemcpyDeviceToDevice, c->st));
        IB_CUDA_CHECK(cudaMemcpyAsync(tp + k * per + g.ns + g.nu, c->qy[k], 8 * (size_t)g.nv, cudaMemcpyDeviceToDevice,
                                      c->st));
      }
      RC(set_frame(c, A.frames.data() + 3 * (size_t)n));
      RC(op_advance(c));
    }
    // reverse the segment
    for (int n = n1 - 1; n >= n0; --n) {
      const int it = (int)(A.it_ckpt[seg] + (n - n0) + 1);
      RC(step_T(a, n - n0, it, A.frames.data() + 3 * (size_t)n, dforces + 2 * (size_t)n * c->nbody,
                A.dframe + 3 * (size_t)n));
    }
  }
  (void)graphs;
  IB_CUDA_CHECK(cudaMemcpyAsync(dframes, A.dframe, 24 * (size_t)A.nsteps, cudaMemcpyDeviceToHost, c->st));
  // the context continues from the end of the forward
  RC(load_state(c, A.ckpt + sd * A.nseg));
  c->itime = A.it_ckpt[A.nseg];
  RC(set_frame(c, A.frames.data() + 3 * (size_t)(A.nsteps - 1)));
  IB_CUDA_CHECK(cudaStreamSynchronize(c->st));
  return check_err(c);
}

}  // namespace ib
