// Euler-Bernoulli beams (body family 3).  The reference declares the family and leaves its
// routines empty (operators_struct.F90:104-106, 146-148, 171-174, 285-288, 378-381, 472-474);
// this is the library's own formulation, coupled the way the reference couples its torsional
// body (operators_struct.F90:14-505) with matrices in place of the hinge's scalars:
//   * a linear (small-deflection) beam clamped at its first point, along the line from its
//     first to its last point; nel Hermite-cubic elements with DOFs (w, dw/ds) at the nodes,
//     the clamped node's removed (ndof = 2 nel); consistent mass and stiffness;
//   * body point j moves by W q along the beam's normal, W = [-sin g Phi; cos g Phi]; point
//     forces act on the DOFs as F = (delta/dt) W^T f;
//   * trapezoidal Newmark with K_eff = 4/dt^2 M + K:
//       dq = K_eff^-1 (M a - K_eff q) + K_eff^-1 F,  a = 4/dt^2 q0 + 4/dt qd0 + qdd0;
//       compute_rhs: delta W (r - jr - qd), r = qd0 + qd + 2/dt (q0 - q),
//                    jr = 2/dt K_eff^-1 (M a - K_eff q);
//       b_times: (2 delta^2 / dt^2) W K_eff^-1 W^T x;   initial_acc: qdd = M^-1 (F - K q).
// The matrices are built on the host at context creation (the beam is linear, so they never
// change); the kernels are dense products on one CTA, which runs every beam in turn.
#include <cmath>
#include <vector>

#include "ctx.cuh"

namespace ib {

namespace {

// inverse of an SPD matrix (row-major, n x n) by Cholesky, in double
bool spd_inverse(const std::vector<double>& A, int n, std::vector<double>* out) {
  std::vector<double> L((size_t)n * n, 0.0);
  for (int j = 0; j < n; ++j) {
    double d = A[(size_t)j * n + j];
    for (int k = 0; k < j; ++k) d -= L[(size_t)j * n + k] * L[(size_t)j * n + k];
    if (!(d > 0.0)) return false;
    const double ljj = std::sqrt(d);
    L[(size_t)j * n + j] = ljj;
    for (int i = j + 1; i < n; ++i) {
      double v = A[(size_t)i * n + j];
      for (int k = 0; k < j; ++k) v -= L[(size_t)i * n + k] * L[(size_t)j * n + k];
      L[(size_t)i * n + j] = v / ljj;
    }
  }
  out->assign((size_t)n * n, 0.0);
  std::vector<double> col(n);
  for (int c = 0; c < n; ++c) {
    for (int i = 0; i < n; ++i) {   // L y = e_c
      double v = i == c ? 1.0 : 0.0;
      for (int k = 0; k < i; ++k) v -= L[(size_t)i * n + k] * col[k];
      col[i] = v / L[(size_t)i * n + i];
    }
    for (int i = n - 1; i >= 0; --i) {   // L^T x = y
      double v = col[i];
      for (int k = i + 1; k < n; ++k) v -= L[(size_t)k * n + i] * col[k];
      col[i] = v / L[(size_t)i * n + i];
    }
    for (int i = 0; i < n; ++i) (*out)[(size_t)i * n + c] = col[i];
  }
  return true;
}

}  // namespace

int beam_build(Ctx* c, const IbBody* bodies, int nbody, std::string* msg) {
  const double dt = c->p.dt;
  int off = 0;
  std::vector<BeamDev> hdev;
  for (int i = 0; i < nbody; ++i) {
    const IbBody& b = bodies[i];
    const int npts = b.npts;
    if (b.fam != 3) { off += 2 * npts; continue; }
    const int nel = b.nelem > 0 ? b.nelem : (npts - 1) / 2;
    if (nel < 1) { *msg = "a beam needs at least one element"; return IB_ERR_ARG; }
    if (!(b.itheta > 0) || !(b.ktheta > 0)) { *msg = "a beam needs mass per length (itheta) and EI (ktheta) > 0"; return IB_ERR_ARG; }
    const int nd = 2 * nel, np2 = 2 * npts;
    const double dx = b.x[npts - 1] - b.x[0], dy = b.y[npts - 1] - b.y[0];
    const double length = std::sqrt(dx * dx + dy * dy);
    const double cg = dx / length, sg = dy / length;
    const double h = length / nel, rho = b.itheta, EI = b.ktheta;
    const double kc = EI / (h * h * h), mc = rho * h / 420.0;
    const double ke[4][4] = {{12.0, 6.0 * h, -12.0, 6.0 * h}, {6.0 * h, 4.0 * h * h, -6.0 * h, 2.0 * h * h},
                             {-12.0, -6.0 * h, 12.0, -6.0 * h}, {6.0 * h, 2.0 * h * h, -6.0 * h, 4.0 * h * h}};
    const double me[4][4] = {{156.0, 22.0 * h, 54.0, -13.0 * h}, {22.0 * h, 4.0 * h * h, 13.0 * h, -3.0 * h * h},
                             {54.0, 13.0 * h, 156.0, -22.0 * h}, {-13.0 * h, -3.0 * h * h, -22.0 * h, 4.0 * h * h}};
    const int NG = 2 * (nel + 1);
    std::vector<double> KG((size_t)NG * NG, 0.0), MG((size_t)NG * NG, 0.0);
    for (int e = 0; e < nel; ++e)
      for (int a = 0; a < 4; ++a)
        for (int q = 0; q < 4; ++q) {
          KG[(size_t)(2 * e + a) * NG + 2 * e + q] += kc * ke[a][q];
          MG[(size_t)(2 * e + a) * NG + 2 * e + q] += mc * me[a][q];
        }
    std::vector<double> K((size_t)nd * nd), M((size_t)nd * nd), Ke((size_t)nd * nd);
    for (int r = 0; r < nd; ++r)
      for (int q = 0; q < nd; ++q) {
        K[(size_t)r * nd + q] = KG[(size_t)(r + 2) * NG + q + 2];
        M[(size_t)r * nd + q] = MG[(size_t)(r + 2) * NG + q + 2];
        Ke[(size_t)r * nd + q] = 4.0 / (dt * dt) * M[(size_t)r * nd + q] + K[(size_t)r * nd + q];
      }
    std::vector<double> Ki, Mi;
    if (!spd_inverse(Ke, nd, &Ki) || !spd_inverse(M, nd, &Mi)) { *msg = "beam matrices not positive definite"; return IB_ERR_ARG; }
    std::vector<double> phi((size_t)npts * nd, 0.0), W((size_t)np2 * nd);
    for (int j = 0; j < npts; ++j) {
      const int e = std::min((int)((long long)j * nel / (npts - 1)), nel - 1);
      const double xi = (double)((long long)j * nel - (long long)e * (npts - 1)) / (double)(npts - 1);
      const double xi2 = xi * xi, xi3 = xi * xi * xi;
      const double nv[4] = {1.0 - 3.0 * xi2 + 2.0 * xi3, h * (xi - 2.0 * xi2 + xi3), 3.0 * xi2 - 2.0 * xi3,
                            h * (xi3 - xi2)};
      for (int a = 0; a < 4; ++a) {
        const int dof = 2 * e + a - 2;
        if (dof >= 0) phi[(size_t)j * nd + dof] = nv[a];
      }
    }
    for (int j = 0; j < npts; ++j)
      for (int q = 0; q < nd; ++q) {
        W[(size_t)j * nd + q] = -sg * phi[(size_t)j * nd + q];
        W[(size_t)(npts + j) * nd + q] = cg * phi[(size_t)j * nd + q];
      }
    // B = W K_eff^-1 W^T
    std::vector<double> KiWt((size_t)nd * np2, 0.0), B((size_t)np2 * np2, 0.0);
    for (int r = 0; r < nd; ++r)
      for (int j = 0; j < np2; ++j) {
        double s = 0.0;
        for (int q = 0; q < nd; ++q) s += Ki[(size_t)r * nd + q] * W[(size_t)j * nd + q];
        KiWt[(size_t)r * np2 + j] = s;
      }
    for (int i2 = 0; i2 < np2; ++i2)
      for (int j = 0; j < np2; ++j) {
        double s = 0.0;
        for (int q = 0; q < nd; ++q) s += W[(size_t)i2 * nd + q] * KiWt[(size_t)q * np2 + j];
        B[(size_t)i2 * np2 + j] = s;
      }
    // device storage of this beam: matrices, reference positions, state (+ scratch)
    const size_t nmat = (size_t)5 * nd * nd + (size_t)np2 * nd + (size_t)npts * nd + (size_t)np2 * np2 + np2 + 10 * (size_t)nd;
    double* mem = nullptr;
    if (cudaMalloc(&mem, 8 * nmat) != cudaSuccess) { *msg = "beam allocation failed"; return IB_ERR_NOMEM; }
    c->beam_mem.push_back(mem);
    cudaMemset(mem, 0, 8 * nmat);
    BeamDev d;
    d.off = off; d.npts = npts; d.ndof = nd; d.sg = sg; d.cg = cg;
    double* q = mem;
    auto put = [&](const std::vector<double>& v) { double* r = q; cudaMemcpy(r, v.data(), 8 * v.size(), cudaMemcpyHostToDevice); q += v.size(); return r; };
    d.M = put(M); d.K = put(K); d.Ke = put(Ke); d.Ki = put(Ki); d.Mi = put(Mi);
    d.W = put(W); d.phi = put(phi); d.B = put(B);
    std::vector<double> xy(np2);
    for (int j = 0; j < npts; ++j) { xy[j] = b.x[j]; xy[npts + j] = b.y[j]; }
    d.xy0 = put(xy);
    d.q = q; d.qd = q + nd; d.qdd = q + 2 * nd; d.q0 = q + 3 * nd; d.qd0 = q + 4 * nd; d.qdd0 = q + 5 * nd;
    d.t1 = q + 6 * nd; d.t2 = q + 7 * nd; d.t3 = q + 8 * nd; d.t4 = q + 9 * nd;
    hdev.push_back(d);
    off += np2;
  }
  c->nbeam = (int)hdev.size();
  c->beams_h = hdev;
  if (c->nbeam > 0) {
    if (cudaMalloc(&c->beams, sizeof(BeamDev) * c->nbeam) != cudaSuccess) { *msg = "beam allocation failed"; return IB_ERR_NOMEM; }
    if (cudaMemcpy(c->beams, hdev.data(), sizeof(BeamDev) * c->nbeam, cudaMemcpyHostToDevice) != cudaSuccess)
      return IB_ERR_CUDA;
    if (cudaDeviceSynchronize() != cudaSuccess) return IB_ERR_CUDA;
  }
  return IB_OK;
}

void beam_free(Ctx* c) {
  for (double* m : c->beam_mem) cudaFree(m);
  c->beam_mem.clear();
  if (c->beams) cudaFree(c->beams);
  c->beams = nullptr;
  c->nbeam = 0;
}

// out[r] = sum_q A[r][q] x[q] over the CTA, one row per thread (the sum in column order)
__device__ void cta_matvec(const double* __restrict__ A, int rows, int cols, const double* x, double* out) {
  for (int r = threadIdx.x; r < rows; r += blockDim.x) {
    double s = 0.0;
    for (int q = 0; q < cols; ++q) s = fma(A[(size_t)r * cols + q], x[q], s);
    out[r] = s;
  }
  __syncthreads();
}

// a = 4/dt^2 q0 + 4/dt qd0 + qdd0 into t1; v = M a - K_eff q into t3
__device__ void beam_mv_residual(const BeamDev& b, double dt) {
  const int nd = b.ndof;
  for (int k = threadIdx.x; k < nd; k += blockDim.x) b.t1[k] = 4.0 / (dt * dt) * b.q0[k] + 4.0 / dt * b.qd0[k] + b.qdd0[k];
  __syncthreads();
  cta_matvec(b.M, nd, nd, b.t1, b.t2);
  cta_matvec(b.Ke, nd, nd, b.q, b.t3);
  for (int k = threadIdx.x; k < nd; k += blockDim.x) b.t3[k] = b.t2[k] - b.t3[k];
  __syncthreads();
}

__global__ void k_beam_rhs(const BeamDev* __restrict__ beams, int nbeam, double dt, double delta, double* y) {
  IB_GRID_DEP_WAIT();
  for (int i = 0; i < nbeam; ++i) {
    const BeamDev b = beams[i];
    const int nd = b.ndof;
    beam_mv_residual(b, dt);
    cta_matvec(b.Ki, nd, nd, b.t3, b.t4);   // K_eff^-1 (M a - K_eff q)
    for (int k = threadIdx.x; k < nd; k += blockDim.x) {
      const double r = b.qd0[k] + b.qd[k] + 2.0 / dt * (b.q0[k] - b.q[k]);
      const double jr = 2.0 / dt * b.t4[k];
      b.t1[k] = delta * (r - jr - b.qd[k]);
    }
    __syncthreads();
    cta_matvec(b.W, 2 * b.npts, nd, b.t1, y + b.off);
  }
}

__global__ void k_beam_dx(const BeamDev* __restrict__ beams, int nbeam, double dt, double delta,
                          const double* __restrict__ f, double* xb, double* yb, double* err) {
  IB_GRID_DEP_WAIT();
  __shared__ double red[32];
  double emax = err[0];   // the torsional bodies' maximum (zero without them)
  for (int i = 0; i < nbeam; ++i) {
    const BeamDev b = beams[i];
    const int nd = b.ndof, np2 = 2 * b.npts;
    beam_mv_residual(b, dt);
    // F = (delta/dt) W^T f into t1 (column sums of W in row order)
    for (int k = threadIdx.x; k < nd; k += blockDim.x) {
      double s = 0.0;
      for (int j = 0; j < np2; ++j) s = fma(b.W[(size_t)j * nd + k], f[b.off + j], s);
      b.t1[k] = delta / dt * s;
    }
    __syncthreads();
    cta_matvec(b.Ki, nd, nd, b.t3, b.t2);   // K_eff^-1 (M a - K_eff q)
    cta_matvec(b.Ki, nd, nd, b.t1, b.t4);   // K_eff^-1 F
    double em = 0.0;
    for (int k = threadIdx.x; k < nd; k += blockDim.x) {
      const double dq = b.t2[k] + b.t4[k];
      em = fmax(em, fabs(dq));
      const double qn = b.q[k] + dq;
      b.q[k] = qn;
      b.qd[k] = -b.qd0[k] + 2.0 / dt * (qn - b.q0[k]);
      b.qdd[k] = -b.qdd0[k] - 4.0 / dt * b.qd0[k] + 4.0 / (dt * dt) * (qn - b.q0[k]);
    }
    for (int o = 16; o > 0; o >>= 1) em = fmax(em, __shfl_xor_sync(0xffffffffu, em, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = em;
    __syncthreads();
    if (threadIdx.x == 0)
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) emax = fmax(emax, red[w]);
    // positions: x0 + (-sin g) d, y0 + cos g d, d = Phi q
    cta_matvec(b.phi, b.npts, nd, b.q, b.t1);
    for (int j = threadIdx.x; j < b.npts; j += blockDim.x) {
      const double px = __dadd_rn(b.xy0[j], __dmul_rn(-b.sg, b.t1[j]));
      const double py = __dadd_rn(b.xy0[b.npts + j], __dmul_rn(b.cg, b.t1[j]));
      xb[b.off + j] = px; xb[b.off + b.npts + j] = px;
      yb[b.off + j] = py; yb[b.off + b.npts + j] = py;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) err[0] = emax;
}

__global__ void k_beam_btimes(const BeamDev* __restrict__ beams, int nbeam, double scale,
                              const double* __restrict__ x, double* y) {
  IB_GRID_DEP_WAIT();
  for (int i = 0; i < nbeam; ++i) {
    const BeamDev b = beams[i];
    const int np2 = 2 * b.npts;
    for (int r = threadIdx.x; r < np2; r += blockDim.x) {
      double s = 0.0;
      for (int q = 0; q < np2; ++q) s = fma(b.B[(size_t)r * np2 + q], x[b.off + q], s);
      y[b.off + r] = y[b.off + r] + s * scale;
    }
    __syncthreads();
  }
}

// St (column-major nf x nf) += scale B on each beam's block
__global__ void k_beam_add_b(const BeamDev* __restrict__ beams, int nbeam, double scale, int nf, double* St) {
  IB_GRID_DEP_WAIT();
  for (int i = 0; i < nbeam; ++i) {
    const BeamDev b = beams[i];
    const int np2 = 2 * b.npts;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < np2 * np2; t += gridDim.x * blockDim.x) {
      const int r = t / np2, q = t % np2;
      double* e = St + (size_t)(b.off + q) * nf + (b.off + r);
      *e = *e + b.B[(size_t)r * np2 + q] * scale;
    }
  }
}

__global__ void k_beam_initial_acc(const BeamDev* __restrict__ beams, int nbeam, double dt, double delta,
                                   const double* __restrict__ f) {
  IB_GRID_DEP_WAIT();
  for (int i = 0; i < nbeam; ++i) {
    const BeamDev b = beams[i];
    const int nd = b.ndof, np2 = 2 * b.npts;
    for (int k = threadIdx.x; k < nd; k += blockDim.x) {
      double s = 0.0;
      for (int j = 0; j < np2; ++j) s = fma(b.W[(size_t)j * nd + k], f[b.off + j], s);
      b.t1[k] = delta / dt * s;
    }
    __syncthreads();
    cta_matvec(b.K, nd, nd, b.q, b.t2);
    for (int k = threadIdx.x; k < nd; k += blockDim.x) b.t3[k] = b.t1[k] - b.t2[k];
    __syncthreads();
    cta_matvec(b.Mi, nd, nd, b.t3, b.qdd);
  }
}

__global__ void k_beam_save(const BeamDev* __restrict__ beams, int nbeam) {
  IB_GRID_DEP_WAIT();
  for (int i = 0; i < nbeam; ++i) {
    const BeamDev b = beams[i];
    for (int k = threadIdx.x; k < b.ndof; k += blockDim.x) {
      b.q0[k] = b.q[k];
      b.qd0[k] = b.qd[k];
      b.qdd0[k] = b.qdd[k];
    }
  }
}

static int after(int rc) { return rc == IB_OK && cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA; }

int launch_beam_rhs(Ctx* c, double* y, cudaStream_t st) {
  if (c->nbeam == 0) return IB_OK;
  count_launch();
  k_beam_rhs<<<1, 256, 0, st>>>(c->beams, c->nbeam, c->p.dt, c->delta, y);
  return after(IB_OK);
}
int launch_beam_dx(Ctx* c, const double* f, cudaStream_t st) {
  if (c->nbeam == 0) return IB_OK;
  count_launch();
  k_beam_dx<<<1, 256, 0, st>>>(c->beams, c->nbeam, c->p.dt, c->delta, f, c->xb, c->yb, c->err_fsi);
  return after(IB_OK);
}
int launch_beam_btimes(Ctx* c, const double* x, double* y, cudaStream_t st) {
  if (c->nbeam == 0) return IB_OK;
  count_launch();
  const double dt = c->p.dt;
  k_beam_btimes<<<1, 256, 0, st>>>(c->beams, c->nbeam, 2.0 * c->delta * c->delta / (dt * dt), x, y);
  return after(IB_OK);
}
int launch_beam_add_b(Ctx* c, double* St, cudaStream_t st) {
  if (c->nbeam == 0) return IB_OK;
  count_launch();
  const double dt = c->p.dt;
  k_beam_add_b<<<64, 256, 0, st>>>(c->beams, c->nbeam, 2.0 * c->delta * c->delta / (dt * dt), c->nf, St);
  return after(IB_OK);
}
int launch_beam_initial_acc(Ctx* c, const double* f, cudaStream_t st) {
  if (c->nbeam == 0) return IB_OK;
  count_launch();
  k_beam_initial_acc<<<1, 256, 0, st>>>(c->beams, c->nbeam, c->p.dt, c->delta, f);
  return after(IB_OK);
}
int launch_beam_save(Ctx* c, cudaStream_t st) {
  if (c->nbeam == 0) return IB_OK;
  count_launch();
  k_beam_save<<<1, 256, 0, st>>>(c->beams, c->nbeam);
  return after(IB_OK);
}

}  // namespace ib
