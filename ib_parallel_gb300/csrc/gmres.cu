// Device GMRES with the semantics of PETSc 3.11 KSPGMRES as the reference
// configures it (variables.F90:565-574): restart 30, classical Gram-Schmidt
// without refinement (borthog2.c), Givens-rotation least squares, nonzero
// initial guess, unpreconditioned residual norm, convergence when the rotated
// residual estimate <= max(rtol*||b||, atol) (KSPConvergedDefault).  Each kernel
// is one CTA; the operator (the Schur matvec) runs between them and reads
// G.xin, writes G.Av.
#include "kernels.cuh"

namespace ib {

constexpr int kGmresThreads = 512;

__device__ double blk_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
    red[32] = s;
  }
  __syncthreads();
  return red[32];
}

__global__ void k_gmres_init(GmresDev G) {
  if (threadIdx.x == 0) {
    G.ist[0] = 0; G.ist[1] = 0; G.ist[2] = 0; G.ist[3] = 0; G.ist[4] = 0;
  }
}

// Cycle start: r = b - A x (A x in G.Av), V0 = r/||r||, tolerance on the first cycle.
__global__ void k_gmres_start(GmresDev G, const double* __restrict__ b, const double* __restrict__ x, double rtol,
                              double atol, int max_it, cudaGraphConditionalHandle h_inner, int use_cond) {
  __shared__ double red[33];
  const int nf = G.nf;
  double pr = 0.0, pb = 0.0;
  for (int i = threadIdx.x; i < nf; i += blockDim.x) {
    double r = b[i] - G.Av[i];
    G.V[i] = r;
    pr += r * r;
    pb += b[i] * b[i];
  }
  double rnorm = sqrt(blk_sum(pr, red));
  double bnorm = sqrt(blk_sum(pb, red));
  int its = G.ist[0];
  double ttol;
  if (its == 0) {
    double rnorm0 = bnorm != 0.0 ? bnorm : rnorm;
    ttol = fmax(rtol * rnorm0, atol);
  } else {
    ttol = G.scal[0];
  }
  double inv = rnorm != 0.0 ? 1.0 / rnorm : 0.0;
  for (int i = threadIdx.x; i < nf; i += blockDim.x) {
    double v = rnorm != 0.0 ? G.V[i] * inv : G.V[i];
    G.V[i] = v;
    G.xin[i] = v;
  }
  if (threadIdx.x == 0) {
    G.scal[0] = ttol;
    G.scal[1] = rnorm;
    G.scal[2] = bnorm;
    G.scal[3] = rnorm;
    G.g[0] = rnorm;
    G.ist[2] = 0;
    int reason = 0;
    if (rnorm == 0.0) reason = 2;                 // KSP_CONVERGED_ATOL (zero residual)
    else if (rnorm <= ttol) reason = 3;           // converged at the initial residual
    else if (its >= max_it) reason = -3;
    G.ist[1] = reason;
    G.ist[3] = reason == 0 ? 1 : 0;
    G.ist[4] += 1;  // restart cycles
    if (use_cond) cudaGraphSetConditional(h_inner, reason == 0 ? 1u : 0u);
  }
}

// One Arnoldi step on w = A V[it] (in G.Av): classical Gram-Schmidt (all projections
// against the unmodified w, one warp per projection), normalisation, Givens update.
__global__ void k_gmres_arnoldi(GmresDev G, int max_it, cudaGraphConditionalHandle h_inner, int use_cond) {
  __shared__ double red[33];
  __shared__ double h[64];
  if (G.ist[3] == 0) {
    if (use_cond && threadIdx.x == 0) cudaGraphSetConditional(h_inner, 0u);
    return;
  }
  const int nf = G.nf, R = G.restart;
  const int it = G.ist[2];
  double* w = G.V + (size_t)(it + 1) * nf;
  const double* Av = G.Av;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int j = warp; j <= it; j += nwarps) {
    const double* vj = G.V + (size_t)j * nf;
    double p = 0.0;
    for (int i = lane; i < nf; i += 32) p += Av[i] * vj[i];
    for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
    if (lane == 0) h[j] = p;
  }
  __syncthreads();
  double pn = 0.0;
  for (int i = threadIdx.x; i < nf; i += blockDim.x) {
    double v = Av[i];
    for (int j = 0; j <= it; ++j) v = v - h[j] * G.V[(size_t)j * nf + i];
    w[i] = v;
    pn += v * v;
  }
  double tt = sqrt(blk_sum(pn, red));
  double inv = tt != 0.0 ? 1.0 / tt : 0.0;
  for (int i = threadIdx.x; i < nf; i += blockDim.x) {
    double v = tt != 0.0 ? w[i] * inv : w[i];
    w[i] = v;
    G.xin[i] = v;
  }
  if (threadIdx.x == 0) {
    double* col = G.H + (size_t)it * (R + 1);
    for (int j = 0; j <= it; ++j) col[j] = h[j];
    col[it + 1] = tt;
    double hapbnd = fabs(tt / G.g[it]);
    if (hapbnd > 1.0e-30) hapbnd = 1.0e-30;
    bool hapend = tt < hapbnd;
    for (int j = 0; j < it; ++j) {
      double t0 = col[j];
      col[j] = G.cs[j] * t0 + G.sn[j] * col[j + 1];
      col[j + 1] = G.cs[j] * col[j + 1] - G.sn[j] * t0;
    }
    double res;
    int reason = 0;
    if (!hapend) {
      double nrm = sqrt(col[it] * col[it] + col[it + 1] * col[it + 1]);
      if (nrm == 0.0) {
        reason = -9;  // KSP_DIVERGED_NULL
        res = G.scal[1];
      } else {
        G.cs[it] = col[it] / nrm;
        G.sn[it] = col[it + 1] / nrm;
        G.g[it + 1] = -(G.sn[it] * G.g[it]);
        G.g[it] = G.cs[it] * G.g[it];
        col[it] = G.cs[it] * col[it] + G.sn[it] * col[it + 1];
        res = fabs(G.g[it + 1]);
      }
    } else {
      res = 0.0;
    }
    int itn = it + 1;
    int its = G.ist[0] + 1;
    G.ist[2] = itn;
    G.ist[0] = its;
    G.scal[1] = res;
    if (reason == 0) {
      if (res <= G.scal[0]) reason = 2;
      else if (hapend) reason = -3;
    }
    G.ist[1] = reason;
    int active = (reason == 0 && itn < R && its < max_it) ? 1 : 0;
    G.ist[3] = active;
    if (use_cond) cudaGraphSetConditional(h_inner, (unsigned)active);
  }
}

// KSPGMRESBuildSoln: back substitution and x += V y.
__global__ void k_gmres_update(GmresDev G, double* __restrict__ x, int max_it, cudaGraphConditionalHandle h_outer,
                               int use_cond) {
  __shared__ double y[64];
  const int nf = G.nf, R = G.restart;
  const int it = G.ist[2];
  if (threadIdx.x == 0 && it > 0) {
    int k = it - 1;
    const double* H = G.H;
    auto HH = [&](int r, int c) { return H[(size_t)c * (R + 1) + r]; };
    y[k] = G.g[k] / HH(k, k);
    for (int i = k - 1; i >= 0; --i) {
      double tt = G.g[i];
      for (int j = i + 1; j <= k; ++j) tt = tt - HH(i, j) * y[j];
      y[i] = tt / HH(i, i);
    }
  }
  __syncthreads();
  if (it > 0) {
    for (int i = threadIdx.x; i < nf; i += blockDim.x) {
      double u = 0.0;
      for (int j = 0; j < it; ++j) u = u + y[j] * G.V[(size_t)j * nf + i];
      x[i] = x[i] + u;
    }
  }
  if (threadIdx.x == 0) {
    G.ist[3] = 0;
    if (use_cond) cudaGraphSetConditional(h_outer, (G.ist[1] == 0 && G.ist[0] < max_it) ? 1u : 0u);
  }
}

__global__ void k_copy(int n, const double* __restrict__ a, double* __restrict__ b) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}

int launch_gmres_init(const GmresDev& G, cudaStream_t st) {
  count_launch();
  k_gmres_init<<<1, 32, 0, st>>>(G);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}
int launch_gmres_start(const GmresDev& G, const double* b, const double* x, double rtol, double atol, int max_it,
                       cudaStream_t st, cudaGraphConditionalHandle h, int use_cond) {
  count_launch();
  k_gmres_start<<<1, kGmresThreads, 0, st>>>(G, b, x, rtol, atol, max_it, h, use_cond);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}
int launch_gmres_arnoldi(const GmresDev& G, int max_it, cudaStream_t st, cudaGraphConditionalHandle h,
                         int use_cond) {
  count_launch();
  k_gmres_arnoldi<<<1, kGmresThreads, 0, st>>>(G, max_it, h, use_cond);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}
int launch_gmres_update(const GmresDev& G, double* x, int max_it, cudaStream_t st, cudaGraphConditionalHandle h,
                        int use_cond) {
  count_launch();
  k_gmres_update<<<1, kGmresThreads, 0, st>>>(G, x, max_it, h, use_cond);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}
int launch_copy(int n, const double* a, double* b, cudaStream_t st) {
  if (n <= 0) return IB_OK;
  count_launch();
  k_copy<<<cdiv(n, 256), 256, 0, st>>>(n, a, b);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

// ---------------------------------------------------------------- Cholesky
// Dense Cholesky of the upper triangle of A (row-major n x n: A[i*n+j], the
// reference factors the upper triangle, PETSc MATSOLVERELEMENTAL), producing the
// lower factor L in place of the lower triangle (L[i*n+j], j<=i).  One CTA,
// right-looking, column by column.
__global__ void k_cholesky(int n, double* A, int* err) {
  __shared__ double piv;
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      double d = A[(size_t)k * n + k];
      if (!(d > 0.0)) { atomicExch(err, IB_ERR_ARG); d = 1.0; }
      piv = sqrt(d);
      A[(size_t)k * n + k] = piv;
    }
    __syncthreads();
    // column k below the diagonal, read from the upper triangle (A[k][i], i>k)
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) A[(size_t)i * n + k] = A[(size_t)k * n + i] / piv;
    __syncthreads();
    // trailing update of the upper triangle: A[r][c] -= L[r][k] L[c][k] for k<r<=c
    long long rem = (long long)(n - k - 1);
    for (long long t = threadIdx.x; t < rem * rem; t += blockDim.x) {
      int r = k + 1 + (int)(t / rem), c = k + 1 + (int)(t % rem);
      if (c < r) continue;
      A[(size_t)r * n + c] -= A[(size_t)r * n + k] * A[(size_t)c * n + k];
    }
    __syncthreads();
  }
}

__global__ void k_chol_solve(int n, const double* __restrict__ L, const double* __restrict__ b, double* x) {
  extern __shared__ double y[];
  for (int i = threadIdx.x; i < n; i += blockDim.x) y[i] = b[i];
  __syncthreads();
  for (int i = 0; i < n; ++i) {  // L y = b
    if (threadIdx.x == 0) y[i] = y[i] / L[(size_t)i * n + i];
    __syncthreads();
    for (int r = i + 1 + threadIdx.x; r < n; r += blockDim.x) y[r] -= L[(size_t)r * n + i] * y[i];
    __syncthreads();
  }
  for (int i = n - 1; i >= 0; --i) {  // L^T x = y
    if (threadIdx.x == 0) y[i] = y[i] / L[(size_t)i * n + i];
    __syncthreads();
    for (int r = threadIdx.x; r < i; r += blockDim.x) y[r] -= L[(size_t)i * n + r] * y[i];
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = y[i];
}

__global__ void k_copy_col(int n, const double* __restrict__ src, double* M, int col) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) M[(size_t)i * n + col] = src[i];
}
__global__ void k_unit(int n, int i, double* e) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) e[t] = (t == i) ? 1.0 : 0.0;
}

int launch_cholesky(int n, double* A, int* d_err, cudaStream_t st) {
  count_launch();
  k_cholesky<<<1, 1024, 0, st>>>(n, A, d_err);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}
int launch_chol_solve(int n, const double* Lf, const double* b, double* x, cudaStream_t st) {
  size_t smem = sizeof(double) * n;
  if (smem > 48 * 1024) {
    IB_CUDA_CHECK(cudaFuncSetAttribute(k_chol_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  count_launch();
  k_chol_solve<<<1, 512, smem, st>>>(n, Lf, b, x);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}
int launch_copy_col(int n, const double* src, double* M, int col, cudaStream_t st) {
  count_launch();
  k_copy_col<<<cdiv(n, 256), 256, 0, st>>>(n, src, M, col);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}
int launch_unit(int n, int i, double* e, cudaStream_t st) {
  count_launch();
  k_unit<<<cdiv(n, 256), 256, 0, st>>>(n, i, e);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

// ---------------------------------------------------------------- fused dense solve
namespace {
struct FusedSmem {
  int nf, R;
  size_t base_doubles() const {
    return (size_t)(R + 1) * nf + 3 * (size_t)nf + (size_t)(R + 1) * R + 5 * (size_t)(R + 1) + 33;
  }
  size_t with_a() const { return base_doubles() + (size_t)nf * nf; }
};
}  // namespace

// One CTA of 32*ceil(nf/32) threads (one vector element per thread), so every scalar FP64
// recurrence and reduction runs on the fewest warps: an FP64 warp instruction occupies its
// SMSP's FP64 pipe for the same time whatever the number of active lanes.  Thread i
// handles element i in every vector loop, as the 512-thread kernels do, and the block sums
// reduce the same per-warp partials in the same order (the extra warps of those kernels add
// zeros), so both solvers produce identical iterates.
__global__ void k_gmres_fused(GmresDev G, const double* __restrict__ Atg, int a_in_smem, const double* __restrict__ b,
                              double* __restrict__ x, double rtol, double atol, int max_it) {
  extern __shared__ double sm[];
  __shared__ int s_reason;
  __shared__ double s_res;
  const int nf = G.nf, R = G.restart;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  double* V = sm;                           // (R+1) x nf
  double* Av = V + (size_t)(R + 1) * nf;    // nf
  double* xs = Av + nf;                     // nf
  double* bs = xs + nf;                     // nf
  double* H = bs + nf;                      // (R+1) x R, column it at H + it*(R+1)
  double* cs = H + (size_t)(R + 1) * R;     // R+1
  double* sn = cs + (R + 1);
  double* g = sn + (R + 1);
  double* h = g + (R + 1);
  double* yv = h + (R + 1);
  double* red = yv + (R + 1);               // 33
  double* As = red + 33;
  const double* At = a_in_smem ? As : Atg;
  if (a_in_smem)
    for (int i = tid; i < nf * nf; i += blockDim.x) As[i] = Atg[i];
  for (int i = tid; i < nf; i += blockDim.x) {
    xs[i] = x[i];
    bs[i] = b[i];
  }
  __syncthreads();

  // out = A in, A column-major, one thread per row (k_dense_mv)
  auto matvec = [&](const double* in, double* out) {
    for (int r = tid; r < nf; r += blockDim.x) {
      double acc = 0.0;
      for (int j = 0; j < nf; ++j) acc = fma(At[(size_t)j * nf + r], in[j], acc);
      out[r] = acc;
    }
    __syncthreads();
  };

  int its = 0, cycles = 0, reason = 0, it = 0;
  double ttol = 0.0;
  for (;;) {
    // cycle start (k_gmres_start): r = b - A x, V0 = r/||r||
    matvec(xs, Av);
    double pr = 0.0, pb = 0.0;
    for (int i = tid; i < nf; i += blockDim.x) {
      double r = bs[i] - Av[i];
      V[i] = r;
      pr += r * r;
      pb += bs[i] * bs[i];
    }
    const double rnorm = sqrt(blk_sum(pr, red));
    const double bnorm = sqrt(blk_sum(pb, red));
    if (its == 0) {
      double rnorm0 = bnorm != 0.0 ? bnorm : rnorm;
      ttol = fmax(rtol * rnorm0, atol);
    }
    const double inv0 = rnorm != 0.0 ? 1.0 / rnorm : 0.0;
    for (int i = tid; i < nf; i += blockDim.x) V[i] = rnorm != 0.0 ? V[i] * inv0 : V[i];
    cycles += 1;
    it = 0;
    reason = 0;
    if (rnorm == 0.0) reason = 2;
    else if (rnorm <= ttol) reason = 3;
    else if (its >= max_it) reason = -3;
    if (tid == 0) {
      g[0] = rnorm;
      s_res = rnorm;
    }
    __syncthreads();
    if (reason != 0) break;
    // Arnoldi steps (k_gmres_arnoldi)
    for (;;) {
      matvec(V + (size_t)it * nf, Av);
      for (int j = warp; j <= it; j += nwarps) {
        const double* vj = V + (size_t)j * nf;
        double p = 0.0;
        for (int i = lane; i < nf; i += 32) p += Av[i] * vj[i];
        for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
        if (lane == 0) h[j] = p;
      }
      __syncthreads();
      double* w = V + (size_t)(it + 1) * nf;
      double pn = 0.0;
      for (int i = tid; i < nf; i += blockDim.x) {
        double v = Av[i];
        for (int j = 0; j <= it; ++j) v = v - h[j] * V[(size_t)j * nf + i];
        w[i] = v;
        pn += v * v;
      }
      const double tt = sqrt(blk_sum(pn, red));
      const double inv = tt != 0.0 ? 1.0 / tt : 0.0;
      for (int i = tid; i < nf; i += blockDim.x) w[i] = tt != 0.0 ? w[i] * inv : w[i];
      if (tid == 0) {
        double* col = H + (size_t)it * (R + 1);
        for (int j = 0; j <= it; ++j) col[j] = h[j];
        col[it + 1] = tt;
        double hapbnd = fabs(tt / g[it]);
        if (hapbnd > 1.0e-30) hapbnd = 1.0e-30;
        bool hapend = tt < hapbnd;
        for (int j = 0; j < it; ++j) {
          double t0 = col[j];
          col[j] = cs[j] * t0 + sn[j] * col[j + 1];
          col[j + 1] = cs[j] * col[j + 1] - sn[j] * t0;
        }
        double res;
        int rsn = 0;
        if (!hapend) {
          double nrm = sqrt(col[it] * col[it] + col[it + 1] * col[it + 1]);
          if (nrm == 0.0) {
            rsn = -9;
            res = s_res;
          } else {
            cs[it] = col[it] / nrm;
            sn[it] = col[it + 1] / nrm;
            g[it + 1] = -(sn[it] * g[it]);
            g[it] = cs[it] * g[it];
            col[it] = cs[it] * col[it] + sn[it] * col[it + 1];
            res = fabs(g[it + 1]);
          }
        } else {
          res = 0.0;
        }
        if (rsn == 0) {
          if (res <= ttol) rsn = 2;
          else if (hapend) rsn = -3;
        }
        s_res = res;
        s_reason = rsn;
      }
      __syncthreads();
      reason = s_reason;
      it += 1;
      its += 1;
      if (reason != 0 || it >= R || its >= max_it) break;
    }
    // KSPGMRESBuildSoln (k_gmres_update): back substitution and x += V y
    if (tid == 0 && it > 0) {
      int k = it - 1;
      auto HH = [&](int r, int c) { return H[(size_t)c * (R + 1) + r]; };
      yv[k] = g[k] / HH(k, k);
      for (int i = k - 1; i >= 0; --i) {
        double tt = g[i];
        for (int j = i + 1; j <= k; ++j) tt = tt - HH(i, j) * yv[j];
        yv[i] = tt / HH(i, i);
      }
    }
    __syncthreads();
    if (it > 0) {
      for (int i = tid; i < nf; i += blockDim.x) {
        double u = 0.0;
        for (int j = 0; j < it; ++j) u = u + yv[j] * V[(size_t)j * nf + i];
        xs[i] = xs[i] + u;
      }
    }
    __syncthreads();
    if (reason != 0 || its >= max_it) break;
  }
  for (int i = tid; i < nf; i += blockDim.x) x[i] = xs[i];
  if (tid == 0) {
    G.ist[0] = its;
    G.ist[1] = reason;
    G.ist[2] = it;
    G.ist[3] = 0;
    G.ist[4] = cycles;
    G.scal[0] = ttol;
    G.scal[1] = s_res;
  }
}

int launch_gmres_fused(const GmresDev& G, const double* At, const double* b, double* x, double rtol, double atol,
                       int max_it, cudaStream_t st) {
  // one element per thread and the same element-to-warp map as the 512-thread kernels
  if (G.nf <= 0 || G.nf > kGmresThreads) return IB_ERR_ARG;
  const int threads = 32 * ((G.nf + 31) / 32);
  FusedSmem fs{G.nf, G.restart};
  int dev = 0, optin = 0;
  IB_CUDA_CHECK(cudaGetDevice(&dev));
  IB_CUDA_CHECK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const size_t limit = (size_t)optin - 1024;   // static shared memory of the kernel and the reductions
  int a_in = 1;
  size_t bytes = 8 * fs.with_a();
  if (bytes > limit) {
    a_in = 0;
    bytes = 8 * fs.base_doubles();
    if (bytes > limit) return IB_ERR_ARG;
  }
  IB_CUDA_CHECK(cudaFuncSetAttribute(k_gmres_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  count_launch();
  k_gmres_fused<<<1, threads, bytes, st>>>(G, At, a_in, b, x, rtol, atol, max_it);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

}  // namespace ib
