// Device GMRES with the semantics of PETSc 3.11 KSPGMRES as the reference
// configures it (variables.F90:565-574): restart 30, classical Gram-Schmidt
// without refinement (borthog2.c), Givens-rotation least squares, nonzero initial
// guess, unpreconditioned residual norm, convergence when the rotated residual
// estimate <= max(rtol*||b||, atol) (KSPConvergedDefault).
//
// Two drivers share one arithmetic.  The graph solver runs one CTA per kernel with the
// operator (the Schur matvec) between them, reading G.xin and writing G.Av.  The cluster
// solver (k_gmres_cluster) runs a whole solve on an assembled dense operator across a
// cluster of kSlices CTAs, each owning one slice of the unknowns.  Every inner product and
// norm is summed the way the cluster must sum it: a sequential partial per slice, then the
// kSlices partials in slice order; and the dense product splits each row into kSlices
// column segments reduced by a fixed shuffle tree.  So both drivers produce identical
// iterates.
#include <cooperative_groups.h>

#include "kernels.cuh"

namespace ib {

namespace cg = cooperative_groups;

constexpr int kGmresThreads = 512;

// [lo, hi) of slice c of n unknowns
__device__ __forceinline__ int slice_size(int n) { return (n + kSlices - 1) / kSlices; }
__device__ __forceinline__ void slice_range(int n, int c, int* lo, int* hi) {
  int ns = slice_size(n);
  *lo = min(n, c * ns);
  *hi = min(n, *lo + ns);
}

// Givens update of Arnoldi step `it` (KSPGMRESUpdateHessenberg): the new Hessenberg column is
// h[0..it], tt; the previous rotations are applied with the rotated value carried in a
// register (one dependent FMA per rotation), then the new rotation, the rotated residual g
// and the convergence reason.  Writes H column `it` (ld = restart+1).
__device__ void givens_step(double* __restrict__ col, const double* __restrict__ h, double tt, int it,
                            double* __restrict__ cs, double* __restrict__ sn, double* __restrict__ g, double prev_res,
                            double ttol, double* res_out, int* reason_out) {
  double hapbnd = fabs(tt / g[it]);
  if (hapbnd > 1.0e-30) hapbnd = 1.0e-30;
  const bool hapend = tt < hapbnd;
  double c = h[0];
  for (int j = 0; j < it; ++j) {
    const double nxt = h[j + 1];
    const double cj = cs[j], sj = sn[j];
    col[j] = fma(sj, nxt, cj * c);
    c = fma(-sj, c, cj * nxt);
  }
  col[it + 1] = tt;
  double res;
  int reason = 0;
  if (!hapend) {
    const double nrm = sqrt(fma(c, c, tt * tt));
    if (nrm == 0.0) {
      reason = -9;  // KSP_DIVERGED_NULL
      res = prev_res;
      col[it] = c;
    } else {
      const double ci = c / nrm, si = tt / nrm;
      cs[it] = ci;
      sn[it] = si;
      g[it + 1] = -(si * g[it]);
      g[it] = ci * g[it];
      col[it] = fma(si, tt, ci * c);
      res = fabs(g[it + 1]);
    }
  } else {
    col[it] = c;
    res = 0.0;
  }
  if (reason == 0) {
    if (res <= ttol) reason = 2;
    else if (hapend) reason = -3;
  }
  *res_out = res;
  *reason_out = reason;
}

// KSPGMRESBuildSoln back substitution: y[0..k] from H (ld = R+1) and g.
__device__ void back_substitute(const double* __restrict__ H, int R, const double* __restrict__ g, int k,
                                double* __restrict__ y) {
  auto HH = [&](int r, int c) { return H[(size_t)c * (R + 1) + r]; };
  y[k] = g[k] / HH(k, k);
  for (int i = k - 1; i >= 0; --i) {
    double tt = g[i];
    for (int j = i + 1; j <= k; ++j) tt = fma(-HH(i, j), y[j], tt);
    y[i] = tt / HH(i, i);
  }
}

__global__ void k_gmres_init(GmresDev G) {
  if (threadIdx.x == 0) {
    G.ist[0] = 0; G.ist[1] = 0; G.ist[2] = 0; G.ist[3] = 0; G.ist[4] = 0;
  }
}

// Cycle start: r = b - A x (A x in G.Av), V0 = r/||r||, tolerance on the first cycle.
__global__ void k_gmres_start(GmresDev G, const double* __restrict__ b, const double* __restrict__ x, double rtol,
                              double atol, int max_it, cudaGraphConditionalHandle h_inner, int use_cond) {
  __shared__ double part[2 * kSlices];
  __shared__ double s_norm[2];
  const int nf = G.nf, tid = threadIdx.x;
  for (int i = tid; i < nf; i += blockDim.x) G.V[i] = b[i] - G.Av[i];
  __syncthreads();
  if (tid < 2 * kSlices) {
    int lo, hi;
    slice_range(nf, tid % kSlices, &lo, &hi);
    const double* v = tid < kSlices ? G.V : b;
    double a = 0.0;
    for (int i = lo; i < hi; ++i) a = fma(v[i], v[i], a);
    part[tid] = a;
  }
  __syncthreads();
  if (tid == 0) {
    double r2 = part[0], b2 = part[kSlices];
    for (int c = 1; c < kSlices; ++c) {
      r2 += part[c];
      b2 += part[kSlices + c];
    }
    s_norm[0] = sqrt(r2);
    s_norm[1] = sqrt(b2);
  }
  __syncthreads();
  const double rnorm = s_norm[0], bnorm = s_norm[1];
  const int its = G.ist[0];
  double ttol;
  if (its == 0) {
    double rnorm0 = bnorm != 0.0 ? bnorm : rnorm;
    ttol = fmax(rtol * rnorm0, atol);
  } else {
    ttol = G.scal[0];
  }
  const double inv = rnorm != 0.0 ? 1.0 / rnorm : 0.0;
  for (int i = tid; i < nf; i += blockDim.x) {
    double v = rnorm != 0.0 ? G.V[i] * inv : G.V[i];
    G.V[i] = v;
    G.xin[i] = v;
  }
  if (tid == 0) {
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
// against the unmodified w), normalisation, Givens update.
__global__ void k_gmres_arnoldi(GmresDev G, int max_it, cudaGraphConditionalHandle h_inner, int use_cond) {
  __shared__ double part[64 * kSlices];
  __shared__ double h[64];
  __shared__ double s_tt;
  if (G.ist[3] == 0) {
    if (use_cond && threadIdx.x == 0) cudaGraphSetConditional(h_inner, 0u);
    return;
  }
  const int nf = G.nf, R = G.restart, tid = threadIdx.x;
  const int it = G.ist[2];
  double* w = G.V + (size_t)(it + 1) * nf;
  const double* Av = G.Av;
  // projections: a partial per (j, slice), then the slices in order
  for (int q = tid; q < (it + 1) * kSlices; q += blockDim.x) {
    const int j = q / kSlices, c = q % kSlices;
    int lo, hi;
    slice_range(nf, c, &lo, &hi);
    const double* vj = G.V + (size_t)j * nf;
    double a = 0.0;
    for (int i = lo; i < hi; ++i) a = fma(Av[i], vj[i], a);
    part[q] = a;
  }
  __syncthreads();
  if (tid <= it) {
    double s = part[tid * kSlices];
    for (int c = 1; c < kSlices; ++c) s += part[tid * kSlices + c];
    h[tid] = s;
  }
  __syncthreads();
  for (int i = tid; i < nf; i += blockDim.x) {
    double v = Av[i];
    for (int j = 0; j <= it; ++j) v = fma(-h[j], G.V[(size_t)j * nf + i], v);
    w[i] = v;
  }
  __syncthreads();
  if (tid < kSlices) {
    int lo, hi;
    slice_range(nf, tid, &lo, &hi);
    double a = 0.0;
    for (int i = lo; i < hi; ++i) a = fma(w[i], w[i], a);
    part[tid] = a;
  }
  __syncthreads();
  if (tid == 0) {
    double s = part[0];
    for (int c = 1; c < kSlices; ++c) s += part[c];
    s_tt = sqrt(s);
  }
  __syncthreads();
  const double tt = s_tt;
  const double inv = tt != 0.0 ? 1.0 / tt : 0.0;
  for (int i = tid; i < nf; i += blockDim.x) {
    double v = tt != 0.0 ? w[i] * inv : w[i];
    w[i] = v;
    G.xin[i] = v;
  }
  if (tid == 0) {
    double* col = G.H + (size_t)it * (R + 1);
    double res;
    int reason;
    givens_step(col, h, tt, it, G.cs, G.sn, G.g, G.scal[1], G.scal[0], &res, &reason);
    const int itn = it + 1;
    const int its = G.ist[0] + 1;
    G.ist[2] = itn;
    G.ist[0] = its;
    G.scal[1] = res;
    G.ist[1] = reason;
    const int active = (reason == 0 && itn < R && its < max_it) ? 1 : 0;
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
  if (threadIdx.x == 0 && it > 0) back_substitute(G.H, R, G.g, it - 1, y);
  __syncthreads();
  if (it > 0) {
    for (int i = threadIdx.x; i < nf; i += blockDim.x) {
      double u = 0.0;
      for (int j = 0; j < it; ++j) u = fma(y[j], G.V[(size_t)j * nf + i], u);
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

// ---------------------------------------------------------------- cluster dense solve
namespace {
// Shared-memory layout of one CTA of the cluster solver (doubles).
struct ClusterSmem {
  int nf, R, ns;
  size_t base() const {
    return (size_t)(R + 1) * ns + nf + 3 * (size_t)ns + 2 * (size_t)(R + 1) + (size_t)(R + 1) * R +
           4 * (size_t)(R + 1) + 8;
  }
  size_t with_a() const { return base() + (size_t)ns * nf; }
};
}  // namespace

// One restarted GMRES solve on the assembled operator A (column-major, At[j*nf + r] = A[r][j])
// across a cluster of kSlices CTAs.  CTA c owns the rows and vector elements of slice c: its
// rows of A, its slice of every Krylov vector, of x and of b.  Per Arnoldi step:
//   A: the product of its rows with the full current vector (kSlices threads per row), and
//      its partial projections; meanwhile the last warp applies the Givens update of the
//      previous step;                                                        cluster barrier
//      the previous step's convergence decision is read from CTA 0 (every CTA branches
//      alike), then the projections are summed over the slices in order;
//   B: w = A v - sum h_j v_j on the slice and its partial norm;              cluster barrier
//   C: the norm, the normalised slice;                                       cluster barrier
//   D: every CTA gathers the full new vector through distributed shared memory.
// No thread waits on a flag: the only waits are the cluster and CTA barriers, which every
// thread of every CTA reaches the same number of times.
__global__ void __cluster_dims__(kSlices, 1, 1)
    k_gmres_cluster(GmresDev G, const double* __restrict__ At, int a_in_smem, const double* __restrict__ b,
                    double* __restrict__ x, double rtol, double atol, int max_it) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int nf = G.nf, R = G.restart;
  const int ns = slice_size(nf);
  int r0, r1;
  slice_range(nf, rank, &r0, &r1);
  const int nl = r1 - r0;
  const int tid = threadIdx.x, lane = tid & 31;
  const int nwork = (int)blockDim.x - 32;     // the last warp applies the Givens updates
  const bool gwarp = tid >= nwork;
  extern __shared__ double sm[];
  double* Vs = sm;                                  // (R+1) x ns
  double* vfull = Vs + (size_t)(R + 1) * ns;        // nf
  double* avs = vfull + nf;                         // ns
  double* xsl = avs + ns;                           // ns
  double* bsl = xsl + ns;                           // ns
  double* hp = bsl + ns;                            // R+1 partial projections (read remotely)
  double* h = hp + (R + 1);                         // R+1
  double* H = h + (R + 1);                          // (R+1) x R
  double* cs = H + (size_t)(R + 1) * R;
  double* sn = cs + (R + 1);
  double* g = sn + (R + 1);
  double* yv = g + (R + 1);
  double* scal = yv + (R + 1);                      // [0],[1] partials (read remotely), [2] tt, [3] res,
                                                    // [4] 1/tt, [5] rnorm, [6] bnorm, [7] ttol
  double* As = scal + 8;                            // nl x nf row-major when a_in_smem
  __shared__ int s_reason;                          // read remotely from CTA 0
  auto remote = [&](double* p, int c) -> const double* { return cl.map_shared_rank(p, c); };
  auto bar_work = [&]() { asm volatile("bar.sync 1, %0;" ::"r"(nwork)); };

  if (a_in_smem)
    for (int q = tid; q < nl * nf; q += blockDim.x) {
      const int rl = q / nf, j = q - rl * nf;
      As[q] = At[(size_t)j * nf + r0 + rl];
    }
  for (int i = tid; i < nl; i += blockDim.x) {
    xsl[i] = x[r0 + i];
    bsl[i] = b[r0 + i];
  }
  __syncthreads();

  // avs = rows of A times vfull: kSlices column segments per row, reduced by a fixed tree
  const int cw = slice_size(nf);
  auto matvec = [&]() {
    for (int base = 0; base < ns * kSlices; base += nwork) {
      const int q = base + tid, rl = q / kSlices, seg = q % kSlices;
      double p = 0.0;
      if (rl < nl) {
        const int j0 = min(nf, seg * cw), j1 = min(nf, j0 + cw);
        if (a_in_smem) {
          const double* Ar = As + (size_t)rl * nf;
          for (int j = j0; j < j1; ++j) p = fma(Ar[j], vfull[j], p);
        } else {
          for (int j = j0; j < j1; ++j) p = fma(At[(size_t)j * nf + r0 + rl], vfull[j], p);
        }
      }
      p += __shfl_xor_sync(0xffffffffu, p, 4);
      p += __shfl_xor_sync(0xffffffffu, p, 2);
      p += __shfl_xor_sync(0xffffffffu, p, 1);
      if (rl < nl && seg == 0) avs[rl] = p;
    }
  };
  auto gather = [&](double* src, int stride_slot) {   // vfull[i] = slot of the owner's slice
    for (int i = tid; i < nf; i += blockDim.x) {
      const int c = i / ns;
      vfull[i] = remote(src + (size_t)stride_slot * ns, c)[i - c * ns];
    }
  };

  int its = 0, cycles = 0, reason = 0, k = 0;
  double ttol = 0.0;
  for (;;) {
    // ---- cycle start (k_gmres_start): r = b - A x, V0 = r/||r||
    cl.sync();                                    // every x slice is final
    for (int i = tid; i < nf; i += blockDim.x) {
      const int c = i / ns;
      vfull[i] = remote(xsl, c)[i - c * ns];
    }
    __syncthreads();
    if (!gwarp) matvec();
    __syncthreads();
    for (int i = tid; i < nl; i += blockDim.x) Vs[i] = bsl[i] - avs[i];
    __syncthreads();
    if (tid == 0) {
      double a = 0.0, bb = 0.0;
      for (int i = 0; i < nl; ++i) a = fma(Vs[i], Vs[i], a);
      for (int i = 0; i < nl; ++i) bb = fma(bsl[i], bsl[i], bb);
      scal[0] = a;
      scal[1] = bb;
    }
    cl.sync();
    if (tid == 0) {
      double r2 = remote(scal, 0)[0], b2 = remote(scal, 0)[1];
      for (int c = 1; c < kSlices; ++c) {
        r2 += remote(scal, c)[0];
        b2 += remote(scal, c)[1];
      }
      const double rnorm = sqrt(r2), bnorm = sqrt(b2);
      if (its == 0) {
        double rnorm0 = bnorm != 0.0 ? bnorm : rnorm;
        scal[7] = fmax(rtol * rnorm0, atol);
      }
      scal[5] = rnorm;
      scal[6] = bnorm;
      scal[3] = rnorm;
      g[0] = rnorm;
      int rs = 0;
      if (rnorm == 0.0) rs = 2;
      else if (rnorm <= scal[7]) rs = 3;
      else if (its >= max_it) rs = -3;
      s_reason = rs;
    }
    __syncthreads();
    {
      const double rnorm = scal[5];
      const double inv = rnorm != 0.0 ? 1.0 / rnorm : 0.0;
      for (int i = tid; i < nl; i += blockDim.x) Vs[i] = rnorm != 0.0 ? Vs[i] * inv : Vs[i];
    }
    cycles += 1;
    cl.sync();                                    // V0 slices and CTA 0's decision are visible
    reason = *cl.map_shared_rank(&s_reason, 0);
    ttol = scal[7];
    if (reason != 0) break;
    gather(Vs, 0);
    __syncthreads();
    // ---- Arnoldi steps (k_gmres_arnoldi), the Givens update of step k-1 during step k
    k = 0;
    for (;;) {
      if (!gwarp) {
        matvec();
        bar_work();
        if (tid <= k) {
          double a = 0.0;
          const double* vj = Vs + (size_t)tid * ns;
          for (int i = 0; i < nl; ++i) a = fma(avs[i], vj[i], a);
          hp[tid] = a;
        }
      } else if (k > 0 && lane == 0) {
        double res;
        int rs;
        givens_step(H + (size_t)(k - 1) * (R + 1), h, scal[2], k - 1, cs, sn, g, scal[3], ttol, &res, &rs);
        scal[3] = res;
        s_reason = rs;
      }
      cl.sync();                                  // partial projections; Givens of step k-1
      if (k > 0) {
        reason = *cl.map_shared_rank(&s_reason, 0);
        if (reason != 0 || k >= R || its >= max_it) break;
      }
      if (tid <= k) {
        double s = remote(hp, 0)[tid];
        for (int c = 1; c < kSlices; ++c) s += remote(hp, c)[tid];
        h[tid] = s;
      }
      __syncthreads();
      double* w = Vs + (size_t)(k + 1) * ns;
      for (int i = tid; i < nl; i += blockDim.x) {
        double v = avs[i];
        for (int j = 0; j <= k; ++j) v = fma(-h[j], Vs[(size_t)j * ns + i], v);
        w[i] = v;
      }
      __syncthreads();
      if (tid == 0) {
        double a = 0.0;
        for (int i = 0; i < nl; ++i) a = fma(w[i], w[i], a);
        scal[0] = a;
      }
      cl.sync();                                  // partial norms
      if (tid == 0) {
        double s = remote(scal, 0)[0];
        for (int c = 1; c < kSlices; ++c) s += remote(scal, c)[0];
        const double tt = sqrt(s);
        scal[2] = tt;
        scal[4] = tt != 0.0 ? 1.0 / tt : 0.0;
      }
      __syncthreads();
      {
        const double tt = scal[2], inv = scal[4];
        for (int i = tid; i < nl; i += blockDim.x) w[i] = tt != 0.0 ? w[i] * inv : w[i];
      }
      cl.sync();                                  // the new vector's slices
      gather(Vs, k + 1);
      __syncthreads();
      its += 1;
      k += 1;
    }
    // ---- KSPGMRESBuildSoln (k_gmres_update): back substitution and x += V y on the slice
    if (tid == 0 && k > 0) back_substitute(H, R, g, k - 1, yv);
    __syncthreads();
    if (k > 0)
      for (int i = tid; i < nl; i += blockDim.x) {
        double u = 0.0;
        for (int j = 0; j < k; ++j) u = fma(yv[j], Vs[(size_t)j * ns + i], u);
        xsl[i] = xsl[i] + u;
      }
    __syncthreads();
    if (reason != 0 || its >= max_it) break;
  }
  for (int i = tid; i < nl; i += blockDim.x) x[r0 + i] = xsl[i];
  if (rank == 0 && tid == 0) {
    G.ist[0] = its;
    G.ist[1] = reason;
    G.ist[2] = k;
    G.ist[3] = 0;
    G.ist[4] = cycles;
    G.scal[0] = ttol;
    G.scal[1] = scal[3];
  }
  cl.sync();                                      // no CTA exits while others read its memory
}

int launch_gmres_fused(const GmresDev& G, FusedPlan* plan, const double* At, const double* b, double* x, double rtol,
                       double atol, int max_it, cudaStream_t st) {
  if (plan->state < 0) {
    plan->state = 0;
    if (G.nf <= 0 || G.restart > 63) return IB_ERR_ARG;
    ClusterSmem cs{G.nf, G.restart, (G.nf + kSlices - 1) / kSlices};
    // at least R+1 work threads: one per projection of the longest Arnoldi step
    const int work = max(64, 32 * ((cs.ns * kSlices + 31) / 32));
    const int threads = work + 32;
    if (threads > 1024) return IB_ERR_ARG;
    int dev = 0, optin = 0;
    IB_CUDA_CHECK(cudaGetDevice(&dev));
    IB_CUDA_CHECK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const size_t limit = (size_t)optin - 1024;
    int a_in = 1;
    size_t bytes = 8 * cs.with_a();
    if (bytes > limit) {
      a_in = 0;
      bytes = 8 * cs.base();
      if (bytes > limit) return IB_ERR_ARG;
    }
    IB_CUDA_CHECK(cudaFuncSetAttribute(k_gmres_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    // the cluster must fit on the device as launched
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kSlices);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = bytes;
    cfg.stream = st;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, k_gmres_cluster, &cfg) != cudaSuccess || nclusters < 1) {
      cudaGetLastError();
      return IB_ERR_ARG;
    }
    plan->threads = threads;
    plan->a_in = a_in;
    plan->bytes = bytes;
    plan->state = 1;
  }
  if (plan->state != 1) return IB_ERR_ARG;
  count_launch();
  k_gmres_cluster<<<kSlices, plan->threads, plan->bytes, st>>>(G, At, plan->a_in, b, x, rtol, atol, max_it);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

}  // namespace ib
