// Device GMRES with the semantics of PETSc 3.11 KSPGMRES as the reference
// configures it (variables.F90:565-574): restart 30, classical Gram-Schmidt
// without refinement (borthog2.c), Givens-rotation least squares, nonzero initial
// guess, unpreconditioned residual norm, convergence when the rotated residual
// estimate <= max(rtol*||b||, atol) (KSPConvergedDefault).
//
// Two drivers share one arithmetic.  The graph solver runs one CTA per kernel with the
// operator (the Schur matvec) between them, reading G.xin and writing G.Av.  The cluster
// solver (k_gmres_cluster) runs a whole solve on an assembled dense operator across a
// cluster of kSlices CTAs, each owning one slice of the unknowns.  Every inner product,
// norm and Gram-Schmidt update is summed in the fixed order kernels.cuh states, which the
// graph kernels evaluate with one thread per sum and the cluster with lanes and shuffle
// trees; so both drivers produce identical iterates.
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

static_assert(kSlices == 8, "the pairwise trees below are written for 8 slices");

// The fixed summation orders, one thread per sum (the cluster solver's lane forms match).
__device__ __forceinline__ double slice_dot_seq(const double* __restrict__ a, const double* __restrict__ b, int lo,
                                                int hi) {
  const int n = hi - lo, LP = slice_blocks_p2(n);
  // the pairwise tree over the LP block sums, streamed: merge equal-sized subtrees
  double st[32];
  int sz[32], top = 0;
  for (int k = 0; k < LP; ++k) {
    double p[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int i = lo + 4 * k + t;
      p[t] = i < hi ? a[i] * b[i] : 0.0;
    }
    double v = (p[0] + p[1]) + (p[2] + p[3]);
    int w = 1;
    while (top > 0 && sz[top - 1] == w) {
      v = st[top - 1] + v;
      w *= 2;
      --top;
    }
    st[top] = v;
    sz[top] = w;
    ++top;
  }
  return st[0];
}
__device__ __forceinline__ double tree8_seq(const double* p) {
  return ((p[0] + p[1]) + (p[2] + p[3])) + ((p[4] + p[5]) + (p[6] + p[7]));
}
// Row i of w = Av - sum_{j<=it} h_j V_j (V with row pitch ld).
__device__ __forceinline__ double cgs_row_seq(double av, const double* __restrict__ h, const double* __restrict__ V,
                                              size_t ld, int i, int it) {
  double p[8];
#pragma unroll
  for (int g = 0; g < 8; ++g) {
    double t = g == 0 ? av : 0.0;
    for (int j = g; j <= it; j += 8) t = fma(-h[j], V[(size_t)j * ld + i], t);
    p[g] = t;
  }
  return tree8_seq(p);
}

// Happy breakdown (KSPGMRESUpdateHessenberg): tt < min(|tt/g|, haptol = 1e-30).  The bound
// never exceeds haptol, so the quotient is formed only when tt itself is below it.
__device__ __forceinline__ bool happy_breakdown(double tt, double g) {
  if (!(tt < 1.0e-30)) return false;
  double hapbnd = fabs(tt / g);
  if (hapbnd > 1.0e-30) hapbnd = 1.0e-30;
  return tt < hapbnd;
}

// Norm of a new Krylov vector from its squared norm s: tt and the scale 1/tt applied to it
// (rsqrt and a product: a square root and a division cost about 600 cycles each here).
__device__ __forceinline__ void norm_and_scale(double s, double* tt, double* inv) {
  if (s > 0.0) {
    const double r = rsqrt(s);
    *inv = r;
    *tt = s * r;
  } else {
    *tt = sqrt(s);
    *inv = 0.0;
  }
}

// Givens update of Arnoldi step `it` (KSPGMRESUpdateHessenberg): the new Hessenberg column is
// h[0..it], tt; the previous rotations are applied with the rotated value carried in a
// register (one dependent FMA per rotation), then the new rotation (from rsqrt of c^2+tt^2),
// the rotated residual g and the convergence reason.  Writes H column `it` (ld = restart+1).
__device__ void givens_step(double* __restrict__ col, const double* __restrict__ h, double tt, int it,
                            double* __restrict__ cs, double* __restrict__ sn, double* __restrict__ g, double prev_res,
                            double ttol, double* res_out, int* reason_out) {
  const bool hapend = happy_breakdown(tt, g[it]);
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
    const double r2 = fma(c, c, tt * tt);
    if (r2 == 0.0) {
      reason = -9;  // KSP_DIVERGED_NULL
      res = prev_res;
      col[it] = c;
    } else {
      const double rn = rsqrt(r2);
      const double ci = c * rn, si = tt * rn;
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

// KSPGMRESBuildSoln back substitution y[0..k] = R^-1 g (R the rotated Hessenberg, ld = R+1), on
// one whole warp: the pivot reciprocals at once, then a column sweep (y_j = r_j / R_jj as
// r_j * (1/R_jj); every r_l, l < j, loses R_lj y_j on its own lane).  rc: k+1 doubles.
__device__ void back_substitute(const double* __restrict__ H, int R, const double* __restrict__ g, int k,
                                double* __restrict__ y, double* __restrict__ rc) {
  const int lane = threadIdx.x & 31;
  auto HH = [&](int r, int c) { return H[(size_t)c * (R + 1) + r]; };
  for (int l = lane; l <= k; l += 32) {
    y[l] = g[l];
    rc[l] = __drcp_rn(HH(l, l));
  }
  __syncwarp();
  for (int j = k; j >= 0; --j) {
    const double yj = y[j] * rc[j];
    __syncwarp();
    for (int l = lane; l < j; l += 32) y[l] = fma(-HH(l, j), yj, y[l]);
    if (lane == 0) y[j] = yj;
    __syncwarp();
  }
}

__global__ void k_gmres_init(GmresDev G) {
  IB_GRID_DEP_WAIT();
  if (threadIdx.x == 0) {
    G.ist[0] = 0; G.ist[1] = 0; G.ist[2] = 0; G.ist[3] = 0; G.ist[4] = 0;
  }
}

// Cycle start: r = b - A x (A x in G.Av), V0 = r/||r||, tolerance on the first cycle.
__global__ void k_gmres_start(GmresDev G, const double* __restrict__ b, const double* __restrict__ x, double rtol,
                              double atol, int max_it, cudaGraphConditionalHandle h_inner, int use_cond) {
  IB_GRID_DEP_WAIT();
  __shared__ double part[2 * kSlices];
  __shared__ double s_norm[2];
  const int nf = G.nf, tid = threadIdx.x;
  for (int i = tid; i < nf; i += blockDim.x) G.V[i] = b[i] - G.Av[i];
  __syncthreads();
  if (tid < 2 * kSlices) {
    int lo, hi;
    slice_range(nf, tid % kSlices, &lo, &hi);
    const double* v = tid < kSlices ? G.V : b;
    part[tid] = slice_dot_seq(v, v, lo, hi);
  }
  __syncthreads();
  if (tid == 0) {
    s_norm[0] = sqrt(tree8_seq(part));
    s_norm[1] = sqrt(tree8_seq(part + kSlices));
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
  IB_GRID_DEP_WAIT();
  __shared__ double part[64 * kSlices];
  __shared__ double h[64];
  __shared__ double s_tt[2];
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
    part[q] = slice_dot_seq(Av, G.V + (size_t)j * nf, lo, hi);
  }
  __syncthreads();
  if (tid <= it) h[tid] = tree8_seq(part + tid * kSlices);
  __syncthreads();
  for (int i = tid; i < nf; i += blockDim.x) w[i] = cgs_row_seq(Av[i], h, G.V, nf, i, it);
  __syncthreads();
  if (tid < kSlices) {
    int lo, hi;
    slice_range(nf, tid, &lo, &hi);
    part[tid] = slice_dot_seq(w, w, lo, hi);
  }
  __syncthreads();
  if (tid == 0) norm_and_scale(tree8_seq(part), &s_tt[0], &s_tt[1]);
  __syncthreads();
  const double tt = s_tt[0];
  const double inv = s_tt[1];
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
  IB_GRID_DEP_WAIT();
  __shared__ double y[64], rc[64];
  const int nf = G.nf, R = G.restart;
  const int it = G.ist[2];
  if (threadIdx.x < 32 && it > 0) back_substitute(G.H, R, G.g, it - 1, y, rc);
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
    // the iteration cap reached inside a cycle ends the solve as KSP_DIVERGED_ITS
    if (G.ist[1] == 0 && G.ist[0] >= max_it) G.ist[1] = -3;
    if (use_cond) cudaGraphSetConditional(h_outer, G.ist[1] == 0 ? 1u : 0u);
  }
}

__global__ void k_copy(int n, const double* __restrict__ a, double* __restrict__ b) {
  IB_GRID_DEP_WAIT();
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
  IB_GRID_DEP_WAIT();
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

// L L^T x = b with the Cholesky factor L (row-major, lower): forward then backward substitution
// in blocks of 32 unknowns.  Each block first subtracts what the solved unknowns contribute (one
// warp per unknown, lanes across the solved ones, a fixed shuffle tree), then warp 0 solves the
// block's 32 x 32 triangle, staged in shared memory, with shuffles; no block-wide barrier inside
// the triangles.
__global__ void k_chol_solve(int n, const double* __restrict__ L, const double* __restrict__ b, double* x) {
  IB_GRID_DEP_WAIT();
  extern __shared__ double y[];   // n unknowns, then the diagonal block (32 x 33)
  double* dg = y + n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = threadIdx.x; i < n; i += blockDim.x) y[i] = b[i];
  __syncthreads();
  auto warp_sum = [](double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
  };
  for (int b0 = 0; b0 < n; b0 += 32) {   // L y = b
    const int nb = min(32, n - b0);
    for (int r = b0 + warp; r < b0 + nb; r += nw) {
      double acc = 0.0;
      for (int c = lane; c < b0; c += 32) acc = fma(L[(size_t)r * n + c], y[c], acc);
      acc = warp_sum(acc);
      if (lane == 0) y[r] -= acc;
    }
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) dg[(t / nb) * 33 + t % nb] = L[(size_t)(b0 + t / nb) * n + b0 + t % nb];
    __syncthreads();
    if (warp == 0) {
      double yr = lane < nb ? y[b0 + lane] : 0.0;
      for (int i = 0; i < nb; ++i) {
        if (lane == i) yr = yr / dg[i * 33 + i];
        const double yi = __shfl_sync(0xffffffffu, yr, i);
        if (lane > i && lane < nb) yr -= dg[lane * 33 + i] * yi;
      }
      if (lane < nb) y[b0 + lane] = yr;
    }
    __syncthreads();
  }
  for (int b1 = n; b1 > 0; b1 -= 32) {   // L^T x = y
    const int b0 = max(0, b1 - 32), nb = b1 - b0;
    for (int c = b0 + warp; c < b1; c += nw) {
      double acc = 0.0;
      for (int r = b1 + lane; r < n; r += 32) acc = fma(L[(size_t)r * n + c], y[r], acc);
      acc = warp_sum(acc);
      if (lane == 0) y[c] -= acc;
    }
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) dg[(t / nb) * 33 + t % nb] = L[(size_t)(b0 + t / nb) * n + b0 + t % nb];
    __syncthreads();
    if (warp == 0) {
      double yr = lane < nb ? y[b0 + lane] : 0.0;
      for (int i = nb - 1; i >= 0; --i) {
        if (lane == i) yr = yr / dg[i * 33 + i];
        const double xi = __shfl_sync(0xffffffffu, yr, i);
        if (lane < i) yr -= dg[i * 33 + lane] * xi;
      }
      if (lane < nb) y[b0 + lane] = yr;
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = y[i];
}

__global__ void k_copy_col(int n, const double* __restrict__ src, double* M, int col) {
  IB_GRID_DEP_WAIT();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) M[(size_t)i * n + col] = src[i];
}
__global__ void k_unit(int n, int i, double* e) {
  IB_GRID_DEP_WAIT();
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
  size_t smem = sizeof(double) * ((size_t)n + 32 * 33);
  IB_CUDA_CHECK(allow_dyn_smem(k_chol_solve, smem));
  count_launch();
  k_chol_solve<<<1, 1024, smem, st>>>(n, Lf, b, x);
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
    return (size_t)(R + 1) * ns + nf + 4 * (size_t)ns + 2 * (size_t)(R + 1) + (size_t)(R + 1) * R +
           4 * (size_t)(R + 1) + 8 + 2 * (size_t)R + 32;
  }
  size_t with_a() const { return base() + (size_t)ns * nf; }
};
}  // namespace

// Warps 0-2 run the dense product and the projections; warp 3 the Givens update meanwhile;
// all four the rest.  Each warp sits on its own SM sub-partition, and an FP64 instruction
// holds its sub-partition's FP64 pipe for the same time whatever its active lanes, so every
// sum below is spread over lanes (shuffle trees) rather than run down one thread.
constexpr int kClusterThreads = 128;
constexpr int kProdThreads = 96;

// givens_step's arithmetic on one whole warp (it < 32): lane j holds rotation j and the
// product cs[j]*h[j+1] in registers, the chain of rotated values runs on every lane in step
// (each step's operands by shuffle, so nothing waits on shared memory), lane j keeps the value
// before rotation j and forms column entry j.
__device__ void givens_step_warp(double* __restrict__ col, const double* __restrict__ h, double tt, int it,
                                 double* __restrict__ cs, double* __restrict__ sn, double* __restrict__ g,
                                 double prev_res, double ttol, double* res_out, int* reason_out) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const bool mine = lane < it;
  const double csj = mine ? cs[lane] : 0.0, snj = mine ? sn[lane] : 0.0;
  const double hj1 = mine ? h[lane + 1] : 0.0;
  const double pj = csj * hj1;
  const double gi = g[it];   // read by every lane before lane 0 rewrites it
  double c = h[0], cmine = 0.0;
#pragma unroll 8
  for (int j = 0; j < it; ++j) {
    const double sj = __shfl_sync(full, snj, j), pp = __shfl_sync(full, pj, j);
    if (lane == j) cmine = c;
    c = fma(-sj, c, pp);
  }
  if (mine) col[lane] = fma(snj, hj1, csj * cmine);
  const bool hapend = happy_breakdown(tt, gi);
  const double r2 = fma(c, c, tt * tt);
  const double rn = r2 != 0.0 ? rsqrt(r2) : 0.0;
  const double ci = c * rn, si = tt * rn;
  if (lane == 0) {
    col[it + 1] = tt;
    double res;
    int reason = 0;
    if (!hapend) {
      if (r2 == 0.0) {
        reason = -9;  // KSP_DIVERGED_NULL
        res = prev_res;
        col[it] = c;
      } else {
        cs[it] = ci;
        sn[it] = si;
        g[it + 1] = -(si * gi);
        g[it] = ci * gi;
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
  __syncwarp();
}

// One restarted GMRES solve on the assembled operator A (column-major, At[j*nf + r] = A[r][j])
// across a cluster of kSlices CTAs.  CTA c owns the rows and vector elements of slice c: its
// rows of A, its slice of every Krylov vector, of x and of b.  Per Arnoldi step:
//   A: warps 0-2 form the product of its rows with the full current vector (rows in groups of
//      S lanes) and its partial projections; meanwhile warp 3 applies the Givens update of
//      the previous step;                                                    cluster barrier
//      the previous step's convergence decision is read from CTA 0 (every CTA branches
//      alike), then the projections are summed over the slices (8 lanes per projection);
//   B: w = A v - sum h_j v_j on the slice (8 lanes per row) and its partial norm, the
//      unscaled slice kept for the others to read;                           cluster barrier
//   C: every CTA gathers the unscaled slices while forming the norm, then scales its gathered
//      copy and its own slice by 1/norm.
// No thread waits on a flag: the only waits are the cluster and CTA barriers, which every
// thread of every CTA reaches the same number of times.
__global__ void __cluster_dims__(kSlices, 1, 1) __launch_bounds__(kClusterThreads)
    k_gmres_cluster(GmresDev G, const double* __restrict__ At, int a_in_smem, const double* __restrict__ b,
                    double* __restrict__ x, double rtol, double atol, int max_it) {
  IB_GRID_DEP_WAIT();
  const unsigned full = 0xffffffffu;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int nf = G.nf, R = G.restart;
  const int ns = slice_size(nf);
  int r0, r1;
  slice_range(nf, rank, &r0, &r1);
  const int nl = r1 - r0;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
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
  double* gbuf = scal + 8;                          // 2R: Givens scratch
  double* wbuf = gbuf + 2 * (size_t)R;              // ns: the new vector before scaling (read remotely)
  double* nblk = wbuf + ns;                         // 32: block partials of its norm
  double* As = nblk + 32;                           // nl x nf row-major when a_in_smem
  __shared__ int s_reason;                          // read remotely from CTA 0
  auto remote = [&](double* p, int c) -> const double* { return cl.map_shared_rank(p, c); };
  auto bar_prod = [&]() { asm volatile("bar.sync 1, %0;" ::"r"(kProdThreads)); };
  // slice partial of a.b in the fixed order: lane blk of an aligned group of LP lanes forms
  // block blk ((p0+p1)+(p2+p3) over rows 4blk..4blk+3), the group's xor tree the rest (valid
  // on every lane of the group); every lane of the warp calls it
  const int LP = slice_blocks_p2(nl);
  auto slice_dot_lanes = [&](const double* a, const double* bb, int blk, bool on) -> double {
    double p[4] = {0.0, 0.0, 0.0, 0.0};
    if (on)
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int i = 4 * blk + t;
        if (i < nl) p[t] = a[i] * bb[i];
      }
    double v = (p[0] + p[1]) + (p[2] + p[3]);
    for (int off = 1; off < LP; off <<= 1) v += __shfl_xor_sync(full, v, off);
    return v;
  };
  // pairwise tree over an aligned group of 8 lanes (valid on all 8)
  auto tree8 = [&](double p) -> double {
    p += __shfl_xor_sync(full, p, 1);
    p += __shfl_xor_sync(full, p, 2);
    p += __shfl_xor_sync(full, p, 4);
    return p;
  };

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

  // avs = rows of A times vfull (warps 0-2): rows in groups of S lanes, one column segment
  // per lane, joined by seg_tree (k_dense_mv's layout and order)
  const int S = mv_segments(nf), gpw = 32 / S, cw = (nf + S - 1) / S;
  const int grp = lane / S, seg = lane - grp * S;
  // When the slice's rows take one pass of the three warps and a segment fits, each lane keeps
  // its segment of its row in registers for the whole solve (the same two chains, same order)
  constexpr int kRegSeg = 20;
  const bool a_in_regs = nl <= 3 * gpw && cw <= kRegSeg;
  const int rl_r = warp * gpw + grp;
  const bool live_r = warp < 3 && grp < gpw && rl_r < nl;
  const int j0_r = min(nf, seg * cw), len_r = live_r ? min(nf, j0_r + cw) - j0_r : 0;
  double areg[kRegSeg];
  auto matvec = [&]() {
    if (a_in_regs) {
      double p = 0.0;
      if (live_r) {
        double e = 0.0, o = 0.0;
        const double* v = vfull + j0_r;
#pragma unroll
        for (int t = 0; t < kRegSeg; t += 2) {
          if (t + 1 < len_r) {
            e = fma(areg[t], v[t], e);
            o = fma(areg[t + 1], v[t + 1], o);
          } else if (t < len_r) {
            e = fma(areg[t], v[t], e);
          }
        }
        p = e + o;
      }
      p = seg_tree(p, seg, S);
      if (live_r && seg == 0) avs[rl_r] = p;
      return;
    }
    for (int rb = 0; rb < nl; rb += 3 * gpw) {
      const int rl = rb + warp * gpw + grp;
      const bool live = grp < gpw && rl < nl;
      double p = 0.0;
      if (live) {
        const int j0 = min(nf, seg * cw), j1 = min(nf, j0 + cw);
        if (a_in_smem) {
          const double* Ar = As + (size_t)rl * nf;
              p = seg_dot(j0, j1, [&](int j, double acc) { return fma(Ar[j], vfull[j], acc); });
        } else {
          p = seg_dot(j0, j1, [&](int j, double acc) { return fma(At[(size_t)j * nf + r0 + rl], vfull[j], acc); });
        }
      }
      p = seg_tree(p, seg, S);
      if (live && seg == 0) avs[rl] = p;
    }
  };
  auto gather = [&](double* src, int stride_slot) {   // vfull[i] = slot of the owner's slice
    for (int i = tid; i < nf; i += blockDim.x) {
      const int c = i / ns;
      vfull[i] = remote(src + (size_t)stride_slot * ns, c)[i - c * ns];
    }
  };

  if (a_in_regs) {
#pragma unroll
    for (int t = 0; t < kRegSeg; ++t) {
      const int j = j0_r + t;
      areg[t] = 0.0;
      if (t < len_r) areg[t] = a_in_smem ? As[(size_t)rl_r * nf + j] : At[(size_t)j * nf + r0 + rl_r];
    }
  }
  int its = 0, cycles = 0, reason = 0, k = 0;
  double ttol = 0.0;
  for (;;) {
    // ---- cycle start (k_gmres_start): r = b - A x, V0 = r/||r||
    cl.sync();                                    // every x slice is final
    gather(xsl, 0);
    __syncthreads();
    if (warp < 3) matvec();
    __syncthreads();
    for (int i = tid; i < nl; i += blockDim.x) Vs[i] = bsl[i] - avs[i];
    __syncthreads();
    if (warp == 0) {   // lanes 0-15: ||r||^2 partial, lanes 16-31: ||b||^2 partial
      const double* v = lane < 16 ? Vs : bsl;
      const double t = slice_dot_lanes(v, v, lane & 15, (lane & 15) < LP);
      if (lane == 0) scal[0] = t;
      if (lane == 16) scal[1] = t;
    }
    cl.sync();
    if (warp == 0) {   // lanes 0-7: the slices' r partials, lanes 8-15: their b partials
      const double p = tree8(lane < 16 ? remote(scal, lane & 7)[lane >> 3] : 0.0);
      const double nrm = sqrt(p);
      const double rnorm = __shfl_sync(full, nrm, 0), bnorm = __shfl_sync(full, nrm, 8);
      if (lane == 0) {
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
      if (warp < 3) {
        matvec();
        bar_prod();
        for (int q0 = 0; q0 < LP * (k + 1); q0 += kProdThreads) {   // LP lanes per projection
          const int q = q0 + tid, j = q / LP, blk = q - j * LP;
          const bool on = j <= k;
          const double t = slice_dot_lanes(avs, Vs + (size_t)(on ? j : 0) * ns, blk, on);
          if (on && blk == 0) hp[j] = t;
        }
      } else if (k > 0) {
        double res = 0.0;
        int rs = 0;
        givens_step_warp(H + (size_t)(k - 1) * (R + 1), h, scal[2], k - 1, cs, sn, g, scal[3], ttol, &res, &rs);
        if (lane == 0) {
          scal[3] = res;
          s_reason = rs;
        }
      }
      cl.sync();                                  // partial projections; Givens of step k-1
      {
        // the first pass's slice partials are loaded together with CTA 0's decision
        const int j = tid >> 3;
        double p = j <= k ? remote(hp, tid & 7)[j] : 0.0;
        if (k > 0) {
          reason = *cl.map_shared_rank(&s_reason, 0);
          if (reason != 0 || k >= R || its >= max_it) break;
        }
        p = tree8(p);
        if (j <= k && (tid & 7) == 0) h[j] = p;
        for (int q0 = kClusterThreads; q0 < 8 * (k + 1); q0 += kClusterThreads) {   // 8 lanes (slices) per j
          const int q = q0 + tid, jj = q >> 3;
          const double pp = tree8(jj <= k ? remote(hp, q & 7)[jj] : 0.0);
          if (jj <= k && (q & 7) == 0) h[jj] = pp;
        }
      }
      __syncthreads();
      // w = avs - sum_j h_j V_j on the slice (8 lanes, one chain each, per row) into wbuf; the
      // lanes 0, 8, 16, 24 of a warp hold 4 consecutive rows: one block of the norm partial
      const int npass = (8 * nl + kClusterThreads - 1) / kClusterThreads;
      for (int q0 = 0; q0 < 8 * nl; q0 += kClusterThreads) {
        const int q = q0 + tid, i = q >> 3, gq = q & 7;
        double p = 0.0;
        if (i < nl) {
          p = gq == 0 ? avs[i] : 0.0;
          for (int j = gq; j <= k; j += 8) p = fma(-h[j], Vs[(size_t)j * ns + i], p);
        }
        p = tree8(p);
        if (i < nl && gq == 0) wbuf[i] = p;
        double sq = i < nl ? p * p : 0.0;
        sq += __shfl_xor_sync(full, sq, 8);
        sq += __shfl_xor_sync(full, sq, 16);
        if (lane == 0) nblk[q >> 5] = sq;
      }
      __syncthreads();
      if (warp == 0) {
        double v = lane < LP && lane < 4 * npass ? nblk[lane] : 0.0;
        for (int off = 1; off < LP; off <<= 1) v += __shfl_xor_sync(full, v, off);
        if (lane == 0) scal[0] = v;
      }
      cl.sync();                                  // partial norms and the unscaled slices
      // the new vector: every CTA gathers the unscaled slices while warp 0 forms the norm,
      // then scales its gathered copy and its own slice alike (the products of a normalise-
      // then-gather, with one cluster barrier fewer)
      {
        const double pn = (warp == 0 && lane < 8) ? remote(scal, lane)[0] : 0.0;
        for (int i = tid; i < nf; i += blockDim.x) {
          const int c = i / ns;
          vfull[i] = remote(wbuf, c)[i - c * ns];
        }
        if (warp == 0) {
          const double sq = tree8(pn);
          if (lane == 0) {
            double tt, inv;
            norm_and_scale(sq, &tt, &inv);
            scal[2] = tt;
            scal[4] = inv;
          }
        }
      }
      __syncthreads();
      {
        const double tt = scal[2], inv = scal[4];
        double* w = Vs + (size_t)(k + 1) * ns;
        for (int i = tid; i < nl; i += blockDim.x) w[i] = tt != 0.0 ? wbuf[i] * inv : wbuf[i];
        for (int i = tid; i < nf; i += blockDim.x) vfull[i] = tt != 0.0 ? vfull[i] * inv : vfull[i];
      }
      __syncthreads();
      its += 1;
      k += 1;
    }
    // ---- KSPGMRESBuildSoln (k_gmres_update): back substitution and x += V y on the slice
    if (warp == 0 && k > 0) back_substitute(H, R, g, k - 1, yv, gbuf);
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
    G.ist[1] = reason == 0 && its >= max_it ? -3 : reason;   // KSP_DIVERGED_ITS
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
    if (G.nf <= 0 || G.restart > 32) return IB_ERR_ARG;   // the Givens warp holds a rotation per lane
    ClusterSmem cs{G.nf, G.restart, (G.nf + kSlices - 1) / kSlices};
    if (slice_blocks_p2(cs.ns) > 16) return IB_ERR_ARG;   // a slice's norm blocks on 16 lanes
    const int threads = kClusterThreads;
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
    IB_CUDA_CHECK(allow_dyn_smem(k_gmres_cluster, bytes));
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
