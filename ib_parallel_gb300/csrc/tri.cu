// Chunked per-mode tridiagonal solver (see tri.cuh).
#include <cmath>
#include <vector>

#include "tri.cuh"

namespace ib {

void tri_chunking(int n, int* s, int* C) {
  // chunk period d = s+1 divides n; pick the divisor closest to sqrt(n), at most 32 chunks
  int best = n, bestd = 1;
  for (int d = 2; d <= n; ++d) {
    if (n % d) continue;
    int c = n / d;
    if (c > 32) continue;
    int score = std::abs(d * d - n);
    if (score < best) { best = score; bestd = d; }
  }
  *s = bestd - 1;
  *C = n / bestd;
}

size_t tri_table_doubles(int nx, int s, int C) { return (size_t)nx * (3 * (size_t)s + 2 * (size_t)(C - 1) + 2); }

int tri_build(TriOp* op, int nx, int ny, const double* shift, double sigma, double* dev) {
  int s = 0, C = 0;
  tri_chunking(ny + 1, &s, &C);
  op->nx = nx; op->ny = ny; op->s = s; op->C = C; op->sigma = sigma;
  const size_t S = (size_t)s * nx, R = (size_t)(C > 1 ? C - 1 : 1) * nx;
  std::vector<double> inv(S), sinv(S), gL(S), inv2(R, 0.0), e2(R, 0.0);
  std::vector<long double> beta(s), d(s), g(s);
  for (int k = 0; k < nx; ++k) {
    long double a = 2.0L + (long double)shift[k];
    beta[0] = a;
    for (int j = 1; j < s; ++j) beta[j] = a - 1.0L / beta[j - 1];
    for (int j = 0; j < s; ++j) {
      inv[(size_t)j * nx + k] = (double)(1.0L / beta[j]);
      sinv[(size_t)j * nx + k] = (double)((long double)sigma / beta[j]);
    }
    // response to a unit value just left of the chunk: T_s g = e_0
    d[0] = 1.0L / beta[0];
    for (int j = 1; j < s; ++j) d[j] = d[j - 1] / beta[j];
    g[s - 1] = d[s - 1];
    for (int j = s - 2; j >= 0; --j) g[j] = d[j] + g[j + 1] / beta[j];
    for (int j = 0; j < s; ++j) gL[(size_t)j * nx + k] = (double)g[j];
    // interface system tridiag(-B, A, -B), size C-1
    long double A = a - 2.0L * g[0], B = g[s - 1];
    long double bp = A;
    for (int c = 0; c < C - 1; ++c) {
      if (c > 0) bp = A - B * B / bp;
      inv2[(size_t)c * nx + k] = (double)(1.0L / bp);
      e2[(size_t)c * nx + k] = (double)(B / bp);
    }
  }
  op->inv = dev;
  op->sinv = dev + S;
  op->gL = dev + 2 * S;
  op->inv2 = dev + 3 * S;
  op->e2 = dev + 3 * S + R;
  IB_CUDA_CHECK(cudaMemcpy(op->inv, inv.data(), 8 * S, cudaMemcpyHostToDevice));
  IB_CUDA_CHECK(cudaMemcpy(op->sinv, sinv.data(), 8 * S, cudaMemcpyHostToDevice));
  IB_CUDA_CHECK(cudaMemcpy(op->gL, gL.data(), 8 * S, cudaMemcpyHostToDevice));
  IB_CUDA_CHECK(cudaMemcpy(op->inv2, inv2.data(), 8 * R, cudaMemcpyHostToDevice));
  IB_CUDA_CHECK(cudaMemcpy(op->e2, e2.data(), 8 * R, cudaMemcpyHostToDevice));
  return IB_OK;
}

// One CTA: Mb consecutive modes x C chunks (thread t: mode t % Mb, chunk t / Mb).  The
// CTA's ny x Mb tile and its factor tables are staged in shared memory, so the
// sequential recurrences run on shared-memory latency.
__global__ void k_tri(TriOp op, const double* F, double* U, int ld, int Mb) {
  extern __shared__ double sm[];
  const int C = op.C, s = op.s, d = s + 1, nx = op.nx, ny = op.ny;
  double* tile = sm;                       // ny x Mb
  double* t_inv = tile + (size_t)ny * Mb;  // s x Mb
  double* t_sinv = t_inv + s * Mb;
  double* t_gL = t_sinv + s * Mb;
  double* t_inv2 = t_gL + s * Mb;          // (C-1) x Mb
  double* t_e2 = t_inv2 + (C - 1) * Mb;
  double* pfirst = t_e2 + (C - 1) * Mb;    // C x Mb
  double* plast = pfirst + C * Mb;
  double* yv = plast + C * Mb;             // (C+1) x Mb
  const int k0 = blockIdx.x * Mb;
  const int nthr = blockDim.x;
  // stage the tile and the tables (coalesced along modes): thread t owns mode column t % Mb
  // and rows t / Mb + i * (nthr / Mb); no division inside the loops
  const int rstep = nthr / Mb;
  const int kl0 = threadIdx.x % Mb, r00 = threadIdx.x / Mb;
  const bool kin = k0 + kl0 < nx && r00 < rstep;
  {
    const double* src = F + k0 + kl0;
    for (int r = r00; r < ny; r += 4 * rstep) {
      double v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        int rr = r + u * rstep;
        v[u] = (kin && rr < ny) ? src[(size_t)rr * ld] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        int rr = r + u * rstep;
        if (rr < ny && r00 < rstep) tile[rr * Mb + kl0] = v[u];
      }
    }
  }
  for (int q = threadIdx.x; q < s * Mb; q += nthr) {
    int j = q / Mb, kl = q - j * Mb, k = min(k0 + kl, nx - 1);
    t_inv[q] = op.inv[(size_t)j * nx + k];
    t_sinv[q] = op.sinv[(size_t)j * nx + k];
    t_gL[q] = op.gL[(size_t)j * nx + k];
  }
  for (int q = threadIdx.x; q < (C - 1) * Mb; q += nthr) {
    int j = q / Mb, kl = q - j * Mb, k = min(k0 + kl, nx - 1);
    t_inv2[q] = op.inv2[(size_t)j * nx + k];
    t_e2[q] = op.e2[(size_t)j * nx + k];
  }
  __syncthreads();
  const int t = threadIdx.x;
  const int kl = t % Mb, c = t / Mb;
  const bool active = c < C;
  // phase 1: chunk solves with zero ends; interface rows keep sigma*f until phase 3
  if (active) {
    double* col = tile + c * d * Mb + kl;
    const double* ti = t_inv + kl;
    const double* ts = t_sinv + kl;
    double dp = 0.0;
    for (int j = 0; j < s; ++j) {
      dp = fma(ts[j * Mb], col[j * Mb], ti[j * Mb] * dp);
      col[j * Mb] = dp;
    }
    plast[c * Mb + kl] = dp;
    double u = dp;
    for (int j = s - 2; j >= 0; --j) {
      u = fma(ti[j * Mb], u, col[j * Mb]);
      col[j * Mb] = u;
    }
    pfirst[c * Mb + kl] = u;
  }
  __syncthreads();
  // phase 2: interface values, one thread per mode
  if (c == 0) {
    double dp = 0.0;
    for (int ci = 1; ci < C; ++ci) {
      int q = (ci - 1) * Mb + kl;
      double h = fma(op.sigma, tile[(ci * d - 1) * Mb + kl], plast[(ci - 1) * Mb + kl] + pfirst[ci * Mb + kl]);
      dp = fma(t_e2[q], dp, t_inv2[q] * h);
      yv[ci * Mb + kl] = dp;
    }
    double y = 0.0;
    for (int ci = C - 1; ci >= 1; --ci) {
      y = fma(t_e2[(ci - 1) * Mb + kl], y, yv[ci * Mb + kl]);
      yv[ci * Mb + kl] = y;
    }
    yv[kl] = 0.0;
    yv[C * Mb + kl] = 0.0;
  }
  __syncthreads();
  // phase 3: add the interface responses; interface rows take the interface values
  if (active) {
    double* col = tile + c * d * Mb + kl;
    const double* tg = t_gL + kl;
    double yl = yv[c * Mb + kl], yr = yv[(c + 1) * Mb + kl];
    for (int j = 0; j < s; ++j) {
      double u = col[j * Mb];
      u = fma(yl, tg[j * Mb], u);
      u = fma(yr, tg[(s - 1 - j) * Mb], u);
      col[j * Mb] = u;
    }
    if (c >= 1) col[-Mb] = yl;
  }
  __syncthreads();
  if (kin) {
    double* dst = U + k0 + kl0;
    for (int r = r00; r < ny; r += rstep) dst[(size_t)r * ld] = tile[r * Mb + kl0];
  }
}

size_t tri_smem(const TriOp& op, int Mb) {
  return sizeof(double) * (size_t)Mb * ((size_t)op.ny + 3 * op.s + 2 * (op.C - 1) + 2 * op.C + op.C + 1);
}

int tri_solve(const TriOp& op, const double* F, double* U, int ld, const TriLaunch& L, cudaStream_t st) {
  int Mb = L.Mb;
  int threads = Mb * op.C;
  threads = ((threads + 31) / 32) * 32;
  if (threads > 1024) { Mb = 1024 / op.C; threads = ((Mb * op.C + 31) / 32) * 32; }
  size_t smem = tri_smem(op, Mb);
  if (smem > 48 * 1024) {
    if (cudaFuncSetAttribute(k_tri, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return IB_ERR_CUDA;
  }
  count_launch();
  k_tri<<<cdiv(op.nx, Mb), threads, smem, st>>>(op, F, U, ld, Mb);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

}  // namespace ib
