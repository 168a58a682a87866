// Chunked per-mode tridiagonal solver (see tri.cuh).
#include <algorithm>
#include <cmath>
#include <thread>
#include <vector>

#include "tri.cuh"

namespace ib {

void tri_chunking(int n, int nx, int* s, int* C) {
  // The chunk period d = s+1 divides n, at most 32 chunks.  Every FP64 warp instruction holds
  // its SM sub-partition's FP64 pipe for the same time whatever its active lanes, so the cost
  // of one solve is the FP64 instructions of one chunk thread (about 5 per chunk row and one
  // per interface) times the warps a sub-partition runs, minimised over the launch shapes
  // (Mb modes x C chunks per CTA, Mb a power of two) the tuner can pick.
  constexpr int kSMs = 152;   // GB300: 4 sub-partitions each
  long long best = -1;
  int bestd = n;
  for (int d = 2; d <= n; ++d) {
    if (n % d) continue;
    const int c = n / d;
    if (c > 32) continue;
    const long long per = 5LL * (d - 1) + c;
    for (int Mb = 1; Mb <= 32; Mb *= 2) {
      if (Mb * c > 1024) break;
      const long long wpc = (Mb * c + 31) / 32;                 // warps per CTA
      const long long ncta = (nx + Mb - 1) / Mb;
      const long long mult = ((ncta + kSMs - 1) / kSMs * wpc + 3) / 4;   // warps per sub-partition
      const long long cost = per * mult;
      if (best < 0 || cost < best || (cost == best && d > bestd)) { best = cost; bestd = d; }
    }
  }
  *s = bestd - 1;
  *C = n / bestd;
}

size_t tri_table_doubles(int nx, int s, int C) {
  const size_t m = C > 1 ? (size_t)(C - 1) : 1;
  return (size_t)nx * (3 * (size_t)s + m * m);
}

int tri_build(TriOp* op, int nx, int ny, const double* shift, double sigma, double* dev) {
  int s = 0, C = 0;
  tri_chunking(ny + 1, nx, &s, &C);
  op->nx = nx; op->ny = ny; op->s = s; op->C = C; op->sigma = sigma;
  const int m = C > 1 ? C - 1 : 1;
  const size_t S = (size_t)s * nx, R = (size_t)m * m * nx;
  std::vector<double> tab(3 * S + R, 0.0);
  double* inv = tab.data();
  double* sinv = inv + S;
  double* gL = inv + 2 * S;
  double* rinv = inv + 3 * S;
  // the modes are independent: they are split over host threads (long double arithmetic is
  // software-emulated on some hosts and costs milliseconds per operator otherwise)
  auto modes = [&](int k0, int k1) {
  std::vector<long double> beta(s), d(s), g(s), bp(m), z(m), x(m);
  for (int k = k0; k < k1; ++k) {
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
    if (C < 2) continue;
    // interface system tridiag(-B, A, -B) of size m = C-1, tabulated as its dense inverse
    // (one Thomas solve per unit vector, in extended precision)
    long double A = a - 2.0L * g[0], B = g[s - 1];
    bp[0] = A;
    for (int c = 1; c < m; ++c) bp[c] = A - B * B / bp[c - 1];
    for (int j = 0; j < m; ++j) {
      for (int c = 0; c < m; ++c) z[c] = ((c == j ? 1.0L : 0.0L) + (c > 0 ? B * z[c - 1] : 0.0L)) / bp[c];
      x[m - 1] = z[m - 1];
      for (int c = m - 2; c >= 0; --c) x[c] = z[c] + (B / bp[c]) * x[c + 1];
      for (int c = 0; c < m; ++c) rinv[((size_t)c * m + j) * nx + k] = (double)x[c];
    }
  }
  };
  const int nth = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
  if (nth == 1 || nx < 64) {
    modes(0, nx);
  } else {
    std::vector<std::thread> th;
    for (int t = 0; t < nth; ++t) th.emplace_back(modes, (int)((long long)nx * t / nth), (int)((long long)nx * (t + 1) / nth));
    for (auto& x : th) x.join();
  }
  op->inv = dev;
  op->sinv = dev + S;
  op->gL = dev + 2 * S;
  op->rinv = dev + 3 * S;
  IB_CUDA_CHECK(cudaMemcpy(dev, tab.data(), 8 * tab.size(), cudaMemcpyHostToDevice));
  return IB_OK;
}

// Row r of mode k's right-hand side with the boundary terms (TriBc).
__device__ __forceinline__ double tri_rhs(const TriBc& b, int ny, int nx, int r, int k, double f) {
  double v = b.post_scale == 1.0 ? f : b.post_scale * f;
  if (b.sd) {
    v = fma(__ldg(b.sk2 + k), b.sd[(k & 1) * ny + r], v);
    if (r == 0) v += b.edge[k];
    if (r == ny - 1) v += b.edge[nx + k];
  }
  return v;
}

// One CTA: Mb consecutive modes x C chunks (thread t: mode t % Mb, chunk t / Mb, so a warp
// holds 32/Mb chunks of Mb modes).  The CTA's ny x Mb tile and its factor tables are staged
// in shared memory, so the sequential recurrences run on shared-memory latency.  The
// interface values come from the tabulated inverse of the interface system: every chunk
// thread forms one of them with C-1 independent products, instead of one thread per mode
// running a 2(C-1)-step recurrence while the rest of its warp idles (an FP64 warp
// instruction costs the same issue time whatever its active lanes).
__global__ void k_tri(TriOp op, const double* __restrict__ F, double* U, int ld, int Mb, TriBc bc) {
  IB_GRID_DEP_WAIT();
  extern __shared__ double sm[];
  const int C = op.C, s = op.s, d = s + 1, nx = op.nx, ny = op.ny;
  const int m = C > 1 ? C - 1 : 1;
  const int trows = 3 * s + (C > 1 ? m * m : 0);   // table rows staged: inv, sinv, gL, rinv
  double* tile = sm;                       // ny x Mb
  double* t_inv = tile + (size_t)ny * Mb;  // s x Mb
  double* t_sinv = t_inv + s * Mb;
  double* t_gL = t_sinv + s * Mb;
  double* t_r = t_gL + s * Mb;             // m*m x Mb
  double* pfirst = t_inv + (size_t)trows * Mb;  // C x Mb
  double* plast = pfirst + C * Mb;
  double* hv = plast + C * Mb;             // (C+1) x Mb: interface right-hand sides
  double* yv = hv + (C + 1) * Mb;          // (C+1) x Mb: interface values
  const int k0 = blockIdx.x * Mb;
  const int nthr = blockDim.x;
  // stage the tile (rows of F) and the tables (rows of op.inv.., contiguous with stride nx),
  // coalesced along modes, 8 loads in flight per thread: thread t owns mode column t % Mb
  // and rows t / Mb + i * (nthr / Mb)
  const int rstep = nthr / Mb;
  const int kl0 = threadIdx.x % Mb, r00 = threadIdx.x / Mb;
  const bool kin = k0 + kl0 < nx && r00 < rstep;
  {
    const double* src = F + k0 + kl0;
    const double* tsrc = op.inv + min(k0 + kl0, nx - 1);
    const int tot = ny + trows;
    for (int r = r00; r < tot; r += 8 * rstep) {
      double v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        int rr = r + u * rstep;
        v[u] = 0.0;
        if (rr < ny) {
          if (kin) {
            double f = src[(size_t)rr * ld];
            if (bc.add2) f = f + bc.add2[(size_t)rr * ld + k0 + kl0];
            v[u] = tri_rhs(bc, ny, nx, rr, k0 + kl0, f);
          }
        }
        else if (rr < tot) v[u] = __ldg(tsrc + (size_t)(rr - ny) * nx);
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        int rr = r + u * rstep;
        if (rr < tot && r00 < rstep) tile[rr * Mb + kl0] = v[u];
      }
    }
  }
  __syncthreads();
  const int t = threadIdx.x;
  const int kl = t % Mb, c = t / Mb;
  const bool active = c < C;
  // phase 1: chunk solves with zero ends; interface rows keep f until phase 2
  if (active) {
    double* col = tile + c * d * Mb + kl;
    const double* ti = t_inv + kl;
    const double* ts = t_sinv + kl;
    double dp = 0.0;
    for (int j = 0; j < s; ++j) {
      dp = fma(ti[j * Mb], dp, ts[j * Mb] * col[j * Mb]);
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
  // phase 2a: right-hand side of interface c (between chunks c-1 and c)
  if (active && c >= 1)
    hv[c * Mb + kl] = fma(op.sigma, tile[(c * d - 1) * Mb + kl], plast[(c - 1) * Mb + kl] + pfirst[c * Mb + kl]);
  __syncthreads();
  // phase 2b: interface value c = row c-1 of the interface inverse times the right-hand sides
  if (active) {
    if (c >= 1) {
      const double* rr = t_r + (size_t)(c - 1) * m * Mb + kl;
      const double* hh = hv + Mb + kl;
      double y0 = 0.0, y1 = 0.0;
      int j = 0;
      for (; j + 1 < m; j += 2) {
        y0 = fma(rr[j * Mb], hh[j * Mb], y0);
        y1 = fma(rr[(j + 1) * Mb], hh[(j + 1) * Mb], y1);
      }
      if (j < m) y0 = fma(rr[j * Mb], hh[j * Mb], y0);
      yv[c * Mb + kl] = y0 + y1;
    } else {
      yv[kl] = 0.0;
      yv[C * Mb + kl] = 0.0;
    }
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

// The same solve with each thread's chunk in registers (S = op.s known at compile time): the
// chunk rows and the interface row above are loaded straight from F (all loads in flight at
// once), the thread's row of the interface inverse is prefetched into registers, only the
// pivot and response tables (shared by a mode's chunks) are staged in shared memory, and the
// result is stored straight to U.  Same arithmetic as k_tri.  In place allowed: a thread
// writes only the rows it read, after the CTA's barriers.
constexpr int kTriMaxM = 31;   // interfaces (C-1) the register prefetch holds
template <int S>
__device__ __forceinline__ void tri_reg_body(const TriOp& op, const double* __restrict__ F, double* U, int ld, int Mb,
                                             const TriBc& bc, double* sm) {
  const int C = op.C, d = S + 1, nx = op.nx;
  const int m = C > 1 ? C - 1 : 1;
  double* t_inv = sm;                      // S x Mb
  double* t_sinv = t_inv + S * Mb;
  double* t_gL = t_sinv + S * Mb;
  double* pfirst = t_gL + S * Mb;          // C x Mb
  double* plast = pfirst + C * Mb;
  double* hv = plast + C * Mb;             // (C+1) x Mb
  double* yv = hv + (C + 1) * Mb;          // (C+1) x Mb
  const int k0 = blockIdx.x * Mb, nthr = blockDim.x;
  const int t = threadIdx.x, kl = t % Mb, c = t / Mb;
  const int k = min(k0 + kl, nx - 1);
  const bool chunk = c < C, store = chunk && k0 + kl < nx;
  const int r0 = c * d;
  // the tables are constant (built at creation): fetched before the wait for the previous
  // kernel, so that under a programmatic edge they arrive while it finishes
  double rr[kTriMaxM];
#pragma unroll
  for (int j = 0; j < kTriMaxM; ++j)
    rr[j] = (chunk && c >= 1 && j < m) ? __ldg(op.rinv + ((size_t)(c - 1) * m + j) * nx + k) : 0.0;
  for (int q = t; q < 3 * S * Mb; q += nthr) {
    const int row = q / Mb, kk = q - row * Mb;
    t_inv[q] = __ldg(op.inv + (size_t)row * nx + min(k0 + kk, nx - 1));
  }
  IB_GRID_DEP_WAIT();
  double f[S];
#pragma unroll
  for (int j = 0; j < S; ++j) f[j] = chunk ? F[(size_t)(r0 + j) * ld + k] : 0.0;
  double fi = (chunk && c >= 1) ? F[(size_t)(r0 - 1) * ld + k] : 0.0;
  if (chunk && bc.add2) {
#pragma unroll
    for (int j = 0; j < S; ++j) f[j] = f[j] + bc.add2[(size_t)(r0 + j) * ld + k];
    if (c >= 1) fi = fi + bc.add2[(size_t)(r0 - 1) * ld + k];
  }
  if (chunk && (bc.sd || bc.post_scale != 1.0)) {
    // boundary terms (tri_rhs) on the chunk rows and the interface row above; row 0 is chunk
    // 0's first row and row ny-1 chunk C-1's last
    const double ps = bc.post_scale;
    if (bc.sd) {
      const double a = __ldg(bc.sk2 + k);
      const double* sdk = bc.sd + (k & 1) * op.ny;
#pragma unroll
      for (int j = 0; j < S; ++j) f[j] = fma(a, sdk[r0 + j], ps == 1.0 ? f[j] : ps * f[j]);
      if (c >= 1) fi = fma(a, sdk[r0 - 1], ps == 1.0 ? fi : ps * fi);
      if (c == 0) f[0] += bc.edge[k];
      if (c == C - 1) f[S - 1] += bc.edge[nx + k];
    } else {
#pragma unroll
      for (int j = 0; j < S; ++j) f[j] *= ps;
      fi *= ps;
    }
  }
  __syncthreads();
  // phase 1: chunk solve with zero ends (the products sigma/pivot * f are off the forward
  // recurrence, which takes one FMA per row)
  if (chunk) {
    double dp = 0.0;
#pragma unroll
    for (int j = 0; j < S; ++j) {
      dp = fma(t_inv[j * Mb + kl], dp, t_sinv[j * Mb + kl] * f[j]);
      f[j] = dp;
    }
    plast[c * Mb + kl] = dp;
    double u = dp;
#pragma unroll
    for (int j = S - 2; j >= 0; --j) {
      u = fma(t_inv[j * Mb + kl], u, f[j]);
      f[j] = u;
    }
    pfirst[c * Mb + kl] = u;
  }
  __syncthreads();
  // phase 2a: right-hand side of interface c
  if (chunk && c >= 1) hv[c * Mb + kl] = fma(op.sigma, fi, plast[(c - 1) * Mb + kl] + pfirst[c * Mb + kl]);
  __syncthreads();
  // phase 2b: interface value c
  if (chunk) {
    if (c >= 1) {
      const double* hh = hv + Mb + kl;
      double y0 = 0.0, y1 = 0.0;
#pragma unroll
      for (int j = 0; j + 1 < kTriMaxM; j += 2) {
        if (j + 1 < m) {
          y0 = fma(rr[j], hh[j * Mb], y0);
          y1 = fma(rr[j + 1], hh[(j + 1) * Mb], y1);
        } else if (j < m) {
          y0 = fma(rr[j], hh[j * Mb], y0);
        }
      }
      if ((kTriMaxM & 1) && m == kTriMaxM) y0 = fma(rr[kTriMaxM - 1], hh[(kTriMaxM - 1) * Mb], y0);
      yv[c * Mb + kl] = y0 + y1;
    } else {
      yv[kl] = 0.0;
      yv[C * Mb + kl] = 0.0;
    }
  }
  __syncthreads();
  // phase 3: interface responses, straight to U
  if (store) {
    const double yl = yv[c * Mb + kl], yr = yv[(c + 1) * Mb + kl];
    double* dst = U + k;
#pragma unroll
    for (int j = 0; j < S; ++j) {
      double u = f[j];
      u = fma(yl, t_gL[j * Mb + kl], u);
      u = fma(yr, t_gL[(S - 1 - j) * Mb + kl], u);
      dst[(size_t)(r0 + j) * ld] = u;
    }
    if (c >= 1) dst[(size_t)(r0 - 1) * ld] = yl;
  }
}

template <int S>
__global__ void __launch_bounds__(256) k_tri_reg(TriOp op, const double* __restrict__ F, double* U, int ld, int Mb,
                                                 TriBc bc) {
  extern __shared__ double sm[];
  tri_reg_body<S>(op, F, U, ld, Mb, bc, sm);   // waits for the previous kernel after its tables
}

// The same solve for every item of a batch, blockIdx.y picking the item (its tables, input,
// output and boundary terms); the items share the chunking.
template <int S>
__global__ void __launch_bounds__(256) k_tri_reg_batch(const __grid_constant__ TriBatch b, int ld, int Mb) {
  extern __shared__ double sm[];
  const int y = blockIdx.y;
  tri_reg_body<S>(b.op[y], b.F[y], b.U[y], ld, Mb, b.bc[y], sm);
}

static size_t tri_reg_smem(const TriOp& op, int Mb) {
  return sizeof(double) * (size_t)Mb * (3 * (size_t)op.s + 2 * (size_t)op.C + 2 * ((size_t)op.C + 1));
}

template <int S>
static int launch_tri_reg(const TriOp& op, const double* F, double* U, int ld, int Mb, int threads, const TriBc& bc,
                          cudaStream_t st) {
  const size_t smem = tri_reg_smem(op, Mb);
  if (allow_dyn_smem(k_tri_reg<S>, smem) != cudaSuccess) return IB_ERR_CUDA;
  count_launch();
  k_tri_reg<S><<<cdiv(op.nx, Mb), threads, smem, st>>>(op, F, U, ld, Mb, bc);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

size_t tri_smem(const TriOp& op, int Mb) {
  const size_t m = op.C > 1 ? (size_t)(op.C - 1) : 0;
  return sizeof(double) * (size_t)Mb * ((size_t)op.ny + 3 * (size_t)op.s + m * m + 2 * (size_t)op.C + 2 * ((size_t)op.C + 1));
}

int tri_solve(const TriOp& op, const double* F, double* U, int ld, const TriLaunch& L, cudaStream_t st,
              const TriBc& bc) {
  int Mb = L.Mb;
  int threads = Mb * op.C;
  threads = ((threads + 31) / 32) * 32;
  if (threads > 1024) { Mb = 1024 / op.C; threads = ((Mb * op.C + 31) / 32) * 32; }
  if (op.C - 1 <= kTriMaxM && op.C <= 256) {
    // at most 256 threads (the register-resident chunk needs the registers)
    const int Mr = std::max(1, std::min(Mb, 256 / op.C));
    const int tr = ((Mr * op.C + 31) / 32) * 32;
    switch (op.s) {
#define IB_TRI_REG(SS) \
      case SS: return launch_tri_reg<SS>(op, F, U, ld, Mr, tr, bc, st);
      IB_TRI_REG(1) IB_TRI_REG(2) IB_TRI_REG(3) IB_TRI_REG(4) IB_TRI_REG(5) IB_TRI_REG(6) IB_TRI_REG(7)
      IB_TRI_REG(8) IB_TRI_REG(9) IB_TRI_REG(11) IB_TRI_REG(12) IB_TRI_REG(14) IB_TRI_REG(15) IB_TRI_REG(19)
      IB_TRI_REG(23) IB_TRI_REG(24) IB_TRI_REG(29) IB_TRI_REG(31) IB_TRI_REG(39)
#undef IB_TRI_REG
      default: break;
    }
  }
  size_t smem = tri_smem(op, Mb);
  if (allow_dyn_smem(k_tri, smem) != cudaSuccess) return IB_ERR_CUDA;
  count_launch();
  k_tri<<<cdiv(op.nx, Mb), threads, smem, st>>>(op, F, U, ld, Mb, bc);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

template <int S>
static int launch_tri_reg_batch(const TriBatch& b, int ld, int Mb, int threads, cudaStream_t st) {
  const size_t smem = tri_reg_smem(b.op[0], Mb);
  if (allow_dyn_smem(k_tri_reg_batch<S>, smem) != cudaSuccess) return IB_ERR_CUDA;
  count_launch();
  k_tri_reg_batch<S><<<dim3(cdiv(b.op[0].nx, Mb), b.n), threads, smem, st>>>(b, ld, Mb);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

bool tri_batch_supported(const TriOp& op) {
  if (op.C - 1 > kTriMaxM || op.C > 256) return false;
  switch (op.s) {
    case 1: case 2: case 3: case 4: case 5: case 6: case 7: case 8: case 9: case 11: case 12: case 14:
    case 15: case 19: case 23: case 24: case 29: case 31: case 39: return true;
    default: return false;
  }
}

int tri_solve_batch(const TriBatch& b, int ld, const TriLaunch& L, cudaStream_t st) {
  if (b.n < 1 || b.n > kTriBatch) return IB_ERR_ARG;
  const TriOp& o = b.op[0];
  if (!tri_batch_supported(o)) return IB_ERR_ARG;
  for (int i = 1; i < b.n; ++i)
    if (b.op[i].nx != o.nx || b.op[i].ny != o.ny || b.op[i].s != o.s || b.op[i].C != o.C) return IB_ERR_ARG;
  const int Mr = std::max(1, std::min(L.Mb, 256 / o.C));
  const int tr = ((Mr * o.C + 31) / 32) * 32;
  switch (o.s) {
#define IB_TRI_REG(SS) \
    case SS: return launch_tri_reg_batch<SS>(b, ld, Mr, tr, st);
    IB_TRI_REG(1) IB_TRI_REG(2) IB_TRI_REG(3) IB_TRI_REG(4) IB_TRI_REG(5) IB_TRI_REG(6) IB_TRI_REG(7)
    IB_TRI_REG(8) IB_TRI_REG(9) IB_TRI_REG(11) IB_TRI_REG(12) IB_TRI_REG(14) IB_TRI_REG(15) IB_TRI_REG(19)
    IB_TRI_REG(23) IB_TRI_REG(24) IB_TRI_REG(29) IB_TRI_REG(31) IB_TRI_REG(39)
#undef IB_TRI_REG
    default: return IB_ERR_ARG;
  }
}

}  // namespace ib
