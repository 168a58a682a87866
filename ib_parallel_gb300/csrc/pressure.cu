// Pressure recovery (calculate_pressure, operators_pressure.F90:110-437): on every level, the
// cell-centred pressure coefficient 2 (P - |u|^2 / 2) from the state after a step, with
//     D D^T P = D N(q) - D E^T f / dt
// solved coarse to fine: the coarsest level's boundary values from its own velocity
// (get_bc_phi1), each finer level's from the coarser level's pressure around its footprint
// (get_bc_phi2), the right-hand side of a finer level restricted onto the coarser ones
// (coarsify_pressure).  The solve on one level, ddti (myfft.F90:192-203), is the 2-D DST-I of
// the m x n cell grid with the eigenvalues of D D^T: as for ctci, the y direction is a per-mode
// tridiagonal solve, and the x direction -- length m, whose m + 1 (801 at 800 cells) the FFT's
// radices 2, 3, 5 do not divide -- is a product with the DST-I matrix W (m x m), with FP64 FMAs:
// the same product on the FP64 tensor cores (mma.sync m8n8k4, kept as the measured alternative)
// ran 686 us against 623 us at 800 x 400 on GB300, whose FP64 tensor path is no faster than its
// FP64 pipe.  Arithmetic follows the reference's expressions: products
// that the reference rounds before a sum are rounded separately here (no contraction).
#include <cmath>
#include <vector>

#include "ctx.cuh"

namespace ib {

// ------------------------------------------------------------------ x transform by GEMM
// C (R x N) = A (R x K) B (K x N), row-major, FP64.  CTA tile 32 x 32 x 16 (325 CTAs for the
// 400 x 800 x 800 product at 800 x 400 cells: a 64 x 64 tile left most SMs idle with 91), four
// warps in 2 x 2, each warp 16 x 16 = 2 x 2 tiles of 8 x 8.  One mma.sync.m8n8k4.f64: lane l
// holds A[l/4][l%4], B[l%4][l/4] and C[l/4][2(l%4) + {0,1}] of its 8 x 4, 4 x 8 and 8 x 8
// tiles.  The FMA variant gives each thread 4 rows x 2 columns of the tile.
constexpr int kPM = 32, kPN = 32, kPK = 16;

__device__ __forceinline__ void mma_f64(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

template <bool MMA>
__global__ void __launch_bounds__(128) k_pgemm(int R, int N, int K, const double* __restrict__ A, int lda,
                                               const double* __restrict__ B, int ldb, double* __restrict__ C,
                                               int ldc) {
  IB_GRID_DEP_WAIT();
  __shared__ double As[kPM][kPK + 1];
  __shared__ double Bs[kPK][kPN + 1];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r0 = blockIdx.y * kPM, c0 = blockIdx.x * kPN;
  const int wr = warp >> 1, wc = warp & 1;
  const int tr = (tid >> 4) * 4, tc = (tid & 15) * 2;   // FMA: rows tr..tr+3, columns tc, tc+1
  double acc[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) acc[i] = 0.0;
  for (int k0 = 0; k0 < K; k0 += kPK) {
    for (int t = tid; t < kPM * kPK; t += 128) {
      const int r = t / kPK, k = t % kPK;
      As[r][k] = (r0 + r < R && k0 + k < K) ? A[(size_t)(r0 + r) * lda + k0 + k] : 0.0;
    }
    for (int t = tid; t < kPK * kPN; t += 128) {
      const int k = t / kPN, c = t % kPN;
      Bs[k][c] = (k0 + k < K && c0 + c < N) ? B[(size_t)(k0 + k) * ldb + c0 + c] : 0.0;
    }
    __syncthreads();
    if (MMA) {
#pragma unroll
      for (int kk = 0; kk < kPK; kk += 4) {
        double a[2], b[2];
#pragma unroll
        for (int i = 0; i < 2; ++i) a[i] = As[wr * 16 + i * 8 + (lane >> 2)][kk + (lane & 3)];
#pragma unroll
        for (int j = 0; j < 2; ++j) b[j] = Bs[kk + (lane & 3)][wc * 16 + j * 8 + (lane >> 2)];
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int j = 0; j < 2; ++j) mma_f64(acc[(i * 2 + j) * 2], acc[(i * 2 + j) * 2 + 1], a[i], b[j]);
      }
    } else {
#pragma unroll
      for (int kk = 0; kk < kPK; ++kk) {
        const double b0 = Bs[kk][tc], b1 = Bs[kk][tc + 1];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const double a = As[tr + i][kk];
          acc[i * 2] = fma(a, b0, acc[i * 2]);
          acc[i * 2 + 1] = fma(a, b1, acc[i * 2 + 1]);
        }
      }
    }
    __syncthreads();
  }
  if (MMA) {
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int r = r0 + wr * 16 + i * 8 + (lane >> 2), c = c0 + wc * 16 + j * 8 + 2 * (lane & 3) + h;
          if (r < R && c < N) C[(size_t)r * ldc + c] = acc[(i * 2 + j) * 2 + h];
        }
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int r = r0 + tr + i, c = c0 + tc + j;
        if (r < R && c < N) C[(size_t)r * ldc + c] = acc[i * 2 + j];
      }
  }
}

static int launch_pgemm(bool mma, int R, int N, int K, const double* A, int lda, const double* B, int ldb, double* C,
                        int ldc, cudaStream_t st) {
  dim3 grid(cdiv(N, kPN), cdiv(R, kPM));
  count_launch();
  if (mma) k_pgemm<true><<<grid, 128, 0, st>>>(R, N, K, A, lda, B, ldb, C, ldc);
  else k_pgemm<false><<<grid, 128, 0, st>>>(R, N, K, A, lda, B, ldb, C, ldc);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}

// ------------------------------------------------------------------ stencils
// velocity-squared term fac ((qx(i+1,j)+qx(i,j))^2 + (qy(i,j+1)+qy(i,j))^2) of cell (i, j)
// (1-based), q = q + q0 (get_bc_phi1 :731-767, static_plus_dynamic :842-853); every product
// rounded before the sum, as the reference evaluates it
__device__ __forceinline__ double qsq(const GridDims& g, const double* qx, const double* q0x, const double* qy,
                                      const double* q0y, int i, int j, double fac) {
  const int ux = (j - 1) * g.nux + (i - 1), vy = (j - 1) * g.nvx + (i - 1);
  const double a = (qx[ux + 1] + q0x[ux + 1]) + (qx[ux] + q0x[ux]);
  const double b = (qy[vy + g.nvx] + q0y[vy + g.nvx]) + (qy[vy] + q0y[vy]);
  return __dmul_rn(fac, __dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)));
}

// nonlinear_corner (:441-455) at vertex (I, J), I = 2..m, J = 2..n
__global__ void k_p_corner(GridDims g, const double* __restrict__ om, const double* __restrict__ qx,
                           const double* __restrict__ q0x, const double* __restrict__ qy,
                           const double* __restrict__ q0y, double* __restrict__ oqx, double* __restrict__ oqy) {
  IB_GRID_DEP_WAIT();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.ns) return;
  const int I = t % g.nsx + 2, J = t / g.nsx + 2;
  const int v = (J - 1) * g.nvx + (I - 1), u = (J - 1) * g.nux + (I - 1);
  const double w = om[t];
  oqx[t] = 0.5 * ((qy[v] + q0y[v]) + (qy[v - 1] + q0y[v - 1])) * w;
  oqy[t] = -0.5 * ((qx[u] + q0x[u]) + (qx[u - g.nux] + q0x[u - g.nux])) * w;
}

// a vertex field with its ghost ring (left, right columns; bottom, top rows, which win at the
// corners), as nonlinear_corner2edge fills it (:459-481)
__device__ __forceinline__ double ghosted(const GridDims& g, const double* f, const double* ring, int I, int J) {
  if (J == 1) return ring[g.bottom + I - 1];
  if (J == g.n + 1) return ring[g.top + I - 1];
  if (I == 1) return ring[g.left + J - 1];
  if (I == g.m + 1) return ring[g.right + J - 1];
  return f[(J - 2) * g.nsx + (I - 2)];
}

// nonlinear_corner2edge (:459-501) divided by del^2: u-faces then v-faces
__global__ void k_p_corner2edge(GridDims g, const double* __restrict__ oqx, const double* __restrict__ oqy,
                                const double* __restrict__ ubc, const double* __restrict__ vbc, double d2,
                                double* __restrict__ nlx, double* __restrict__ nly) {
  IB_GRID_DEP_WAIT();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < g.nu) {
    const int i = t % g.nux + 1, j = t / g.nux + 1;
    nlx[t] = 0.5 * (ghosted(g, oqx, ubc, i, j + 1) + ghosted(g, oqx, ubc, i, j)) / d2;
  } else if (t < g.nu + g.nv) {
    const int s = t - g.nu;
    const int i = s % g.nvx + 1, j = s / g.nvx + 1;
    nly[s] = 0.5 * (ghosted(g, oqy, vbc, i + 1, j) + ghosted(g, oqy, vbc, i, j)) / d2;
  }
}

__global__ void k_p_fdt(int nf, const double* __restrict__ f, double dt, double* __restrict__ out) {
  IB_GRID_DEP_WAIT();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nf) out[t] = f[t] / dt;
}

// divergence (:505-516) of face fields into cell (i, j): mode 0 out = -div, 1 out += div
__global__ void k_p_div(GridDims g, const double* __restrict__ hx, const double* __restrict__ hy,
                        double* __restrict__ out, int mode) {
  IB_GRID_DEP_WAIT();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.m * g.n) return;
  const int i = t % g.m + 1, j = t / g.m + 1;
  const int u = (j - 1) * g.nux + (i - 1), v = (j - 1) * g.nvx + (i - 1);
  const double d = hx[u + 1] - hx[u] + hy[v + g.nvx] - hy[v];
  out[t] = mode == 0 ? -d : out[t] + d;
}

// coarsify_pressure (:529-563): full-weighting sum at even cell (i, j) of the fine field
__device__ __forceinline__ double p_weight(const double* p, int m, int i, int j) {
  auto P = [&](int a, int b) { return p[(b - 1) * m + (a - 1)]; };
  const double s1 = P(i + 1, j) + P(i, j + 1) + P(i - 1, j) + P(i, j - 1);
  const double s2 = P(i + 1, j + 1) + P(i + 1, j - 1) + P(i - 1, j - 1) + P(i - 1, j + 1);
  return __dadd_rn(__dadd_rn(P(i, j), __dmul_rn(0.5, s1)), __dmul_rn(0.25, s2));
}
// coarse cell (m/4 + i/2 + 1, n/4 + j/2 + 1) from the four sums around fine cell (i+1, j+1),
// i, j = 2..m-4, n-4 even (the coarse field is cleared first)
__global__ void k_p_coarsify(GridDims g, const double* __restrict__ fine, double* __restrict__ coarse) {
  IB_GRID_DEP_WAIT();
  const int nxi = (g.m - 4) / 2, nyj = (g.n - 4) / 2;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nxi * nyj) return;
  const int i = 2 * (t % nxi) + 2, j = 2 * (t / nxi) + 2;
  const double a = p_weight(fine, g.m, i, j), b = p_weight(fine, g.m, i + 2, j);
  const double c = p_weight(fine, g.m, i, j + 2), d = p_weight(fine, g.m, i + 2, j + 2);
  const double yy = __dadd_rn(__dadd_rn(__dadd_rn(a, __dmul_rn(3.0, b)), __dmul_rn(3.0, c)), __dmul_rn(9.0, d)) / 16.0;
  coarse[(g.n / 4 + j / 2) * g.m + (g.m / 4 + i / 2)] = yy;
}

// get_bc_phi1 (:731-767): ring (left[n], right[n], bottom[m], top[m]) of the coarsest level
__global__ void k_p_bc_phi1(GridDims g, const double* __restrict__ qx, const double* __restrict__ q0x,
                            const double* __restrict__ qy, const double* __restrict__ q0y, double fac,
                            double* __restrict__ ring) {
  IB_GRID_DEP_WAIT();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = g.m, n = g.n;
  if (t >= 2 * m + 2 * n) return;
  int i, j;
  if (t < n) { i = 1; j = t + 1; }
  else if (t < 2 * n) { i = m; j = t - n + 1; }
  else if (t < 2 * n + m) { i = t - 2 * n + 1; j = 1; }
  else { i = t - 2 * n - m + 1; j = n; }
  ring[t] = qsq(g, qx, q0x, qy, q0y, i, j, fac);
}

// get_bc_phi2 (:771-817): a finer level's ring from the coarse cells just outside its footprint
__global__ void k_p_bc_phi2(GridDims g, const double* __restrict__ p, double* __restrict__ ring) {
  IB_GRID_DEP_WAIT();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = g.m, n = g.n;
  if (t >= 2 * m + 2 * n) return;
  auto P = [&](int a, int b) { return p[(b - 1) * m + (a - 1)]; };
  int side, q;   // 0 left, 1 right, 2 bottom, 3 top; q = slot along the side
  if (t < n) { side = 0; q = t; }
  else if (t < 2 * n) { side = 1; q = t - n; }
  else if (t < 2 * n + m) { side = 2; q = t - 2 * n; }
  else { side = 3; q = t - 2 * n - m; }
  const int h = q & 1;
  double v;
  if (side >= 2) {
    const int i = q / 2 + 1 + m / 4;
    const int j = side == 2 ? n / 4 : 3 * n / 4 + 1, jn = side == 2 ? j + 1 : j - 1;
    v = 0.25 * (2 * P(i, j) + P(i, jn) + P(h ? i + 1 : i - 1, j));
  } else {
    const int j = q / 2 + 1 + n / 4;
    const int i = side == 0 ? m / 4 : 3 * m / 4 + 1, in = side == 0 ? i + 1 : i - 1;
    v = 0.25 * (2 * P(i, j) + P(in, j) + P(i, h ? j + 1 : j - 1));
  }
  ring[t] = v;
}

// apply_bc_phi (:821-838): left, right, bottom, top subtracted in that order
__global__ void k_p_apply_bc(GridDims g, double* __restrict__ rhs, const double* __restrict__ ring) {
  IB_GRID_DEP_WAIT();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = g.m, n = g.n;
  if (t >= m * n) return;
  const int i = t % m + 1, j = t / m + 1;
  if (i != 1 && i != m && j != 1 && j != n) return;
  double v = rhs[t];
  if (i == 1) v = v - ring[j - 1];
  if (i == m) v = v - ring[n + j - 1];
  if (j == 1) v = v - ring[2 * n + i - 1];
  if (j == n) v = v - ring[2 * n + m + i - 1];
  rhs[t] = v;
}

// static_plus_dynamic (:842-853) and the pressure-coefficient scale 2
__global__ void k_p_final(GridDims g, double* __restrict__ p, const double* __restrict__ qx,
                          const double* __restrict__ q0x, const double* __restrict__ qy,
                          const double* __restrict__ q0y, double fac) {
  IB_GRID_DEP_WAIT();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.m * g.n) return;
  const int i = t % g.m + 1, j = t / g.m + 1;
  p[t] = 2.0 * __dsub_rn(p[t], qsq(g, qx, q0x, qy, q0y, i, j, fac));
}

// ------------------------------------------------------------------ set-up and the solve
static int pressure_setup(Ctx* c) {
  PressureOp& P = c->pres;
  if (P.ready) return IB_OK;
  const GridDims& g = c->g;
  const int m = g.m, n = g.n, L = c->L;
  const size_t cells = (size_t)m * n;
  int s = 0, C = 0;
  tri_chunking(n + 1, m, &s, &C);
  const size_t tri_n = tri_table_doubles(m, s, C);
  const size_t dbl = (size_t)m * m + tri_n + 2 * (size_t)L * cells + 2 * cells + 2 * (size_t)L * g.ns +
                     (size_t)L * (g.nu + g.nv) + g.nu + g.nv + (size_t)std::max(c->nf, 1) + 2 * (size_t)g.nbc +
                     2 * (size_t)(m + n) + 64;
  IB_CUDA_CHECK(cudaMalloc(&P.mem, 8 * dbl));
  IB_CUDA_CHECK(cudaMemset(P.mem, 0, 8 * dbl));
  double* q = P.mem;
  auto take = [&](size_t k) { double* r = q; q += (k + 3) & ~size_t(3); return r; };
  P.W = take((size_t)m * m);
  double* tri_mem = take(tri_n);
  for (int k = 0; k < L; ++k) { P.rhs.push_back(take(cells)); P.p.push_back(take(cells)); }
  P.y = take(cells);
  P.tmp = take(cells);
  for (int k = 0; k < L; ++k) { P.oqx.push_back(take(g.ns)); P.oqy.push_back(take(g.ns)); }
  for (int k = 0; k < L; ++k) { P.nlx.push_back(take(g.nu)); P.nly.push_back(take(g.nv)); }
  P.hx = take(g.nu); P.hy = take(g.nv);
  P.fdt = take(std::max(c->nf, 1));
  P.ubc = take(g.nbc); P.vbc = take(g.nbc);
  P.ring = take(2 * (size_t)(m + n));
  // W[j][k] = 2 sin(pi (j+1)(k+1) / (m+1)), the DST-I matrix of length m (symmetric)
  {
    std::vector<double> W((size_t)m * m), tab(2 * (size_t)(m + 1));
    const long double PI_L = 3.141592653589793238462643383279502884L;
    const long long M = m + 1;
    for (long long r = 0; r < 2 * M; ++r) tab[r] = (double)(2.0L * sinl(PI_L * (long double)r / (long double)M));
    for (int j = 0; j < m; ++j)
      for (int k = 0; k < m; ++k)   // sin(pi r / M) is 2M-periodic in r
        W[(size_t)j * m + k] = tab[((long long)(j + 1) * (k + 1)) % (2 * M)];
    IB_CUDA_CHECK(cudaMemcpy(P.W, W.data(), 8 * W.size(), cudaMemcpyHostToDevice));
  }
  // ddti = S_x S_y [1 / (lam N)] S_y S_x with lam = -(lx + ly), N = 4 (m+1)(n+1); with
  // S_y diag(1/(lx + ly)) S_y = 2 (n+1) (lx + T_y)^-1, T_y = tridiag(-1, 2, -1) of n rows:
  // ddti = S_x [ -1/(2 (m+1)) (lx(k) + T_y)^-1 ] S_x, lx(k) = 4 sin^2(pi k / (2 (m+1)))
  {
    std::vector<double> lx(m);
    const double pi = 4.0 * std::atan(1.0);
    for (int k = 1; k <= m; ++k) {
      const double sn = std::sin(pi * (double)k / (2.0 * (m + 1)));
      lx[k - 1] = 4.0 * sn * sn;
    }
    RC(tri_build(&P.tri, m, n, lx.data(), -1.0 / (2.0 * (m + 1)), tri_mem));
  }
  IB_CUDA_CHECK(cudaDeviceSynchronize());   // the tables' pageable copies have landed
  P.ready = true;
  return IB_OK;
}

void pressure_free(Ctx* c) {
  if (c->pres.mem) cudaFree(c->pres.mem);
  c->pres = PressureOp{};
}

static int ddti(Ctx* c, const double* rhs, double* out, bool mma) {
  PressureOp& P = c->pres;
  const int m = c->g.m, n = c->g.n;
  RC(launch_pgemm(mma, n, m, m, rhs, m, P.W, m, P.y, m, c->st));
  TriLaunch T;
  T.Mb = 8;
  RC(tri_solve(P.tri, P.y, P.y, m, T, c->st));
  return launch_pgemm(mma, n, m, m, P.y, m, P.W, m, out, m, c->st);
}

int op_pressure(Ctx* c) {
  RC(pressure_setup(c));
  PressureOp& P = c->pres;
  const GridDims& g = c->g;
  const int L = c->L, m = g.m, n = g.n;
  const size_t cells = (size_t)m * n;
  cudaStream_t st = c->st;
  const int B = 256;
  // nonlinear terms on every level, coarse to fine (each finer level's ghost ring is get_bc of
  // the coarser level's vertex products)
  for (int k = L - 1; k >= 0; --k) {
    count_launch();
    k_p_corner<<<cdiv(g.ns, B), B, 0, st>>>(g, c->omega[k], c->qx[k], c->q0x[k], c->qy[k], c->q0y[k], P.oqx[k],
                                            P.oqy[k]);
    if (k == L - 1) {
      IB_CUDA_CHECK(cudaMemsetAsync(P.ubc, 0, 8 * (size_t)g.nbc, st));
      IB_CUDA_CHECK(cudaMemsetAsync(P.vbc, 0, 8 * (size_t)g.nbc, st));
    } else {
      RC(launch_get_bc(g, P.oqx[k + 1], 1.0, P.ubc, st));
      RC(launch_get_bc(g, P.oqy[k + 1], 1.0, P.vbc, st));
    }
    const double d = c->delta * (double)(1 << k);
    count_launch();
    k_p_corner2edge<<<cdiv(g.nu + g.nv, B), B, 0, st>>>(g, P.oqx[k], P.oqy[k], P.ubc, P.vbc, d * d, P.nlx[k],
                                                        P.nly[k]);
  }
  // -D E^T f / dt on the finest level, restricted onto the coarser ones, then D N(q) added
  IB_CUDA_CHECK(cudaMemsetAsync(P.rhs[0], 0, 8 * cells, st));
  if (c->nf > 0) {
    count_launch();
    k_p_fdt<<<cdiv(c->nf, B), B, 0, st>>>(c->nf, c->f, c->p.dt, P.fdt);
    IB_CUDA_CHECK(cudaMemsetAsync(P.hx, 0, 8 * (size_t)g.nu, st));
    IB_CUDA_CHECK(cudaMemsetAsync(P.hy, 0, 8 * (size_t)g.nv, st));
    RC(launch_reg(g, c->nf, P.fdt, c->reg, P.hx, P.hy, st));
    count_launch();
    k_p_div<<<cdiv(cells, B), B, 0, st>>>(g, P.hx, P.hy, P.rhs[0], 0);
  }
  for (int k = 1; k < L; ++k) {
    IB_CUDA_CHECK(cudaMemsetAsync(P.rhs[k], 0, 8 * cells, st));
    count_launch();
    k_p_coarsify<<<cdiv((size_t)((m - 4) / 2) * ((n - 4) / 2), B), B, 0, st>>>(g, P.rhs[k - 1], P.rhs[k]);
  }
  for (int k = 0; k < L; ++k) {
    count_launch();
    k_p_div<<<cdiv(cells, B), B, 0, st>>>(g, P.nlx[k], P.nly[k], P.rhs[k], 1);
  }
  // the solve, coarse to fine
  for (int k = L - 1; k >= 0; --k) {
    count_launch();
    if (k == L - 1) {
      const double d = c->delta * std::pow(2.0, k);
      k_p_bc_phi1<<<cdiv(2 * (m + n), B), B, 0, st>>>(g, c->qx[k], c->q0x[k], c->qy[k], c->q0y[k], 0.125 / (d * d),
                                                      P.ring);
    } else {
      k_p_bc_phi2<<<cdiv(2 * (m + n), B), B, 0, st>>>(g, P.p[k + 1], P.ring);
    }
    count_launch();
    k_p_apply_bc<<<cdiv(cells, B), B, 0, st>>>(g, P.rhs[k], P.ring);
    RC(ddti(c, P.rhs[k], P.p[k], false));
  }
  for (int k = 0; k < L; ++k) {
    const double d = c->delta * std::pow(2.0, k);
    count_launch();
    k_p_final<<<cdiv(cells, B), B, 0, st>>>(g, P.p[k], c->qx[k], c->q0x[k], c->qy[k], c->q0y[k], 0.125 / (d * d));
  }
  IB_CUDA_CHECK(cudaGetLastError());
  P.computed = true;
  return IB_OK;
}

// Average device time (ms) of the pressure grid's x transform (n x m times the m x m DST-I
// matrix) on the FP64 tensor cores (mma) or with FP64 FMAs, over reps launches on inputs
// cycling through fields larger than L2 in total.
int op_time_pressure_transform(Ctx* c, bool mma, int reps, double* avg_ms) {
  RC(pressure_setup(c));
  const int m = c->g.m, n = c->g.n;
  const size_t cells = (size_t)m * n;
  int dev = 0, l2 = 0;
  IB_CUDA_CHECK(cudaGetDevice(&dev));
  IB_CUDA_CHECK(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev));
  const int nbuf = std::max(2, (int)((2 * (size_t)l2 + 8 * cells - 1) / (8 * cells)));
  double* buf = nullptr;
  IB_CUDA_CHECK(cudaMalloc(&buf, 2 * 8 * cells * nbuf));
  int rc = cudaMemsetAsync(buf, 0x3f, 2 * 8 * cells * nbuf, c->st) == cudaSuccess ? IB_OK : IB_ERR_CUDA;
  auto run = [&](int i) {
    double* in = buf + (size_t)(2 * (i % nbuf)) * cells;
    return launch_pgemm(mma, n, m, m, in, m, c->pres.W, m, in + cells, m, c->st);
  };
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (rc == IB_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) rc = IB_ERR_CUDA;
  for (int i = 0; i < nbuf && rc == IB_OK; ++i) rc = run(i);
  if (rc == IB_OK) cudaEventRecord(e0, c->st);
  for (int r = 0; r < reps && rc == IB_OK; ++r) rc = run(r);
  if (rc == IB_OK) cudaEventRecord(e1, c->st);
  if (rc == IB_OK && cudaEventSynchronize(e1) != cudaSuccess) rc = IB_ERR_CUDA;
  float ms = 0.f;
  if (rc == IB_OK) cudaEventElapsedTime(&ms, e0, e1);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamSynchronize(c->st);
  cudaFree(buf);
  RC(rc);
  *avg_ms = ms / reps;
  return IB_OK;
}

}  // namespace ib
