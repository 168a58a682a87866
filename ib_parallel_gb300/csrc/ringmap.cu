// Ring maps: the coarse-to-fine recursions of fluid_predictor (timestepper.F90:103-236,
// operators_fluid.F90:649-663) and of vort2flux (operators_fluid.F90:237-377) without their
// chain of dependent level solves (the state, its layout and the two parity blocks are
// described at RingMaps in ctx.cuh).
//
// The per-level chain runs, for k = L-1 .. 0, a tridiagonal pass of level k and the evaluation
// of level k-1's boundary data from its modes (dst_ring_edge_from_modes): 2L-1 dependent
// launches, each too small to fill the GPU.  Here:
//   1. levels 1..L-1 solved with zero boundary data, one batched launch (the coarsest level
//      has none, so its solve is final);
//   2. the states of those solutions, one batched launch: Ez[k], and R[L-2] from the coarsest;
//   3. R[k-1] = Ez[k] + G_k R[k] for k = L-2 .. 1: L-2 dense products of about
//      (m + n/2)^2 multiply-adds, spread over every SM;
//   4. every level's ring, row sums and edge terms from its state (the arithmetic of
//      dst_ring_edge_from_modes on the state's rows), one batched launch;
//   5. levels 0..L-2 solved with their boundary terms, one batched launch.
// G_k is level k's response: column j is the state of the solve (zero right-hand side) with the
// boundary terms of unit state j, formed at creation with the same expand, solve and extract
// kernels, kTriBatch columns a launch.
//
// Measured at 800 x 400 x 5 (GB300, FP64, graphs): predictor 438 us against 360 for the chain,
// first vort2flux 199 against 166, correction 346 against 302.  Levels 1..L-2 are solved twice,
// the products add (m + n/2)^2 multiply-adds a link, and the batched boundary data issue the
// chain's FP64 work at once, so the GPU's FP64 issue rate, not the chain's latency, sets the time.
#include <algorithm>
#include <chrono>
#include <cstdlib>

#include "ctx.cuh"

namespace ib {

namespace {

constexpr int kRmItems = kTriBatch;   // items (levels, or precomputed columns) of a launch
constexpr int kRmThreads = 256;
constexpr int kRmWarps = kRmThreads / 32;
constexpr int kRmTbSeg = 2 * (kRmWarps - 1);   // ring entries of a bottom/top CTA (kRmWarps vertices)
constexpr int kRmMaxState = 8192;              // larger states keep the per-level chain

// Entry l of parity block b in the state's natural layout [s0 | s1 | vS | vA].
__host__ __device__ __forceinline__ int rm_nat(int N, int NQ, int b, int l) {
  const int Nb = b == 0 ? (N + 1) / 2 : N / 2;
  if (l < Nb) return 2 * l + b;
  if (l < 2 * Nb) return N + 2 * (l - Nb) + b;
  return 2 * N + b * NQ + (l - 2 * Nb);
}

struct RmItems {
  int n = 0;
  const double* in[kRmItems] = {};   // extract: modes (pitch N); expand: state
  double* out[kRmItems] = {};        // extract: state
  double fac[kRmItems] = {};         // expand: the ring's factor
  double* ring[kRmItems] = {};       // expand: nbc entries
  double* sd[kRmItems] = {};         // expand: 2 nsy row terms
  double* edge[kRmItems] = {};       // expand: 2 N edge-row modes
};

// The state of a level's modes: its rows J = n/4+1 and 3n/4+1 (vertex rows n/4-1, 3n/4-1)
// copied, and at the coarse vertices of the left and right sides (rows n/4+1+q, columns
// I = m/4+1 and 3m/4+1) the inverse x transform as one warp's two dot products with W's rows,
// stored as their sum and difference.
__global__ void __launch_bounds__(kRmThreads) k_rm_extract(int N, GridDims g, const double* __restrict__ W,
                                                           const __grid_constant__ RmItems it, int nA) {
  IB_GRID_DEP_WAIT();
  const int y = blockIdx.y;
  const double* __restrict__ spec = it.in[y];
  double* __restrict__ st = it.out[y];
  const int NQ = g.n / 2 + 1;
  int b = blockIdx.x;
  if (b < nA) {
    const int i = b * kRmThreads + (int)threadIdx.x;
    if (i < 2 * N) {
      const int row = i < N ? g.n / 4 - 1 : 3 * g.n / 4 - 1;
      st[i] = spec[(size_t)row * N + (i < N ? i : i - N)];
    }
    return;
  }
  b -= nA;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q = b * kRmWarps + warp;
  if (q >= NQ) return;
  const double* sr = spec + (size_t)(g.n / 4 - 1 + q) * N;
  const double vl = warp_sum(warp_dot_part(sr, W + (size_t)(g.m / 4 - 1) * N, N, lane));
  const double vr = warp_sum(warp_dot_part(sr, W + (size_t)(3 * g.m / 4 - 1) * N, N, lane));
  if (lane == 0) {
    st[2 * N + q] = vl + vr;
    st[2 * N + NQ + q] = vl - vr;
  }
}

// A level's boundary data from its state, as dst_ring_edge_from_modes forms it from the modes:
//  - left/right sides, one thread an entry p = 0..n: coincident vertices copied, midpoints
//    averaged, times fac; the row terms sd[r] = x_l + x_r and sd[nsy + r] = x_l - x_r (r = p-1)
//    straight from vS and vA;
//  - bottom/top sides: kRmWarps coarse vertices a CTA, each a dot product of the state's row
//    with W's row, then the entries;
//  - edge[k], edge[N + k] = fac (E s0)_k, fac (E s1)_k, one warp a mode.
__global__ void __launch_bounds__(kRmThreads) k_rm_expand(int N, GridDims g, const double* __restrict__ W,
                                                          const double* __restrict__ E,
                                                          const __grid_constant__ RmItems it, int nLR, int nTB) {
  IB_GRID_DEP_WAIT();
  __shared__ double sp[kRmWarps];
  const int y = blockIdx.y;
  const double* __restrict__ st = it.in[y];
  const double fac = it.fac[y];
  const int NQ = g.n / 2 + 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int b = blockIdx.x;
  if (b < nLR) {
    const int p = b * kRmThreads + (int)threadIdx.x;
    if (p > g.n) return;
    const double* vS = st + 2 * N;
    const double* vA = vS + NQ;
    const int q = p / 2;
    const double s = (p & 1) ? 0.5 * (vS[q] + vS[q + 1]) : vS[q];
    const double a = (p & 1) ? 0.5 * (vA[q] + vA[q + 1]) : vA[q];
    double* ring = it.ring[y];
    ring[g.left + p] = fac * (0.5 * (s + a));
    ring[g.right + p] = fac * (0.5 * (s - a));
    const int r = p - 1;
    if (r >= 0 && r < g.nsy) {
      it.sd[y][r] = fac * s;
      it.sd[y][g.nsy + r] = fac * a;
    }
    return;
  }
  b -= nLR;
  if (b < 2 * nTB) {
    const int side = b / nTB, cc = b - side * nTB;
    const int len = g.m + 1, qmax = (len - 1) / 2;
    const int q0 = cc * (kRmTbSeg / 2);
    const int q = q0 + warp;
    double acc = 0.0;
    if (q <= qmax) acc = warp_dot_part(st + (size_t)side * N, W + (size_t)(g.m / 4 - 1 + q) * N, N, lane);
    acc = warp_sum(acc);
    if (lane == 0) sp[warp] = acc;
    __syncthreads();
    if ((int)threadIdx.x < kRmTbSeg) {
      const int p = cc * kRmTbSeg + (int)threadIdx.x;
      if (p < len) {
        const int qq = p / 2 - q0;
        const double v = (p & 1) ? 0.5 * (sp[qq] + sp[qq + 1]) : sp[qq];
        it.ring[y][(side == 0 ? g.bottom : g.top) + p] = v * fac;
      }
    }
    return;
  }
  b -= 2 * nTB;
  const int k = b * kRmWarps + warp;
  if (k >= N) return;
  const double2 e = warp_edge_dot(E, N, k, st, st + N, lane);
  if (lane == 0) {
    it.edge[y][k] = fac * e.x;
    it.edge[y][N + k] = fac * e.y;
  }
}

// out = ez + G in on the state (G block-diagonal by parity, each block row-major): one warp an
// output entry, the input staged in block order in shared memory.
__global__ void __launch_bounds__(kRmThreads) k_rm_chain(int N, int NQ, int n0, int n1, const double* __restrict__ G,
                                                         const double* __restrict__ in, const double* __restrict__ ez,
                                                         double* __restrict__ out) {
  IB_GRID_DEP_WAIT();
  extern __shared__ double xs[];
  const int NS = n0 + n1;
  for (int p = threadIdx.x; p < NS; p += kRmThreads) {
    const int b = p >= n0 ? 1 : 0;
    xs[p] = in[rm_nat(N, NQ, b, p - b * n0)];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = blockIdx.x * kRmWarps + warp;
  if (row >= NS) return;
  const int b = row >= n0 ? 1 : 0, l = row - b * n0, nb = b ? n1 : n0;
  const double* gr = G + (b ? (size_t)n0 * n0 : 0) + (size_t)l * nb;
  const double acc = warp_sum(warp_dot_part(gr, xs + b * n0, nb, lane));
  if (lane == 0) {
    const int o = rm_nat(N, NQ, b, l);
    out[o] = ez[o] + acc;
  }
}

// Unit states c0 + y (block b) for the columns of G.
__global__ void k_rm_unit(int N, int NQ, int NS, int b, int c0, double* __restrict__ states) {
  const int y = blockIdx.y;
  const int hot = rm_nat(N, NQ, b, c0 + y);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NS; i += gridDim.x * blockDim.x)
    states[(size_t)y * NS + i] = i == hot ? 1.0 : 0.0;
}

// Column c0 + y of block b of G from the state of its response.
__global__ void k_rm_store(int N, int NQ, int NS, int b, int nb, int c0, const double* __restrict__ states,
                           double* __restrict__ Gb) {
  const int y = blockIdx.y;
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nb) return;
  Gb[(size_t)l * nb + c0 + y] = states[(size_t)y * NS + rm_nat(N, NQ, b, l)];
}

int launch_extract(Ctx* c, const RmItems& it, cudaStream_t st) {
  const GridDims& g = c->g;
  const int N = g.nsx, NQ = g.n / 2 + 1;
  const int nA = cdiv(2 * N, kRmThreads), nB = cdiv(NQ, kRmWarps);
  count_launch();
  k_rm_extract<<<dim3(nA + nB, it.n), kRmThreads, 0, st>>>(N, g, c->wmat, it, nA);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

int launch_expand(Ctx* c, const RmItems& it, cudaStream_t st) {
  const GridDims& g = c->g;
  const int N = g.nsx;
  const int nLR = cdiv(g.n + 1, kRmThreads), nTB = cdiv(g.m + 1, kRmTbSeg), nE = cdiv(N, kRmWarps);
  count_launch();
  k_rm_expand<<<dim3(nLR + 2 * nTB + nE, it.n), kRmThreads, 0, st>>>(N, g, c->wmat, c->emat, it, nLR, nTB);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

int launch_chain(Ctx* c, const double* G, const double* in, const double* ez, double* out, cudaStream_t st) {
  const RingMaps& r = c->rmap;
  const size_t smem = sizeof(double) * (size_t)r.NS;
  if (allow_dyn_smem(k_rm_chain, smem) != cudaSuccess) return IB_ERR_CUDA;
  count_launch();
  k_rm_chain<<<cdiv(r.NS, kRmWarps), kRmThreads, smem, st>>>(r.N, r.NQ, r.nb[0], r.nb[1], G, in, ez, out);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

TriBc ring_bc(Ctx* c, int k, double post_scale) {
  TriBc bc;
  bc.sk2 = c->sk2;
  bc.sd = c->sdv[k];
  bc.edge = c->edgev[k];
  bc.post_scale = post_scale;
  return bc;
}

// G (both blocks) of the solve `op` with ring factor fac, kRmItems columns a round.
int build_map(Ctx* c, const TriOp& op, double fac, double* G, double* scratch) {
  const GridDims& g = c->g;
  RingMaps& r = c->rmap;
  cudaStream_t st = c->st;
  const int N = r.N, NQ = r.NQ, NS = r.NS;
  double* states = scratch;
  double* rings = states + (size_t)kRmItems * NS;
  double* sds = rings + (size_t)kRmItems * g.nbc;
  double* edges = sds + (size_t)kRmItems * 2 * g.nsy;
  double* zero = edges + (size_t)kRmItems * 2 * N;
  double* U = zero + g.ns;
  for (int b = 0; b < 2; ++b) {
    const int nb = r.nb[b];
    double* Gb = G + (b ? (size_t)r.nb[0] * r.nb[0] : 0);
    for (int c0 = 0; c0 < nb; c0 += kRmItems) {
      const int n = std::min(kRmItems, nb - c0);
      count_launch();
      k_rm_unit<<<dim3(cdiv(NS, 256), n), 256, 0, st>>>(N, NQ, NS, b, c0, states);
      IB_CUDA_CHECK(cudaGetLastError());
      RmItems xp, ex;
      TriBatch tb;
      xp.n = ex.n = tb.n = n;
      for (int i = 0; i < n; ++i) {
        double* s_i = states + (size_t)i * NS;
        double* u_i = U + (size_t)i * g.ns;
        xp.in[i] = s_i; xp.fac[i] = fac;
        xp.ring[i] = rings + (size_t)i * g.nbc;
        xp.sd[i] = sds + (size_t)i * 2 * g.nsy;
        xp.edge[i] = edges + (size_t)i * 2 * N;
        tb.op[i] = op; tb.F[i] = zero; tb.U[i] = u_i;
        tb.bc[i].sk2 = c->sk2; tb.bc[i].sd = xp.sd[i]; tb.bc[i].edge = xp.edge[i];
        ex.in[i] = u_i; ex.out[i] = s_i;
      }
      RC(launch_expand(c, xp, st));
      RC(tri_solve_batch(tb, g.nsx, c->tl, st));
      RC(launch_extract(c, ex, st));
      count_launch();
      k_rm_store<<<dim3(cdiv(nb, 256), n), 256, 0, st>>>(N, NQ, NS, b, nb, c0, states, Gb);
      IB_CUDA_CHECK(cudaGetLastError());
    }
  }
  return IB_OK;
}

}  // namespace

void rm_free(Ctx* c) {
  if (c->rmap.mem) cudaFree(c->rmap.mem);
  c->rmap = RingMaps();
}

int rm_prepare(Ctx* c) {
  rm_free(c);
  RingMaps& r = c->rmap;
  const int L = c->L;
  const GridDims& g = c->g;
  // measured slower than the per-level chain (their batched solves, products and boundary
  // data cost more FP64 issue than the chain's latency), so only on request
  const char* e = std::getenv("IB_RING_MAPS");
  if (!e || std::atoi(e) == 0 || L < 3 || L - 1 > kRmItems) return IB_OK;
  if (!tri_batch_supported(c->tri_ctci)) return IB_OK;
  r.N = g.nsx;
  r.NQ = g.n / 2 + 1;
  r.NS = 2 * r.N + 2 * r.NQ;
  r.nb[0] = 2 * ((r.N + 1) / 2) + r.NQ;
  r.nb[1] = 2 * (r.N / 2) + r.NQ;
  if (r.NS > kRmMaxState) { r = RingMaps(); return IB_OK; }
  const size_t gsz = (size_t)r.nb[0] * r.nb[0] + (size_t)r.nb[1] * r.nb[1];
  const size_t dbl = (size_t)(L - 1) * gsz + (size_t)(L - 2) * (g.ns + r.NS) + (size_t)(L - 1) * r.NS;
  const size_t sdbl = (size_t)kRmItems * (r.NS + g.nbc + 2 * (size_t)g.nsy + 2 * (size_t)r.N + g.ns) + g.ns;
  double* scratch = nullptr;
  if (cudaMalloc(&r.mem, dbl * 8) != cudaSuccess || cudaMalloc(&scratch, sdbl * 8) != cudaSuccess) {
    cudaGetLastError();
    if (r.mem) cudaFree(r.mem);
    r = RingMaps();
    return IB_OK;   // the per-level chain
  }
  r.bytes = dbl * 8;
  double* p = r.mem;
  for (int k = 1; k <= L - 2; ++k) { r.Gp[k] = p; p += gsz; }
  r.Gc = p; p += gsz;
  for (int k = 1; k <= L - 2; ++k) { r.Z[k] = p; p += g.ns; }
  for (int k = 1; k <= L - 2; ++k) { r.Ez[k] = p; p += r.NS; }
  for (int k = 0; k <= L - 2; ++k) { r.R[k] = p; p += r.NS; }
  const auto t0 = std::chrono::steady_clock::now();
  int rc = cudaMemsetAsync(scratch, 0, sdbl * 8, c->st) == cudaSuccess ? IB_OK : IB_ERR_CUDA;
  for (int k = 1; k <= L - 2 && rc == IB_OK; ++k) rc = build_map(c, c->tri_pred[k], 0.25 * c->vfac[k], r.Gp[k], scratch);
  if (rc == IB_OK) rc = build_map(c, c->tri_ctci, 1.0, r.Gc, scratch);
  if (rc == IB_OK && cudaStreamSynchronize(c->st) != cudaSuccess) rc = IB_ERR_CUDA;
  cudaFree(scratch);
  if (rc != IB_OK) { rm_free(c); return rc; }
  r.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  r.on = true;
  return IB_OK;
}

int rm_predict(Ctx* c) {
  RingMaps& r = c->rmap;
  const int L = c->L;
  cudaStream_t st = c->st;
  TriBatch tb;
  RmItems ex;
  tb.n = ex.n = L - 1;
  for (int k = 1; k < L; ++k) {
    const bool top = k == L - 1;
    tb.op[k - 1] = c->tri_pred[k];
    tb.F[k - 1] = c->hat[k];
    tb.U[k - 1] = top ? c->hat[k] : r.Z[k];
    ex.in[k - 1] = tb.U[k - 1];
    ex.out[k - 1] = top ? r.R[L - 2] : r.Ez[k];
  }
  RC(tri_solve_batch(tb, c->g.nsx, c->tl, st));
  RC(launch_extract(c, ex, st));
  for (int k = L - 2; k >= 1; --k) RC(launch_chain(c, r.Gp[k], r.R[k], r.Ez[k], r.R[k - 1], st));
  RmItems xp;
  TriBatch fb;
  xp.n = fb.n = L - 1;
  for (int k = 0; k < L - 1; ++k) {
    xp.in[k] = r.R[k]; xp.fac[k] = 0.25 * c->vfac[k];
    xp.ring[k] = c->ringv[k]; xp.sd[k] = c->sdv[k]; xp.edge[k] = c->edgev[k];
    fb.op[k] = c->tri_pred[k]; fb.F[k] = c->hat[k]; fb.U[k] = c->hat[k]; fb.bc[k] = ring_bc(c, k, 1.0);
  }
  RC(launch_expand(c, xp, st));
  return tri_solve_batch(fb, c->g.nsx, c->tl, st);
}

int rm_vort2flux(Ctx* c, double* const* modes, double* F0, bool all_levels, double post0, const double* add0) {
  RingMaps& r = c->rmap;
  const int L = c->L;
  cudaStream_t st = c->st;
  TriBatch tb;
  RmItems ex;
  tb.n = ex.n = L - 1;
  for (int k = 1; k < L; ++k) {
    const bool top = k == L - 1;
    tb.op[k - 1] = c->tri_ctci;
    tb.F[k - 1] = modes[k];
    tb.U[k - 1] = top ? modes[k] : r.Z[k];
    ex.in[k - 1] = tb.U[k - 1];
    ex.out[k - 1] = top ? r.R[L - 2] : r.Ez[k];
  }
  RC(tri_solve_batch(tb, c->g.nsx, c->tl, st));
  RC(launch_extract(c, ex, st));
  for (int k = L - 2; k >= 1; --k) RC(launch_chain(c, r.Gc, r.R[k], r.Ez[k], r.R[k - 1], st));
  RmItems xp;
  TriBatch fb;
  xp.n = L - 1;
  fb.n = all_levels ? L - 1 : 1;
  for (int k = 0; k < L - 1; ++k) {
    xp.in[k] = r.R[k]; xp.fac[k] = 1.0;
    xp.ring[k] = c->ringv[k]; xp.sd[k] = c->sdv[k]; xp.edge[k] = c->edgev[k];
  }
  for (int k = 0; k < fb.n; ++k) {
    fb.op[k] = c->tri_ctci;
    fb.F[k] = modes[k];
    fb.U[k] = k == 0 ? F0 : modes[k];
    fb.bc[k] = ring_bc(c, k, k == 0 ? post0 : 1.0);
    if (k == 0) fb.bc[k].add2 = add0;
  }
  RC(launch_expand(c, xp, st));
  return tri_solve_batch(fb, c->g.nsx, c->tl, st);
}

}  // namespace ib
