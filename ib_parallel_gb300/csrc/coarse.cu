// The coarse levels' part of the band build and of the sub-domain precompute, by superposition.
//
// One column of either (schur_fluid on a source at the finest level: a unit vertex of the band,
// or the patch rot E_o^T e_j of a sub-domain unknown) runs ainv, coarsifies ainv's response up
// the levels, and solves the coarse levels from L-1 down to 1, each handing the next finer
// level its ring (vort2flux, operators_fluid.F90:237-377, with the vorticity of the operator,
// zero outside the centres coarsify writes).  The ring level 1 hands the finest level, ring0,
// is a linear function of the level-1 vorticity alone (the coarser levels' vorticity is its
// coarsified copies), and that function depends on the grid only.  ainv's response falls below
// 1e-18 of its peak beyond trunc_rows vertices of the source in x and in y (the decay rho per
// vertex of the slowest x mode; the 2-D operator decays at least as fast along either axis),
// so a column's level-1 vorticity is, to that level, a combination of the unit vectors of the
// level-1 vertices whose coarsify stencil meets the box the source widened by trunc_rows
// covers.  With R_1[v] the ring0 of a unit vorticity at level-1 vertex v,
//     ring0 = sum over the box's level-1 vertices v of w1[v] R_1[v].
// R_k[v] for a level-k vertex is one level-k solve: the unit vector at v with the ring level
// k+1 hands it, the sum of R_{k+1}[u] over the level-(k+1) vertices u coarsify spreads v onto
// (full weighting: 1 where v is u's centre, 1/2 beside it, 1/4 on its diagonal), transformed
// along x, solved per mode, its ring for level k-1 evaluated from the modes.  Every coarse
// level then solves once per vertex of its footprint instead of once per column; the responses
// are kept for later builds of the same context.
//
// Each level's vertices are spread over the band build's scratch sets, each set's share one
// captured while-loop graph (the vertex index on the device), as the band's columns are.
#include <algorithm>
#include <chrono>
#include <vector>

#include "ctx.cuh"

namespace ib {

namespace {

// Device memory the responses may take: at most a quarter of what is free, and 4 GiB.
constexpr size_t kMaxBytes = 4ull << 30;

__global__ void k_cr_init(int* col, int c0) {
  IB_GRID_DEP_WAIT();
  if (threadIdx.x == 0) *col = c0;
}

__global__ void k_cr_next(int* col, int stride, int n, cudaGraphConditionalHandle h) {
  IB_GRID_DEP_WAIT();
  if (threadIdx.x != 0) return;
  const int c = *col + stride;
  *col = c;
  cudaGraphSetConditional(h, c < n ? 1u : 0u);
}

// The level-(k+1) vertices (interior x index) coarsify spreads level-k interior index i onto,
// with their weights: the coarse vertex a (interior a + m/4 on level k+1) takes the fine
// vertices 2a, 2a+1, 2a+2 with weights 1/2, 1, 1/2 (k_coarsify).
__device__ __forceinline__ int coarse_of(int i, int ca, int off, int* a, double* w) {
  int n = 0;
  if (i & 1) {
    const int q = (i - 1) >> 1;
    if (q >= 0 && q < ca) { a[n] = q + off; w[n] = 1.0; ++n; }
  } else {
    const int q0 = (i >> 1) - 1, q1 = i >> 1;
    if (q0 >= 0 && q0 < ca) { a[n] = q0 + off; w[n] = 0.5; ++n; }
    if (q1 >= 0 && q1 < ca) { a[n] = q1 + off; w[n] = 0.5; ++n; }
  }
  return n;
}

// Vertex *col of a level's pass: its unit vector (the previous one cleared), the row range of
// its transform (its own row; the others zero on the coarsest level, else zero apart from the
// ring's samples at their ends, with the two edge rows transformed), and the ring it receives
// from level k+1 (none on the coarsest level).
__global__ void __launch_bounds__(256) k_cr_item(const int* __restrict__ col, const int* __restrict__ items,
                                                 GridDims g, int top, const int* __restrict__ idx_up,
                                                 const double* __restrict__ R_up, double* __restrict__ vort,
                                                 int* __restrict__ prev, int* __restrict__ rr,
                                                 double* __restrict__ ring, int* __restrict__ err) {
  IB_GRID_DEP_WAIT();
  const int o = items[*col];
  const int i = o % g.nsx, j = o / g.nsx;
  if (threadIdx.x == 0) {
    const int p = *prev;
    if (p >= 0) vort[p] = 0.0;
    vort[o] = 1.0;
    *prev = o;
    rr[0] = j;
    rr[1] = j + 1;
    rr[2] = top ? ROW_ZERO : ROW_EDGES;
  }
  if (top) return;
  int ax[2], ay[2];
  double wx[2], wy[2];
  const int nx = coarse_of(i, g.m / 2 - 1, g.m / 4, ax, wx);
  const int ny = coarse_of(j, g.n / 2 - 1, g.n / 4, ay, wy);
  int slot[4];
  double wt[4];
  int nu = 0;
  for (int b = 0; b < ny; ++b)
    for (int a = 0; a < nx; ++a) {
      const int s = idx_up[ay[b] * g.nsx + ax[a]];
      if (s < 0) {
        if (threadIdx.x == 0) atomicExch(err, 1);
        continue;
      }
      slot[nu] = s;
      wt[nu] = wx[a] * wy[b];   // 1, 1/2 or 1/4: exact
      ++nu;
    }
  for (int t = threadIdx.x; t < g.nbc; t += blockDim.x) {
    double v = 0.0;
    for (int q = 0; q < nu; ++q) v = fma(wt[q], R_up[(size_t)slot[q] * g.nbc + t], v);
    ring[t] = v;
  }
}

// The ring a pass evaluated, into the vertex's slot.
__global__ void k_cr_store(const int* __restrict__ col, const int* __restrict__ items, const int* __restrict__ idx,
                           const double* __restrict__ ring, int nbc, double* __restrict__ R) {
  IB_GRID_DEP_WAIT();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nbc) return;
  R[(size_t)idx[items[*col]] * nbc + t] = ring[t];
}

// The unit vector of the last vertex of a set cleared.
__global__ void k_cr_clear(double* vort, int* prev) {
  IB_GRID_DEP_WAIT();
  if (threadIdx.x != 0) return;
  const int p = *prev;
  if (p >= 0) vort[p] = 0.0;
  *prev = -1;
}

// A column's ring0: the sum over the level-1 vertices its box reaches (rows, then vertices
// along a row, in order) of w1[v] R_1[v], one thread per ring entry.  With w0 given, every CTA
// first forms the box's level-1 values from the finest field itself (k_coarsify's full-weighting
// sum, the same expression) in shared memory; otherwise w1 holds them (launch_coarsify).
__global__ void __launch_bounds__(128) k_cr_ring0(const int* __restrict__ box, GridDims g,
                                                  const double* __restrict__ w0, const double* __restrict__ w1,
                                                  const int* __restrict__ idx1, const double* __restrict__ R1,
                                                  double* __restrict__ ring, int* __restrict__ err) {
  IB_GRID_DEP_WAIT();
  extern __shared__ double wb[];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int ca = g.m / 2 - 1, cb = g.n / 2 - 1;
  // coarse vertex a reads the fine vertices 2a .. 2a+2 (an empty box reaches none)
  const bool empty = box[1] < box[0] || box[3] < box[2];
  const int a0 = max(0, (box[0] - 1) / 2), a1 = empty ? -1 : min(ca - 1, box[1] / 2);
  const int b0 = max(0, (box[2] - 1) / 2), b1 = empty ? -1 : min(cb - 1, box[3] / 2);
  const int na = a1 - a0 + 1;
  if (w0) {
    const int nq = na > 0 && b1 >= b0 ? na * (b1 - b0 + 1) : 0;
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
      const int I = 2 * (a0 + q % na) + 3, J = 2 * (b0 + q / na) + 3;
      auto F = [&](int ii, int jj) { return w0[(jj - 2) * g.nsx + (ii - 2)]; };
      wb[q] = F(I, J) + 0.5 * (F(I + 1, J) + F(I, J + 1) + F(I - 1, J) + F(I, J - 1)) +
              0.25 * (F(I + 1, J + 1) + F(I + 1, J - 1) + F(I - 1, J - 1) + F(I - 1, J + 1));
    }
    __syncthreads();
  }
  double v = 0.0;
  for (int b = b0; b <= b1; ++b) {
    const int row = (b + g.n / 4) * g.nsx + g.m / 4;
    for (int a = a0; a <= a1; ++a) {
      const int o = row + a;
      const int s = idx1[o];
      const double x = w0 ? wb[(b - b0) * na + (a - a0)] : w1[o];
      if (s < 0) {
        if (x != 0.0 && t == 0) atomicExch(err, 1);
        continue;
      }
      if (t < g.nbc) v = fma(x, R1[(size_t)s * g.nbc + t], v);
    }
  }
  if (t < g.nbc) ring[t] = v;
}

// One pass over `n` vertices of level k (their device list at items, slots already assigned),
// spread over the scratch sets as captured while loops; waits for the sets before it returns.
int run_level(Ctx* c, int k, const int* items, int n) {
  Influence& I = c->inf;
  CoarseResp& cr = I.cr;
  const GridDims& g = c->g;
  const int L = c->L;
  const bool top = k == L - 1;
  const int S = std::min(Influence::kBuildStreams, n);
  cudaStream_t st = c->st;
  cudaEvent_t ev = nullptr;
  IB_CUDA_CHECK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaEventRecord(ev, st);
  for (int i = 0; i < S; ++i) cudaStreamWaitEvent(I.bscr[i].st, ev, 0);
  const bool prof = c->prof_on;
  c->prof_on = false;
  int rc = IB_OK;
  long long body_launches = 0;
  std::vector<cudaGraphExec_t> execs(S, nullptr);
  cudaStream_t cap = nullptr;
  if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) rc = IB_ERR_CUDA;
  const long long l0 = launch_count();
  for (int i = 0; i < S && rc == IB_OK; ++i) {
    const SchurScratch& sc = I.bscr[i];
    int* col = sc.prev + 4;
    cudaGraph_t graph = nullptr;
    do {
      if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeRelaxed) != cudaSuccess) { rc = IB_ERR_CUDA; break; }
      count_launch();
      k_cr_init<<<1, 32, 0, cap>>>(col, i);
      cudaGraphConditionalHandle h = 0;
      cudaGraph_t body = nullptr;
      if (cudaGraphConditionalHandleCreate(&h, capture_graph(cap), 1, cudaGraphCondAssignDefault) != cudaSuccess)
        rc = IB_ERR_CUDA;
      if (rc == IB_OK) rc = add_while(cap, h, &body);
      if (rc == IB_OK &&
          cudaStreamBeginCaptureToGraph(sc.st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess)
        rc = IB_ERR_CUDA;
      if (rc == IB_OK) {
        const long long b0 = launch_count();
        count_launch();
        k_cr_item<<<1, 256, 0, sc.st>>>(col, items, g, top ? 1 : 0, top ? nullptr : cr.idx[k + 1],
                                        top ? nullptr : cr.R[k + 1], sc.vort, sc.prev, sc.rr_in, sc.sbc, cr.err);
        DstXArgs a;
        a.in = sc.vort; a.out = sc.spec1;
        a.ring = sc.sbc; a.fac = 1.0;
        a.rowrange = sc.rr_in;
        a.fft_edge_rows = top ? 0 : 1;
        if (rc == IB_OK) rc = dst_pass_x(c->px, g.nsy, g.nsx, top ? PRE_COPY : PRE_APPLYBC, a, g, c->lx, sc.st);
        if (rc == IB_OK) rc = tri_solve(c->tri_ctci, sc.spec1, sc.spec1, g.nsx, c->tl, sc.st);
        if (rc == IB_OK) rc = dst_ring_from_modes(c->px, g, sc.spec1, g.nsx, c->wmat, 1.0, sc.s0, sc.st);
        count_launches(2);
        k_cr_store<<<cdiv(g.nbc, 256), 256, 0, sc.st>>>(col, items, cr.idx[k], sc.s0, g.nbc, cr.R[k]);
        k_cr_next<<<1, 32, 0, sc.st>>>(col, S, n, h);
        body_launches = launch_count() - b0;
        cudaGraph_t tmp;
        if (cudaStreamEndCapture(sc.st, &tmp) != cudaSuccess && rc == IB_OK) rc = IB_ERR_CUDA;
      }
      if (cudaStreamEndCapture(cap, &graph) != cudaSuccess && rc == IB_OK) rc = IB_ERR_CUDA;
      if (rc == IB_OK) make_edges_programmatic(body);
      if (rc == IB_OK && cudaGraphInstantiate(&execs[i], graph, 0) != cudaSuccess) rc = IB_ERR_CUDA;
    } while (false);
    if (graph) cudaGraphDestroy(graph);
  }
  count_launches(-(launch_count() - l0));   // captured, not run
  cudaGetLastError();
  if (rc == IB_OK) {
    for (int i = 0; i < S && rc == IB_OK; ++i)
      if (cudaGraphLaunch(execs[i], I.bscr[i].st) != cudaSuccess) rc = IB_ERR_CUDA;
    if (rc == IB_OK) {
      count_launches(S + (long long)n * body_launches);
      cr.solves += n;
    }
  }
  c->prof_on = prof;
  for (int i = 0; i < S; ++i) {
    const SchurScratch& sc = I.bscr[i];
    count_launch();
    k_cr_clear<<<1, 32, 0, sc.st>>>(sc.vort, sc.prev);
    cudaEventRecord(ev, sc.st);
    cudaStreamWaitEvent(st, ev, 0);
  }
  for (int i = 0; i < S; ++i) cudaStreamSynchronize(I.bscr[i].st);
  for (cudaGraphExec_t e : execs)
    if (e) cudaGraphExecDestroy(e);
  if (cap) cudaStreamDestroy(cap);
  cudaEventDestroy(ev);
  return rc;
}

}  // namespace

void cr_dilate(const GridDims& g, std::vector<unsigned char>& mask, int r) {
  const int nx = g.nsx, ny = g.nsy;
  std::vector<unsigned char> tmp(mask.size(), 0);
  std::vector<int> pre(std::max(nx, ny) + 1);
  for (int j = 0; j < ny; ++j) {   // along x
    pre[0] = 0;
    for (int i = 0; i < nx; ++i) pre[i + 1] = pre[i] + (mask[(size_t)j * nx + i] ? 1 : 0);
    for (int i = 0; i < nx; ++i) {
      const int lo = std::max(0, i - r), hi = std::min(nx - 1, i + r);
      tmp[(size_t)j * nx + i] = pre[hi + 1] - pre[lo] > 0;
    }
  }
  for (int i = 0; i < nx; ++i) {   // along y
    pre[0] = 0;
    for (int j = 0; j < ny; ++j) pre[j + 1] = pre[j] + (tmp[(size_t)j * nx + i] ? 1 : 0);
    for (int j = 0; j < ny; ++j) {
      const int lo = std::max(0, j - r), hi = std::min(ny - 1, j + r);
      mask[(size_t)j * nx + i] = pre[hi + 1] - pre[lo] > 0;
    }
  }
}

int cr_prepare(Ctx* c, const std::vector<unsigned char>& fine_mask) {
  Influence& I = c->inf;
  CoarseResp& cr = I.cr;
  const GridDims& g = c->g;
  const int L = c->L;
  if (L < 2 || !cr.enabled) return IB_ERR_NOMEM;
  auto t0 = std::chrono::steady_clock::now();
  if (!cr.err) {
    IB_CUDA_CHECK(cudaMalloc(&cr.err, sizeof(int)));
    IB_CUDA_CHECK(cudaMemset(cr.err, 0, sizeof(int)));
  }
  const int nx = g.nsx, ny = g.nsy;
  const int ca = g.m / 2 - 1, cb = g.n / 2 - 1;
  // the footprint of every coarse level: level 1 from the marked finest vertices, each coarser
  // level from the finer one's footprint through coarsify's stencil
  std::vector<std::vector<unsigned char>> foot(L);
  foot[1].assign(g.ns, 0);
  for (int b = 0; b < cb; ++b)
    for (int a = 0; a < ca; ++a) {
      bool hit = false;
      for (int jj = 2 * b; jj <= 2 * b + 2 && !hit; ++jj)
        for (int ii = 2 * a; ii <= 2 * a + 2 && !hit; ++ii) hit = fine_mask[(size_t)jj * nx + ii] != 0;
      if (hit) foot[1][(size_t)(b + g.n / 4) * nx + a + g.m / 4] = 1;
    }
  auto coarse_list = [&](int i, int n2, int off, int* out) {
    int n = 0;
    if (i & 1) {
      const int q = (i - 1) / 2;
      if (q >= 0 && q < n2) out[n++] = q + off;
    } else {
      const int q0 = i / 2 - 1, q1 = i / 2;
      if (q0 >= 0 && q0 < n2) out[n++] = q0 + off;
      if (q1 >= 0 && q1 < n2) out[n++] = q1 + off;
    }
    return n;
  };
  for (int k = 2; k < L; ++k) {
    foot[k].assign(g.ns, 0);
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        if (!foot[k - 1][(size_t)j * nx + i]) continue;
        int ax[2], ay[2];
        const int na = coarse_list(i, ca, g.m / 4, ax), nb = coarse_list(j, cb, g.n / 4, ay);
        for (int q = 0; q < nb; ++q)
          for (int p = 0; p < na; ++p) foot[k][(size_t)ay[q] * nx + ax[p]] = 1;
      }
  }
  // the vertices still without a response, level by level, and the memory they need
  std::vector<std::vector<int>> fresh(L);
  size_t need = 0;
  for (int k = 1; k < L; ++k) {
    if (cr.idx_h[k].empty()) cr.idx_h[k].assign(g.ns, -1);
    for (size_t o = 0; o < (size_t)g.ns; ++o)
      if (foot[k][o] && cr.idx_h[k][o] < 0) fresh[k].push_back((int)o);
    need += (size_t)(cr.n[k] + (int)fresh[k].size()) * g.nbc * 8;
  }
  size_t total_new = 0;
  for (int k = 1; k < L; ++k) total_new += fresh[k].size();
  if (total_new == 0) return IB_OK;
  {
    size_t freeb = 0, totalb = 0;
    IB_CUDA_CHECK(cudaMemGetInfo(&freeb, &totalb));
    if (need > std::min(kMaxBytes, (freeb + cr.bytes) / 4)) return IB_ERR_NOMEM;
  }
  IB_CUDA_CHECK(cudaStreamSynchronize(c->st));
  // slots, the maps on the device, room for the new responses (the old ones kept)
  for (int k = 1; k < L; ++k) {
    if (fresh[k].empty()) continue;
    for (int o : fresh[k]) cr.idx_h[k][o] = cr.n[k]++;
    if (!cr.idx[k]) IB_CUDA_CHECK(cudaMalloc(&cr.idx[k], sizeof(int) * (size_t)g.ns));
    IB_CUDA_CHECK(cudaMemcpy(cr.idx[k], cr.idx_h[k].data(), sizeof(int) * (size_t)g.ns, cudaMemcpyHostToDevice));
    if (cr.n[k] > cr.cap[k]) {
      const int cap = std::max(cr.n[k], cr.cap[k] + cr.cap[k] / 4);
      double* R = nullptr;
      IB_CUDA_CHECK(cudaMalloc(&R, 8 * (size_t)cap * g.nbc));
      if (cr.R[k]) {
        IB_CUDA_CHECK(cudaMemcpy(R, cr.R[k], 8 * (size_t)(cr.n[k] - (int)fresh[k].size()) * g.nbc,
                                 cudaMemcpyDeviceToDevice));
        cudaFree(cr.R[k]);
      }
      cr.bytes += 8 * (size_t)(cap - cr.cap[k]) * g.nbc;
      cr.R[k] = R;
      cr.cap[k] = cap;
    }
  }
  if (total_new > cr.items_cap) {
    if (cr.items) cudaFree(cr.items);
    IB_CUDA_CHECK(cudaMalloc(&cr.items, sizeof(int) * total_new));
    cr.items_cap = total_new;
  }
  std::vector<int> all;
  all.reserve(total_new);
  std::vector<size_t> off(L, 0);
  for (int k = L - 1; k >= 1; --k) {
    off[k] = all.size();
    all.insert(all.end(), fresh[k].begin(), fresh[k].end());
  }
  IB_CUDA_CHECK(cudaMemcpy(cr.items, all.data(), sizeof(int) * all.size(), cudaMemcpyHostToDevice));
  // the slots above now claim responses: if the passes fail, the context stops using them (its
  // later builds run the per-column chain)
  int rc = inf_build_scratch(c);
  for (int k = L - 1; k >= 1 && rc == IB_OK; --k)
    if (!fresh[k].empty()) rc = run_level(c, k, cr.items + off[k], (int)fresh[k].size());
  int err = 0;
  if (rc == IB_OK && cudaMemcpy(&err, cr.err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) rc = IB_ERR_CUDA;
  if (rc == IB_OK && err) rc = IB_ERR_STATE;
  if (rc != IB_OK) {
    cr.enabled = false;
    return rc;
  }
  cr.ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return IB_OK;
}

int launch_cr_ring0(Ctx* c, const SchurScratch& sc, cudaStream_t st) {
  const GridDims& g = c->g;
  // a box reaches at most trunc_rows + 6 level-1 vertices along each axis (a sub-domain patch of
  // 8 widened by trunc_rows on both sides); past 48 KB of them coarsify runs on its own first
  const size_t side = (size_t)c->inf.trunc_rows + 6, bytes = 8 * side * side;
  const bool fused = bytes <= 48 * 1024;
  if (!fused) RC(launch_coarsify(g, sc.w[0], sc.w[1], st));
  count_launch();
  k_cr_ring0<<<cdiv(g.nbc, 128), 128, fused ? bytes : 0, st>>>(sc.box, g, fused ? sc.w[0] : nullptr, sc.w[1],
                                                                sc.cr_idx1, sc.cr_R1, sc.sbc, c->inf.cr.err);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

void cr_free(Ctx* c) {
  CoarseResp& cr = c->inf.cr;
  for (int k = 0; k < kMaxLevels; ++k) {
    if (cr.idx[k]) cudaFree(cr.idx[k]);
    if (cr.R[k]) cudaFree(cr.R[k]);
  }
  if (cr.items) cudaFree(cr.items);
  if (cr.err) cudaFree(cr.err);
  const bool en = cr.enabled;
  cr = CoarseResp{};
  cr.enabled = en;
}

}  // namespace ib
