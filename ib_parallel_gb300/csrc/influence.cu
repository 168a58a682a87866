// Influence-matrix evaluation of the Schur operator a_times2 / ab_times
// (operators_fluid.F90:14-120, timestepper.F90:774-782) for moving bodies.
//
// The operator is y = E curl G rot E^T x + B x, where G (vorticity on the finest level ->
// finest-level streamfunction: ainv, then vort2flux with every coarser level) does not
// depend on the body positions.  G is evaluated once on a band of vertices around the
// bodies (one column per band vertex, each a matrix-free application of the fluid part),
// and every FSI iteration assembles the dense nf x nf matrix
//     S_f = P^T K P,   P = rot E^T (one 8 x 8 vertex patch per unknown; curl = rot^T)
// in a few microseconds.  The Krylov iteration then multiplies by S_f instead of running
// the nested-grid solve: the same linear operator, evaluated in another order.
#include <algorithm>
#include <chrono>
#include <cmath>

#include "ctx.cuh"
#include "fsi_dev.cuh"

namespace ib {

namespace {
constexpr int kT = Influence::kTile;   // tile edge (vertices)
constexpr int kP = 64;                 // patch size (8 x 8 vertices)
}  // namespace

// Per unknown k (one CTA of 64 threads): its patch (patch_entry).
__global__ void k_inf_patch(GridDims g, int nf, const int* __restrict__ comp, const int* __restrict__ ix,
                            const int* __restrict__ iy, const double* __restrict__ w,
                            const int* __restrict__ tile_of, int ntx, double* __restrict__ pval,
                            int* __restrict__ pidx, int* __restrict__ used, int* __restrict__ flag) {
  IB_GRID_DEP_WAIT();
  const int k = blockIdx.x, q = threadIdx.x;
  if (k >= nf || q >= kP) return;
  patch_entry(g, k, q, comp[k] == 1, ix[k], iy[k], w + (size_t)k * 49, tile_of, ntx, kT, pval, pidx, used, flag);
}

// Compaction of the touched band vertices (one CTA of 1024 threads).  clear: also clears the
// flags it read, so the next k_inf_patch starts from zero (patches recomputed every iteration;
// a stationary body's patches are computed once and their flags kept).
__global__ void k_inf_compact(int nR, int* __restrict__ used, int* __restrict__ ulist,
                              int* __restrict__ upos, int* __restrict__ nu, int clear) {
  IB_GRID_DEP_WAIT();
  __shared__ int wsum[32];
  __shared__ int base;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if (tid == 0) base = 0;
  __syncthreads();
  for (int c0 = 0; c0 < nR; c0 += 1024) {
    const int i = c0 + tid;
    const int f = (i < nR && used[i]) ? 1 : 0;
    if (f && clear) used[i] = 0;
    int x = f;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int s = wsum[lane], inc = s;
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
      }
      wsum[lane] = inc - s;
    }
    __syncthreads();
    const int pos = base + wsum[wid] + x - f;
    if (i < nR) {
      upos[i] = f ? pos : -1;
      if (f) ulist[pos] = i;
    }
    __syncthreads();
    if (tid == 1023) base = pos + f;
    __syncthreads();
  }
  if (tid == 0) *nu = base;
}

// T[l][u] = sum_q P[q,l] K[ulist[u]][src_q]: the response at every touched vertex to the
// patch of unknown l.  Grid (blocks striding over the touched vertices, nf); K columns are read
// coalesced along rows.
__global__ void k_inf_kp(int nR, const double* __restrict__ K, const double* __restrict__ pval,
                         const int* __restrict__ pidx, const int* __restrict__ ulist, const int* __restrict__ nu,
                         double* __restrict__ T) {
  IB_GRID_DEP_WAIT();
  __shared__ double sv[kP];
  __shared__ int si[kP];
  const int l = blockIdx.y;
  if (threadIdx.x < kP) {
    sv[threadIdx.x] = pval[(size_t)l * kP + threadIdx.x];
    si[threadIdx.x] = pidx[(size_t)l * kP + threadIdx.x];
  }
  __syncthreads();
  const int n = *nu;
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
    const int r = ulist[u];
    double acc = 0.0;
#pragma unroll 8
    for (int q = 0; q < kP; ++q) {
      const int c = si[q];
      if (c >= 0) acc = fma(sv[q], K[(size_t)c * nR + r], acc);
    }
    T[(size_t)l * nR + u] = acc;
  }
}

// BR rows and b_times2 coefficients of the torsional unknowns (one warp per body), so that
// the rank-one B of b_times2 (operators_struct.F90:14-127) can be added to the matrix:
// B[k][l] = BR_k BR_l (delta^2/ds/dt)(2 ds/dt) / K_eff for k, l on the same body.
__global__ void k_inf_bvec(const TorsBody* __restrict__ tb, TorsState ts, double dt, double delta,
                           double* __restrict__ brv, double* __restrict__ bco, int* __restrict__ bod) {
  IB_GRID_DEP_WAIT();
  const int t = blockIdx.x;
  const TorsBody b = tb[t];
  const double sv = ts.sinv[t], cv = ts.cosv[t];
  const double co = btimes_scale(b, dt, delta) / keff(b, dt);
  for (int j = threadIdx.x; j < 2 * b.npts; j += blockDim.x) {
    brv[b.off + j] = br_val(b, sv, cv, j);
    bco[b.off + j] = co;
    bod[b.off + j] = t;
  }
}

// S[k][l] = sum_q P[q,k] T[l][upos(src_q)]  (E curl = P^T), one CTA per row k; also the
// solver's column-major operator St[l][k] = S[k][l] + B[k][l].
__global__ void k_inf_ptk(int nf, int nR, const double* __restrict__ pval, const int* __restrict__ pidx,
                          const int* __restrict__ upos, const double* __restrict__ T,
                          const double* __restrict__ brv, const double* __restrict__ bco,
                          const int* __restrict__ bod, double* __restrict__ S, double* __restrict__ St) {
  IB_GRID_DEP_WAIT();
  __shared__ double sv[kP];
  __shared__ int su[kP];
  const int k = blockIdx.x;
  if (threadIdx.x < kP) {
    const int c = pidx[(size_t)k * kP + threadIdx.x];
    sv[threadIdx.x] = pval[(size_t)k * kP + threadIdx.x];
    su[threadIdx.x] = c >= 0 ? upos[c] : -1;
  }
  __syncthreads();
  const int bk = bod[k];
  for (int l = threadIdx.x; l < nf; l += blockDim.x) {
    const double* Tl = T + (size_t)l * nR;
    double acc = 0.0;
    for (int q = 0; q < kP; ++q) {
      const int u = su[q];
      if (u >= 0) acc = fma(sv[q], Tl[u], acc);
    }
    S[(size_t)k * nf + l] = acc;
    const double bkl = (bk >= 0 && bod[l] == bk) ? brv[k] * brv[l] * bco[k] : 0.0;
    St[(size_t)l * nf + k] = acc + bkl;
  }
}

// y = A x with A column-major (At[j][r] = A[r][j]): kSlices threads per row, each summing one
// column segment in order, combined by a fixed shuffle tree -- the product the cluster
// GMRES solver forms, so that both solvers see identical operator outputs.
__global__ void k_dense_mv(int n, const double* __restrict__ At, const double* __restrict__ x, double* __restrict__ y) {
  IB_GRID_DEP_WAIT();
  // rows in groups of S lanes, 32/S groups per warp (the cluster solver's layout)
  const int S = mv_segments(n), gpw = 32 / S, cw = (n + S - 1) / S;
  const int lane = threadIdx.x & 31, grp = lane / S, seg = lane - grp * S;
  const int r = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * gpw + grp;
  const bool live = grp < gpw && r < n;
  double p = 0.0;
  if (live) {
    const int j0 = min(n, seg * cw), j1 = min(n, j0 + cw);
    p = seg_dot(j0, j1, [&](int j, double acc) { return fma(At[(size_t)j * n + r], x[j], acc); });
  }
  p = seg_tree(p, seg, S);
  if (live && seg == 0) y[r] = p;
}

// Column c of the precompute: unit vorticity at band vertex c (the previous one cleared),
// and the row range of the forward transform (the one nonzero row).
__global__ void k_inf_unit(int c, const int2* __restrict__ tiles, GridDims g, double* vort, int* prev, int* rr_in) {
  IB_GRID_DEP_WAIT();
  if (threadIdx.x != 0) return;
  const int p = *prev;
  if (p >= 0) vort[p] = 0.0;
  const int2 tc = tiles[c / kP];
  const int q = c % kP;
  const int a = tc.x * kT + (q % kT), b = tc.y * kT + q / kT;
  if (a < g.nsx && b < g.nsy) {
    const int o = b * g.nsx + a;
    vort[o] = 1.0;
    *prev = o;
    rr_in[0] = b;
    rr_in[1] = b + 1;
  } else {
    *prev = -1;
    rr_in[0] = 0;
    rr_in[1] = 1;
  }
  rr_in[2] = ROW_ZERO;
}

// The band build's column loops: set i starts at column i and steps by the number of sets.
__global__ void k_inf_col_init(int* col, int c0) {
  IB_GRID_DEP_WAIT();
  if (threadIdx.x == 0) *col = c0;
}
// Unit vector of the column *col (k_inf_unit with the column read on the device).
// Also the rows of each level that hold data: ainv's response on rows b -+ R (the rest below
// 1e-18 of it, written as zeros), and on each coarser level the rows coarsify fills from the
// finer level's data rows (coarse row n/4 + (r-1)/2 from the odd fine rows r in [1, n-3]
// whose 3-row stencil meets them); the other rows of a coarse level are zero apart from the
// ring's first and last samples (closed form), except its two edge rows, which are transformed.
__global__ void k_inf_unit_at(const int* col, const int2* __restrict__ tiles, GridDims g, double* vort, int* prev,
                              int* rr_in, int* rr_lv, int* box, int L, int R) {
  IB_GRID_DEP_WAIT();
  if (threadIdx.x != 0) return;
  const int c = *col;
  const int p = *prev;
  if (p >= 0) vort[p] = 0.0;
  const int2 tc = tiles[c / kP];
  const int q = c % kP;
  const int a = tc.x * kT + (q % kT), b = tc.y * kT + q / kT;
  int lo = 0, hi = 0;
  if (a < g.nsx && b < g.nsy) {
    const int o = b * g.nsx + a;
    vort[o] = 1.0;
    *prev = o;
    rr_in[0] = b;
    rr_in[1] = b + 1;
    lo = max(0, b - R);
    hi = min(g.nsy, b + R + 1);
    box[0] = max(0, a - R);
    box[1] = min(g.nsx - 1, a + R);
  } else {
    *prev = -1;
    rr_in[0] = 0;
    rr_in[1] = 1;
    box[0] = 0;
    box[1] = -1;
  }
  box[2] = lo;
  box[3] = hi - 1;
  rr_in[2] = ROW_ZERO;
  rr_lv[0] = lo; rr_lv[1] = hi; rr_lv[2] = ROW_ZERO;
  for (int l = 1; l < L; ++l) {
    int r0 = max(1, lo - 1), r1 = min(g.n - 3, hi);
    if ((r0 & 1) == 0) r0 += 1;
    if ((r1 & 1) == 0) r1 -= 1;
    if (lo >= hi || r0 > r1) { lo = 0; hi = 0; }
    else { lo = g.n / 4 + (r0 - 1) / 2; hi = g.n / 4 + (r1 - 1) / 2 + 1; }
    rr_lv[3 * l] = lo; rr_lv[3 * l + 1] = hi;
    rr_lv[3 * l + 2] = l == L - 1 ? ROW_ZERO : ROW_EDGES;
  }
}
// The band column *col's rows (k_inf_unit_at's rr_lv for the finest level and box) without a
// unit vector: the strip kernel below forms ainv's modes of it directly.  strip[0..1] = its
// vertex (a, b); strip[2..3] = the rows the previous column's strip occupied.
__global__ void k_inf_strip_rows_at(const int* col, const int2* __restrict__ tiles, GridDims g, int* strip,
                                    int* rr_lv, int* box, int L, int R) {
  IB_GRID_DEP_WAIT();
  if (threadIdx.x != 0) return;
  const int c = *col;
  const int2 tc = tiles[c / kP];
  const int q = c % kP;
  const int a = tc.x * kT + (q % kT), b = tc.y * kT + q / kT;
  strip[2] = rr_lv[0];
  strip[3] = rr_lv[1];
  int lo = 0, hi = 0;
  if (a < g.nsx && b < g.nsy) {
    lo = max(0, b - R);
    hi = min(g.nsy, b + R + 1);
    box[0] = max(0, a - R);
    box[1] = min(g.nsx - 1, a + R);
  } else {
    box[0] = 0;
    box[1] = -1;
  }
  box[2] = lo;
  box[3] = hi - 1;
  strip[0] = a;
  strip[1] = b;
  rr_lv[0] = lo; rr_lv[1] = hi; rr_lv[2] = ROW_ZERO;
  for (int l = 1; l < L; ++l) {   // the coarse levels' rows, as k_inf_unit_at
    int r0 = max(1, lo - 1), r1 = min(g.n - 3, hi);
    if ((r0 & 1) == 0) r0 += 1;
    if ((r1 & 1) == 0) r1 -= 1;
    if (lo >= hi || r0 > r1) { lo = 0; hi = 0; }
    else { lo = g.n / 4 + (r0 - 1) / 2; hi = g.n / 4 + (r1 - 1) / 2 + 1; }
    rr_lv[3 * l] = lo; rr_lv[3 * l + 1] = hi;
    rr_lv[3 * l + 2] = l == L - 1 ? ROW_ZERO : ROW_EDGES;
  }
}

// ainv's modes of a unit vector at band vertex (a, b): the forward transform of the unit vector
// is row a of the DST matrix W on row b, and ainv acts per mode, so on row y of the strip
// specY[y][k] = W[a][k] A_b[y][k], A_b the tabulated response to the unit row.  The previous
// strip's rows outside this one are cleared (specY is zero outside the current strip).
// Grid: x over the modes, y over 2 (2R+1) row slots (the new strip's, then the old one's).
__global__ void k_inf_strip(const int* __restrict__ strip, const int* __restrict__ rr_lv, GridDims g,
                            const double* __restrict__ W, const double* __restrict__ A, int r0, int R,
                            double* __restrict__ specY) {
  IB_GRID_DEP_WAIT();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.nsx) return;
  const int lo = rr_lv[0], hi = rr_lv[1];
  const int sl = blockIdx.y, w = 2 * R + 1;
  if (sl < w) {
    const int y = lo + sl;
    if (y >= hi) return;
    const int a = strip[0], b = strip[1];
    const double* Ab = A + ((size_t)(b - r0) * w + (y - (b - R))) * g.nsx;
    specY[(size_t)y * g.nsx + k] = W[(size_t)a * g.nsx + k] * Ab[k];
  } else {
    const int y = strip[2] + (sl - w);
    if (y < 0 || y >= strip[3] || (y >= lo && y < hi)) return;
    specY[(size_t)y * g.nsx + k] = 0.0;
  }
}

// The unit row r (every mode 1 on row r of a zeroed field) for the strip table.
__global__ void k_inf_unit_row(GridDims g, int r, double* f) {
  IB_GRID_DEP_WAIT();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < g.nsx) f[(size_t)r * g.nsx + k] = 1.0;
}

// K[*col][v] (k_inf_gather with the column read on the device).
__global__ void k_inf_gather_at(const int* col, int nR, const int2* __restrict__ tiles, GridDims g,
                                const double* __restrict__ s, double* __restrict__ K) {
  IB_GRID_DEP_WAIT();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nR) return;
  const int c = *col;
  const int2 tc = tiles[i / kP];
  const int q = i % kP;
  const int a = tc.x * kT + (q % kT), b = tc.y * kT + q / kT;
  K[(size_t)c * nR + i] = (a < g.nsx && b < g.nsy) ? s[b * g.nsx + a] : 0.0;
}
// Next column of this set; the loop continues while one is left.
__global__ void k_inf_col_next(int* col, int stride, int nR, cudaGraphConditionalHandle h) {
  IB_GRID_DEP_WAIT();
  if (threadIdx.x != 0) return;
  const int c = *col + stride;
  *col = c;
  cudaGraphSetConditional(h, c < nR ? 1u : 0u);
}

// Clears a scratch set's unit vector after a build (prev = -1: nothing set).
__global__ void k_inf_clear_unit(double* vort, int* prev) {
  IB_GRID_DEP_WAIT();
  if (threadIdx.x != 0) return;
  const int p = *prev;
  if (p >= 0) vort[p] = 0.0;
  *prev = -1;
}

// K[c][v] = s(band vertex v) for every band vertex (0 for tile vertices outside the grid).
__global__ void k_inf_gather(int c, int nR, const int2* __restrict__ tiles, GridDims g, const double* __restrict__ s,
                             double* __restrict__ K) {
  IB_GRID_DEP_WAIT();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nR) return;
  const int2 tc = tiles[i / kP];
  const int q = i % kP;
  const int a = tc.x * kT + (q % kT), b = tc.y * kT + q / kT;
  K[(size_t)c * nR + i] = (a < g.nsx && b < g.nsy) ? s[b * g.nsx + a] : 0.0;
}

// Room for the strips of n rows (false: not available, the columns transform and solve ainv
// themselves).
bool inf_strip_alloc(Ctx* c, int n) {
  Influence& I = c->inf;
  const size_t need = (size_t)n * (2 * I.trunc_rows + 1) * c->g.nsx;
  size_t freeb = 0, totalb = 0;
  if (cudaMemGetInfo(&freeb, &totalb) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (need > I.strip_cap && 8 * need < freeb / 8) {
    if (I.strips) cudaFree(I.strips);
    I.strips = nullptr;
    I.strip_cap = 0;
    if (cudaMalloc(&I.strips, 8 * need) == cudaSuccess) I.strip_cap = need;
    else cudaGetLastError();
  }
  return need <= I.strip_cap;
}

// ainv's response to a unit row r (every x mode 1 on row r), rows r - trunc_rows .. r + trunc_rows,
// for r = r_lo .. r_hi, into the strips; then every scratch set's ainv modes are cleared, with no
// strip recorded (the strip kernels clear only the rows they wrote last).
int inf_strip_table(Ctx* c, int r_lo, int r_hi) {
  Influence& I = c->inf;
  const GridDims& g = c->g;
  const int R = I.trunc_rows, wrows = 2 * R + 1;
  cudaStream_t st = c->st;
  I.strip_r0 = r_lo;
  I.strip_n = r_hi - r_lo + 1;
  double* F = I.bscr[0].spec1;
  for (int r = r_lo; r <= r_hi; ++r) {
    IB_CUDA_CHECK(cudaMemsetAsync(F, 0, 8 * (size_t)g.ns, st));
    count_launch();
    k_inf_unit_row<<<cdiv(g.nsx, 256), 256, 0, st>>>(g, r, F);
    RC(tri_solve(c->tri_ainv, F, F, g.nsx, c->tl, st));
    const int lo = std::max(0, r - R), hi = std::min(g.nsy, r + R + 1);
    IB_CUDA_CHECK(cudaMemcpyAsync(I.strips + ((size_t)(r - r_lo) * wrows + (lo - (r - R))) * g.nsx,
                                  F + (size_t)lo * g.nsx, 8 * (size_t)(hi - lo) * g.nsx, cudaMemcpyDeviceToDevice,
                                  st));
  }
  for (const SchurScratch& sc : I.bscr) {
    IB_CUDA_CHECK(cudaMemsetAsync(sc.specY, 0, 8 * (size_t)g.ns, st));
    IB_CUDA_CHECK(cudaMemsetAsync(sc.rr_lv, 0, 2 * sizeof(int), st));
  }
  return IB_OK;
}

int inf_alloc(Ctx* c) {
  Influence& I = c->inf;
  const int nf = std::max(c->nf, 1);
  IB_CUDA_CHECK(cudaMalloc(&I.pval, sizeof(double) * (size_t)nf * kP));
  IB_CUDA_CHECK(cudaMalloc(&I.pidx, sizeof(int) * (size_t)nf * kP));
  IB_CUDA_CHECK(cudaMalloc(&I.S, sizeof(double) * (size_t)nf * nf));
  IB_CUDA_CHECK(cudaMalloc(&I.St, sizeof(double) * (size_t)nf * nf));
  IB_CUDA_CHECK(cudaMalloc(&I.brv, sizeof(double) * (size_t)nf));
  IB_CUDA_CHECK(cudaMalloc(&I.bco, sizeof(double) * (size_t)nf));
  IB_CUDA_CHECK(cudaMalloc(&I.bod, sizeof(int) * (size_t)nf));
  IB_CUDA_CHECK(cudaMalloc(&I.flag, sizeof(int) * 16));
  I.nu = I.flag + 4;
  I.rr_in = I.flag + 8;
  I.rr_out = I.flag + 12;
  IB_CUDA_CHECK(cudaMemset(I.flag, 0, sizeof(int) * 16));
  IB_CUDA_CHECK(cudaHostAlloc(&I.h_flag, sizeof(int) * 2, cudaHostAllocDefault));
  I.ntx = cdiv(c->g.nsx, kT);
  I.nty = cdiv(c->g.nsy, kT);
  IB_CUDA_CHECK(cudaMalloc(&I.tile_of, sizeof(int) * (size_t)I.ntx * I.nty));
  return IB_OK;
}

static void free_band(Influence& I) {
  if (I.strips) cudaFree(I.strips);
  I.strips = nullptr;
  I.strip_cap = 0;
  if (I.K) cudaFree(I.K);
  if (I.used) cudaFree(I.used);
  if (I.ulist) cudaFree(I.ulist);
  if (I.upos) cudaFree(I.upos);
  if (I.T) cudaFree(I.T);
  if (I.tiles) cudaFree(I.tiles);
  I.K = nullptr; I.used = I.ulist = I.upos = nullptr; I.T = nullptr; I.tiles = nullptr;
  I.capK = I.capR = 0;
}

// The band build's scratch sets and streams (made on the first build, kept for rebuilds; the
// sub-domain precompute runs its columns on the same sets).
int inf_build_scratch(Ctx* c) {
  Influence& I = c->inf;
  if (!I.bscr.empty()) return IB_OK;
  const GridDims& g = c->g;
  const int S = Influence::kBuildStreams, L = c->L;
  const size_t ns = g.ns, per = (size_t)(4 + L) * ns + (size_t)g.nbc;
  IB_CUDA_CHECK(cudaMalloc(&I.bmem, 8 * per * S));
  IB_CUDA_CHECK(cudaMalloc(&I.bint, sizeof(int) * Influence::kSetInts * S));
  // zero: the unit vectors start from an empty field, and the coarse levels' vorticity stays
  // zero outside the centres coarsify writes
  IB_CUDA_CHECK(cudaMemset(I.bmem, 0, 8 * per * S));
  IB_CUDA_CHECK(cudaMemset(I.bint, 0xff, sizeof(int) * Influence::kSetInts * S));   // prev = -1
  // ainv's response to a unit vector on row b, (1/c1 + lam_x + T_y)^-1 per x mode, decays
  // away from row b at least as fast as rho^|r-b| with rho + 1/rho = 2 + 1/c1 (the slowest
  // mode, lam_x -> 0); past trunc_rows rows it is below 1e-18 of its peak.  Only the input of
  // the coarse levels' chain is cut there (the finest level keeps the exact modes), so the
  // band's columns change at the 1e-18 level.
  {
    const double a = 2.0 + 1.0 / c->cvis[0];
    const double rho = 0.5 * (a - std::sqrt(a * a - 4.0));
    int R = g.nsy;
    if (rho > 0.0 && rho < 1.0) R = (int)std::ceil(18.0 * std::log(10.0) / -std::log(rho)) + 2;
    I.trunc_rows = std::min(R, g.nsy);
  }
  I.bscr.resize(S);
  for (int i = 0; i < S; ++i) {
    SchurScratch& sc = I.bscr[i];
    double* b = I.bmem + per * i;
    sc.vort = b; sc.specY = b + ns; sc.spec1 = b + 2 * ns; sc.s0 = b + 3 * ns;
    for (int k = 0; k < L; ++k) sc.w[k] = b + (4 + k) * ns;
    sc.sbc = b + (4 + L) * ns;
    sc.prev = I.bint + Influence::kSetInts * i;
    sc.rr_in = sc.prev + 1;
    sc.box = sc.prev + 8;
    sc.strip = sc.prev + 12;
    sc.rr_lv = sc.prev + 16;
    if (cudaStreamCreateWithFlags(&sc.st, cudaStreamNonBlocking) != cudaSuccess) {
      sc.st = nullptr;
      return IB_ERR_CUDA;
    }
  }
  return IB_OK;
}

void inf_free(Ctx* c) {
  Influence& I = c->inf;
  for (SchurScratch& sc : I.bscr)
    if (sc.st) cudaStreamDestroy(sc.st);
  if (I.bmem) cudaFree(I.bmem);
  if (I.bint) cudaFree(I.bint);
  cr_free(c);
  free_band(I);
  if (I.pval) cudaFree(I.pval);
  if (I.pidx) cudaFree(I.pidx);
  if (I.S) cudaFree(I.S);
  if (I.St) cudaFree(I.St);
  if (I.brv) cudaFree(I.brv);
  if (I.bco) cudaFree(I.bco);
  if (I.bod) cudaFree(I.bod);
  if (I.flag) cudaFree(I.flag);
  if (I.tile_of) cudaFree(I.tile_of);
  if (I.h_flag) cudaFreeHost(I.h_flag);
  I = Influence{};
}

int inf_patch(Ctx* c, bool cleared) {
  Influence& I = c->inf;
  if (c->nf == 0) return IB_OK;
  if (!cleared) {
    IB_CUDA_CHECK(cudaMemsetAsync(I.flag, 0, sizeof(int), c->st));
    if (I.built) IB_CUDA_CHECK(cudaMemsetAsync(I.used, 0, sizeof(int) * (size_t)I.nR, c->st));
  }
  count_launch();
  k_inf_patch<<<c->nf, kP, 0, c->st>>>(c->g, c->nf, c->reg.comp, c->reg.ix, c->reg.iy, c->reg.w,
                                       I.built ? I.tile_of : nullptr, I.ntx, I.pval, I.pidx, I.used, I.flag);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

static int read_flag(Ctx* c) {
  Influence& I = c->inf;
  IB_CUDA_CHECK(cudaMemcpyAsync(I.h_flag, I.flag, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  IB_CUDA_CHECK(cudaStreamSynchronize(c->st));
  I.flag_h = I.h_flag[0];
  I.patch_fresh = true;
  return IB_OK;
}

// The band: every tile within `margin` vertices of some unknown's patch.  Then one
// matrix-free application of the fluid part per band vertex fills K.
int inf_build(Ctx* c) {
  Influence& I = c->inf;
  const GridDims& g = c->g;
  const int nf = c->nf;
  auto t0 = std::chrono::steady_clock::now();
  std::vector<int> ix(nf), iy(nf);
  IB_CUDA_CHECK(cudaStreamSynchronize(c->st));
  IB_CUDA_CHECK(cudaMemcpy(ix.data(), c->reg.ix, sizeof(int) * nf, cudaMemcpyDeviceToHost));
  IB_CUDA_CHECK(cudaMemcpy(iy.data(), c->reg.iy, sizeof(int) * nf, cudaMemcpyDeviceToHost));
  const int M = c->p.influence_margin > 0 ? c->p.influence_margin : 8;
  std::vector<int> tile_of((size_t)I.ntx * I.nty, -1);
  std::vector<char> mark((size_t)I.ntx * I.nty, 0);
  for (int k = 0; k < nf; ++k) {
    int a0 = std::max(0, ix[k] - 5 - M), a1 = std::min(g.nsx - 1, ix[k] + 2 + M);
    int b0 = std::max(0, iy[k] - 5 - M), b1 = std::min(g.nsy - 1, iy[k] + 2 + M);
    if (a0 > a1 || b0 > b1) continue;
    for (int tb = b0 / kT; tb <= b1 / kT; ++tb)
      for (int ta = a0 / kT; ta <= a1 / kT; ++ta) mark[(size_t)tb * I.ntx + ta] = 1;
  }
  I.tiles_h.clear();
  int bmin = g.nsy, bmax = -1;
  for (int tb = 0; tb < I.nty; ++tb)
    for (int ta = 0; ta < I.ntx; ++ta)
      if (mark[(size_t)tb * I.ntx + ta]) {
        tile_of[(size_t)tb * I.ntx + ta] = (int)I.tiles_h.size();
        I.tiles_h.push_back(make_int2(ta, tb));
        bmin = std::min(bmin, tb * kT);
        bmax = std::max(bmax, std::min(g.nsy - 1, tb * kT + kT - 1));
      }
  I.ntile = (int)I.tiles_h.size();
  I.nR = I.ntile * kP;
  I.built = false;
  // the captured FSI phases bake in the band's buffers and size
  drop_phase(&c->graph_fsi_asm);
  drop_phase(&c->graph_fsi_upd);
  drop_phase(&c->graph_fsi_loop);
  drop_phase(&c->graph_step);
  I.active = false;
  if (I.nR == 0) return IB_ERR_STATE;
  const size_t nK = (size_t)I.nR * I.nR;
  if (nK > I.capK || (size_t)I.nR > I.capR) {
    free_band(I);
    size_t freeb = 0, totalb = 0;
    IB_CUDA_CHECK(cudaMemGetInfo(&freeb, &totalb));
    const size_t need = 8 * nK + (size_t)I.nR * (12 + 8 * (size_t)std::max(nf, 1)) + 8 * (size_t)I.ntile;
    if (need > freeb / 2) return IB_ERR_NOMEM;   // leave the rest of HBM to the caller
    IB_CUDA_CHECK(cudaMalloc(&I.K, 8 * nK));
    IB_CUDA_CHECK(cudaMalloc(&I.used, sizeof(int) * I.nR));
    IB_CUDA_CHECK(cudaMalloc(&I.ulist, sizeof(int) * I.nR));
    IB_CUDA_CHECK(cudaMalloc(&I.upos, sizeof(int) * I.nR));
    IB_CUDA_CHECK(cudaMalloc(&I.T, sizeof(double) * (size_t)I.nR * std::max(nf, 1)));
    I.capK = nK;
    I.capR = I.nR;
  }
  if (I.tiles) cudaFree(I.tiles);
  IB_CUDA_CHECK(cudaMalloc(&I.tiles, sizeof(int2) * I.ntile));
  IB_CUDA_CHECK(cudaMemcpy(I.tiles, I.tiles_h.data(), sizeof(int2) * I.ntile, cudaMemcpyHostToDevice));
  IB_CUDA_CHECK(cudaMemcpy(I.tile_of, tile_of.data(), sizeof(int) * tile_of.size(), cudaMemcpyHostToDevice));
  const int rr_out_h[3] = {bmin, bmax + 1, ROW_SKIP};
  IB_CUDA_CHECK(cudaMemcpy(I.rr_out, rr_out_h, sizeof(rr_out_h), cudaMemcpyHostToDevice));
  // columns: unit vorticity at each band vertex through the fluid part of the operator.  The
  // columns are independent, and each is a chain of small latency-bound launches: they run on
  // kBuildStreams streams at once, column col on set col % kBuildStreams (its own unit
  // vector, scratch fields and output rows), after the work already on the context's stream.
  // Each set's columns run as one captured graph: a while node whose body is one column with
  // the column index on the device, so the host launches one graph per set.
  RC(inf_build_scratch(c));
  // the coarse levels' responses for the level-1 vertices these columns reach (coarse.cu);
  // without them (memory, or switched off) each column runs the coarse chain itself
  bool use_cr = false;
  if (c->L > 1 && I.cr.enabled) {
    std::vector<unsigned char> mask(g.ns, 0);
    for (const int2& t : I.tiles_h)
      for (int q = 0; q < kP; ++q) {
        const int a = t.x * kT + (q % kT), b = t.y * kT + q / kT;
        if (a < g.nsx && b < g.nsy) mask[(size_t)b * g.nsx + a] = 1;
      }
    cr_dilate(g, mask, I.trunc_rows);
    use_cr = cr_prepare(c, mask) == IB_OK;   // else each column runs the coarse chain itself
    cudaGetLastError();
  }
  for (SchurScratch& sc : I.bscr) {
    sc.cr_R1 = use_cr ? I.cr.R[1] : nullptr;
    sc.cr_idx1 = use_cr ? I.cr.idx[1] : nullptr;
  }
  cudaStream_t st = c->st;
  // ainv's response to a unit row, for every band row (the strips the columns scale by their row
  // of W instead of transforming a unit vector and solving ainv each)
  const int R = I.trunc_rows, wrows = 2 * R + 1;
  const bool use_strips = inf_strip_alloc(c, bmax - bmin + 1);
  if (use_strips) RC(inf_strip_table(c, bmin, bmax));
  for (SchurScratch& sc : I.bscr) sc.specY_ready = use_strips;
  const int S = std::min(Influence::kBuildStreams, I.nR);
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
    int* col = sc.prev + 4;   // the set's fifth int (after prev and rr_in)
    cudaGraph_t graph = nullptr;
    do {
      if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeRelaxed) != cudaSuccess) { rc = IB_ERR_CUDA; break; }
      count_launch();
      k_inf_col_init<<<1, 32, 0, cap>>>(col, i);
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
        if (use_strips) {
          count_launches(2);
          k_inf_strip_rows_at<<<1, 32, 0, sc.st>>>(col, I.tiles, g, sc.strip, sc.rr_lv, sc.box, c->L, R);
          k_inf_strip<<<dim3(cdiv(g.nsx, 128), 2 * wrows), 128, 0, sc.st>>>(sc.strip, sc.rr_lv, g, c->wmat,
                                                                           I.strips, I.strip_r0, R, sc.specY);
        } else {
          count_launch();
          k_inf_unit_at<<<1, 32, 0, sc.st>>>(col, I.tiles, g, sc.vort, sc.prev, sc.rr_in, sc.rr_lv, sc.box, c->L,
                                             I.trunc_rows);
        }
        const double* ring0 = nullptr;
        rc = schur_fluid(c, sc.vort, sc.rr_in, I.rr_out, sc.s0, &ring0, &sc);
        count_launches(2);
        k_inf_gather_at<<<cdiv(I.nR, 256), 256, 0, sc.st>>>(col, I.nR, I.tiles, g, sc.s0, I.K);
        k_inf_col_next<<<1, 32, 0, sc.st>>>(col, S, I.nR, h);
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
    if (rc == IB_OK) count_launches(S + (long long)I.nR * body_launches);
  } else {
    // capture unavailable: the same columns launched one by one from the host
    rc = IB_OK;
    for (int col = 0; col < I.nR && rc == IB_OK; ++col) {
      SchurScratch sc = I.bscr[col % S];
      sc.rr_lv = nullptr;   // every row transformed
      sc.cr_R1 = nullptr;   // and the coarse chain run per column
      sc.specY_ready = false;
      count_launch();
      k_inf_unit<<<1, 32, 0, sc.st>>>(col, I.tiles, g, sc.vort, sc.prev, sc.rr_in);
      const double* ring0 = nullptr;
      rc = schur_fluid(c, sc.vort, sc.rr_in, I.rr_out, sc.s0, &ring0, &sc);
      if (rc != IB_OK) break;
      count_launch();
      k_inf_gather<<<cdiv(I.nR, 256), 256, 0, sc.st>>>(col, I.nR, I.tiles, g, sc.s0, I.K);
      if (cudaGetLastError() != cudaSuccess) rc = IB_ERR_CUDA;
    }
  }
  c->prof_on = prof;
  // the context's stream continues after every column; the sets' unit vectors are cleared
  // for the next build
  for (int i = 0; i < S; ++i) {
    const SchurScratch& sc = I.bscr[i];
    count_launch();
    k_inf_clear_unit<<<1, 32, 0, sc.st>>>(sc.vort, sc.prev);
    cudaEventRecord(ev, sc.st);
    cudaStreamWaitEvent(st, ev, 0);
  }
  for (int i = 0; i < S; ++i) cudaStreamSynchronize(I.bscr[i].st);
  for (cudaGraphExec_t e : execs)
    if (e) cudaGraphExecDestroy(e);
  if (cap) cudaStreamDestroy(cap);
  cudaEventDestroy(ev);
  for (SchurScratch& sc : I.bscr) {
    sc.cr_R1 = nullptr;
    sc.specY_ready = false;
  }
  RC(rc);
  IB_CUDA_CHECK(cudaStreamSynchronize(st));
  if (use_cr) {
    int err = 0;
    IB_CUDA_CHECK(cudaMemcpy(&err, I.cr.err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) return IB_ERR_STATE;   // a column met a vertex without a response
  }
  I.columns += I.nR;
  I.builds += 1;
  I.built = true;
  I.patch_fresh = false;
  I.build_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return IB_OK;
}

int inf_prepare(Ctx* c) {
  Influence& I = c->inf;
  I.active = false;
  if (c->p.schur_mode == 1 || c->nf == 0) return IB_OK;
  if (!I.patch_fresh) {
    RC(inf_patch(c));
    RC(read_flag(c));
  }
  if (I.flag_h & 2) { I.fallbacks += 1; return IB_OK; }
  if (!I.built || (I.flag_h & 1)) {
    int rc = inf_build(c);
    if (rc == IB_ERR_NOMEM || rc == IB_ERR_STATE) { I.fallbacks += 1; return IB_OK; }
    RC(rc);
    RC(inf_patch(c));
    RC(read_flag(c));
    if (I.flag_h) { I.fallbacks += 1; return IB_OK; }
  }
  RC(inf_assemble(c));
  I.assemblies += 1;
  I.active = true;
  return IB_OK;
}

// The assembly kernels alone (no host decisions): S, St from K and the current patches.
int inf_assemble_kp(Ctx* c, cudaStream_t st, bool clear_used) {
  Influence& I = c->inf;
  count_launch();
  k_inf_compact<<<1, 1024, 0, st>>>(I.nR, I.used, I.ulist, I.upos, I.nu, clear_used ? 1 : 0);
  count_launch();
  // the touched vertices are typically a fifth of the band: a quarter of its blocks, striding
  k_inf_kp<<<dim3(std::max(1, cdiv(I.nR, 128) / 4), c->nf), 128, 0, st>>>(I.nR, I.K, I.pval, I.pidx, I.ulist, I.nu,
                                                                        I.T);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

int inf_assemble_b(Ctx* c, cudaStream_t st) {
  Influence& I = c->inf;
  // -1: no B term (unknowns of rigid bodies; k_inf_bvec sets every torsional body's own)
  if (c->nt < c->nbody) IB_CUDA_CHECK(cudaMemsetAsync(I.bod, 0xff, sizeof(int) * (size_t)c->nf, st));
  if (c->nt > 0) {
    count_launch();
    k_inf_bvec<<<c->nt, 32, 0, st>>>(c->tb, c->ts, c->p.dt, c->delta, I.brv, I.bco, I.bod);
  }
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

int inf_assemble_ptk(Ctx* c, cudaStream_t st) {
  Influence& I = c->inf;
  count_launch();
  k_inf_ptk<<<c->nf, 128, 0, st>>>(c->nf, I.nR, I.pval, I.pidx, I.upos, I.T, I.brv, I.bco, I.bod, I.S, I.St);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

int inf_assemble(Ctx* c) {
  RC(inf_assemble_kp(c, c->st, false));
  RC(inf_assemble_b(c, c->st));
  RC(inf_assemble_ptk(c, c->st));
  return launch_beam_add_b(c, c->inf.St, c->st);   // the beams' dense blocks of B
}

// y = (S + B) x from the assembled column-major operator (B is part of it).
int inf_dense_mv(Ctx* c, const double* x, double* y) {
  c->n_matvec += 1;
  count_launch();
  const int gpw = 32 / mv_segments(c->nf);
  k_dense_mv<<<cdiv(32LL * cdiv(c->nf, gpw), 128), 128, 0, c->st>>>(c->nf, c->inf.St, x, y);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

}  // namespace ib
