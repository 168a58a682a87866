// Batched DST-I (FFTW RODFT00 semantics) for the spectral Poisson and
// Crank-Nicolson solves of myfft.F90:161-216.
//
// Y_k = 2 sum_{j=1}^{N} x_j sin(pi j k / M),  k = 1..N,  M = N+1 (unnormalised).
//
// One line of length N is transformed through a complex FFT of length P = M/2:
//   y_j = sin(j pi/M)(x_j + x_{M-j}) + (x_j - x_{M-j})/2,     y_0 = 0
//   Z   = FFT_P(y_0 + i y_1, y_2 + i y_3, ...)
//   2Y  = unpacked real FFT of y (length M)
//   D_{2k}   = -Im(2Y_k),      D_1 = Re(Y_0),   D_{2k+1} = D_{2k-1} + Re(2Y_k)
// (the classic odd-extension sine transform; the odd outputs are a prefix sum).
// The complex FFT is a Stockham auto-sort with radices 2, 3, 4 and 5 run in
// shared memory over all (line, butterfly) items of a CTA.
#pragma once
#include "ib_common.cuh"

namespace ib {

constexpr int kMaxRadices = 16;
constexpr int kMaxBatch = 16;   // levels one batched x pass can carry

// sum_k sr[k] wc[k] over k < N on one warp (the lane's partial sums, not yet reduced): four
// accumulators (k = lane + 32(4t + a)) keep four loads per operand in flight.  warp_sum then
// adds the lanes' values (the same butterfly order on every lane).
__device__ __forceinline__ double warp_dot_part(const double* __restrict__ sr, const double* __restrict__ wc, int N,
                                                int lane) {
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  int k = lane;
  for (; k + 96 < N; k += 128) {
    a0 = fma(sr[k], wc[k], a0);
    a1 = fma(sr[k + 32], wc[k + 32], a1);
    a2 = fma(sr[k + 64], wc[k + 64], a2);
    a3 = fma(sr[k + 96], wc[k + 96], a3);
  }
  if (k < N) a0 = fma(sr[k], wc[k], a0);
  if (k + 32 < N) a1 = fma(sr[k + 32], wc[k + 32], a1);
  if (k + 64 < N) a2 = fma(sr[k + 64], wc[k + 64], a2);
  return (a0 + a1) + (a2 + a3);
}

__device__ __forceinline__ double warp_sum(double acc) {
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  return acc;
}

// A mode row's inverse x transform at a point and at its mirror image.  W's row N-1-r is
// (-1)^k times row r in mode k, so the two values are e + o and e - o, with e and o the row's
// sums over even and odd modes.  A lane of warp_dot_part meets only modes of its own parity,
// so reducing the lanes within each parity gives both at the cost of one dot product.
// Returns (e + o, e - o) on every lane.
__device__ __forceinline__ double2 warp_sum_mirror(double acc) {
  for (int o = 16; o > 1; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  const double other = __shfl_xor_sync(0xffffffffu, acc, 1);
  const bool odd = threadIdx.x & 1;
  const double e = odd ? other : acc, o = odd ? acc : other;
  return make_double2(e + o, e - o);
}

// (E s0)_k and (E s1)_k from the parity-compact edge matrix (dst_edge_matrix: row k holds
// E[k][2t + (k & 1)], t < (N+1)/2), for two mode rows at once; lane-strided in t, two chains,
// then the warp's sums.
__device__ __forceinline__ double2 warp_edge_dot(const double* __restrict__ Ec, int N, int k,
                                                 const double* __restrict__ s0, const double* __restrict__ s1,
                                                 int lane) {
  const int Nh = (N + 1) / 2, pk = k & 1, nk = pk ? N / 2 : Nh;
  const double* ek = Ec + (size_t)k * Nh;
  s0 += pk;
  s1 += pk;
  double a0 = 0.0, a1 = 0.0, b0 = 0.0, b1 = 0.0;
  int t = lane;
  for (; t + 32 < nk; t += 64) {
    const double e0 = ek[t], e1 = ek[t + 32];
    a0 = fma(e0, s0[2 * t], a0);
    b0 = fma(e0, s1[2 * t], b0);
    a1 = fma(e1, s0[2 * t + 64], a1);
    b1 = fma(e1, s1[2 * t + 64], b1);
  }
  if (t < nk) {
    a0 = fma(ek[t], s0[2 * t], a0);
    b0 = fma(ek[t], s1[2 * t], b0);
  }
  return make_double2(warp_sum(a0 + a1), warp_sum(b0 + b1));
}

struct DstPlan {
  int N = 0, M = 0, P = 0;
  int nrad = 0;
  int rad[kMaxRadices] = {0};
  double2* tw = nullptr;   // P entries: the Stockham stages' twiddles, stage by stage (dst.cu)
  double2* uw = nullptr;   // P/2 entries: exp(-2 pi i k / M)
  double* sn = nullptr;    // P+1 entries: sin(j pi / M)
};

// Launch geometry of one pass (chosen by the tuner in dst.cu).
struct DstLaunch {
  int B = 1;       // lines per CTA
  int NT = 128;    // threads per CTA
  int narrow_scan = 0;   // 1: one warp scans each line (fewer FP64 instructions); 0: all warps
};

int dst_plan_create(DstPlan* p, int N);   // N = M-1, M divisible by 4, M = 2^a 3^b 5^c
void dst_plan_destroy(DstPlan* p);
// Doubles of device memory the tables of a plan of length N occupy (0 if N is unsupported).
size_t dst_plan_table_doubles(int N);
// Fills a plan's tables into caller-provided device memory (no allocation; the plan must not
// be passed to dst_plan_destroy).  dev must hold dst_plan_table_doubles(N) doubles, 16-byte aligned.
int dst_plan_init_external(DstPlan* p, int N, double* dev, cudaStream_t st);

enum DstPre { PRE_COPY = 0, PRE_COMBINE = 1, PRE_APPLYBC = 2, PRE_PRED = 3, PRE_ROT = 4 };
enum DstYMode { YMODE_NONE = 0 };

struct DstXArgs {
  const double* in = nullptr;    // nlines rows, row pitch ld
  const double* in2 = nullptr;   // PRE_COMBINE second operand
  const double* in3 = nullptr;   // PRE_COMBINE third operand
  const double* in4 = nullptr;   // PRE_PRED vorticity
  double ca = 1.0, cb = 0.0;     // PRE_COMBINE: ca*in + cb*in2 + in3
  double alpha = 0.0, beta = 0.0;  // PRE_PRED: + alpha*w + beta*(sum of the 4 neighbours of w)
  const double* ring = nullptr;  // PRE_APPLYBC boundary ring; PRE_PRED without in3: first rhsbc ring
  double fac = 1.0;              // PRE_APPLYBC factor; PRE_PRED without in3: rhsbc factor
  // PRE_PRED without in3: rhsbc (timestepper.F90:184-189) is formed on the fly from `ring`
  double* save = nullptr;        // PRE_PRED: receives a copy of `in` (may alias in2)
  // PRE_ROT: rot (operators_fluid.F90:203-233) of the face fields in (u-faces) and in2
  // (v-faces), read only inside the face box box[0..3] = i0, j0, ni, nj (zero outside)
  const int* box = nullptr;
  double* out = nullptr;         // nlines rows, pitch ld
  // optional output post-op: out = DST(row) + post_scale * post_add
  const double* post_add = nullptr;
  double post_scale = 0.0;
  // optional per-row treatment (ROW_*); rows not listed are transformed
  const unsigned char* rowmode = nullptr;
  int rowmode_level0 = 0;        // in a batch, levels below this transform every row
  double row_scale = 0.0;        // ROW_SCALE rows: row_scale * in2 (lin2[level])
  // optional device range [rr[0], rr[1]) of transformed rows; others get mode rr[2]
  const int* rowrange = nullptr;
  int row_margin = 0;            // rowrange widened by this many rows on each side (clamped)
  int fft_edge_rows = 0;         // with rowrange: rows 0 and nrows-1 are transformed as well
  int* rows_used = nullptr;      // receives the (widened) range of transformed rows
  // optional strided row subset: line i is row row0 + i*row_step, i < nlines (0: all rows)
  int nlines = 0, row0 = 0, row_step = 0;
  // optional batch over grid levels (PRE_COPY, PRE_PRED): level l (blockIdx.y) reads lin[l] and
  // writes lout[l], each a full field of pitch ld; in/out are then unused.  PRE_PRED takes every
  // other operand and coefficient of level l from the l-arrays below.
  int nlev = 0;
  const double* lin[kMaxBatch] = {};
  double* lout[kMaxBatch] = {};
  const double* lin2[kMaxBatch] = {};
  const double* lin4[kMaxBatch] = {};
  const double* lring[kMaxBatch] = {};
  double* lsave[kMaxBatch] = {};
  double lca[kMaxBatch] = {}, lcb[kMaxBatch] = {}, lalpha[kMaxBatch] = {}, lbeta[kMaxBatch] = {};
  double lfac[kMaxBatch] = {};
};

// Per-row treatment in the x pass.  ROW_EDGES: the row (after the pre-op) is zero
// except its first and last samples, whose transform is closed form:
// Y_k = 2 sin(pi k/M) (x_1 + (-1)^(k+1) x_N).  ROW_SCALE: the row's transform is known,
// row_scale times the same row of in2 (lin2 of the level in a batch): a row equal to the
// inverse transform S Y of modes Y has the transform S S Y = 2m Y.
enum RowMode { ROW_ZERO = 0, ROW_FFT = 1, ROW_EDGES = 2, ROW_SKIP = 3, ROW_SCALE = 4 };

struct DstYArgs {
  double* a = nullptr;           // field (in/out), rows of pitch ld
};

// x direction: lines are the (n-1) rows of an (n-1)x(m-1) field, N = m-1.
int dst_pass_x(const DstPlan& px, int nrows, int ld, DstPre pre, const DstXArgs& a,
               const GridDims& g, const DstLaunch& L, cudaStream_t st);
// y direction: lines are the (m-1) columns, N = n-1 (the plain 2-D DST only).
int dst_pass_y(const DstPlan& py, int ncols, int ld, DstYMode mode, const DstYArgs& a,
               const DstLaunch& L, cudaStream_t st);

size_t dst_smem_x(const DstPlan& p, int B);

// The DST-I matrix of the x transform, W[j][k] = 2 sin(pi (j+1)(k+1)/M), N x N (symmetric).
int dst_matrix_table(const DstPlan& px, double* dev_out);
// out = post_scale*post_add + S_x(apply_bc(ring)) on every row (factor 1, zero field): the two
// edge rows by dot products with W (fft_edges: by the FFT line transform, fewer FP64 instructions
// and a longer chain), the interior rows in closed form 2 sin(pi k/M)(x_1 + (-1)^(k+1) x_N) from
// sk2[k-1] = 2 sin(pi k/M) (dst_sin2_table).  In place allowed (out == post_add).
int dst_x_bc_modes(const DstPlan& px, const GridDims& g, const double* ring, const double* W, const double* sk2,
                   const double* post_add, double post_scale, double* out, cudaStream_t st,
                   bool fft_edges = false);
// ring = fac * get_bc of the inverse x transform of a coarser level's modes (spec, pitch ld),
// evaluated at the points get_bc reads only (dot products with W).
int dst_ring_from_modes(const DstPlan& px, const GridDims& g, const double* spec, int ld, const double* W, double fac,
                        double* ring, cudaStream_t st);
// The same ring, plus the boundary terms the finer level's solve adds to its right-hand side
// modes (tri_solve's TriBc): sd (2 x nsy) the sums and differences of the ring's left and right
// entries 1..n-1, edge (2 x N) the x transforms of its bottom and top entries 1..m-1, from the
// edge matrix E (dst_edge_matrix) and the coarse modes of the two rows get_bc reads.
int dst_ring_edge_from_modes(const DstPlan& px, const GridDims& g, const double* spec, int ld, const double* W,
                             const double* E, double fac, double* ring, double* sd, double* edge, cudaStream_t st);
// E = W P: P maps the coarse modes of one row to the get_bc values on entries 1..m-1 of a finer
// level's bottom or top side, so W P maps them to that side's x transform.  The side's points
// are symmetric about the centre column, so E[k][k'] vanishes unless k and k' have the same
// parity: only those entries are kept, row k holding E[k][2t + (k & 1)] for t < (N+1)/2 (zero
// past N-1), N x (N+1)/2 doubles.  Computed on the device at set-up (synchronous).
int dst_edge_matrix(const DstPlan& px, const GridDims& g, const double* W, double* E);
// sk2[k-1] = 2 sin(pi k/M), k = 1..N, into N doubles of device memory.
int dst_sin2_table(const DstPlan& px, double* dev_out);
size_t dst_smem_y(const DstPlan& p, int B, DstYMode mode);

}  // namespace ib
