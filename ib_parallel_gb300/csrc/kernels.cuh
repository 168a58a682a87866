// Launchers of the grid, interface and structure kernels.
#pragma once
#include "ib_common.cuh"

namespace ib {

// stencil.cu -- operators_fluid.F90
int launch_nonlinear(const GridDims& g, const double* om, const double* bc, const double* qx, const double* q0x,
                     const double* qy, const double* q0y, double* nlx, double* nly, cudaStream_t st);
int launch_rot(const GridDims& g, const double* hx, const double* hy, double* vort, cudaStream_t st);
int launch_curl(const GridDims& g, const double* s, const double* sbc, double* qx, double* qy, cudaStream_t st);
int launch_coarsify(const GridDims& g, const double* fine, double* coarse, cudaStream_t st);
int launch_get_bc(const GridDims& g, const double* s, double fac, double* ring, cudaStream_t st);
// Rings of every level in one launch: dst[l] = fac * get_bc(src[l]), zero where src[l] is null.
constexpr int kMaxLevels = 16;
struct RingBatch {
  const double* src[kMaxLevels] = {};
  double* dst[kMaxLevels] = {};
};
int launch_get_bc_levels(const GridDims& g, const RingBatch& rb, int nlev, double fac, cudaStream_t st);
// curl of every level in one launch: level l from s[l] with ghosts from the ring sbc[l]
// the frame fluxes of every level (k_frame_flux)
struct FrameLevels {
  double* q0x[kMaxLevels] = {};
  double* q0y[kMaxLevels] = {};
};
// lines: nlev (n + m) doubles of scratch
int launch_frame_flux(const GridDims& g, const FrameLevels& fl, int nlev, double delta, double offx, double offy,
                      double u, double v, double w, double cx, double cy, double* lines, cudaStream_t st);

struct CurlBatch {
  const double* s[kMaxLevels] = {};
  const double* sbc[kMaxLevels] = {};
  double* qx[kMaxLevels] = {};
  double* qy[kMaxLevels] = {};
};
int launch_curl_levels(const GridDims& g, const CurlBatch& cb, int nlev, cudaStream_t st);
// nonlinear terms then rot of every level (two launches): level l's nonlinear terms of om[l]
// (ghosts from the ring bc[l], fluxes q + q0) into the scratch nlx[l], nly[l], their rot into out[l]
struct NlBatch {
  const double* om[kMaxLevels] = {};
  const double* bc[kMaxLevels] = {};
  const double* qx[kMaxLevels] = {};
  const double* q0x[kMaxLevels] = {};
  const double* qy[kMaxLevels] = {};
  const double* q0y[kMaxLevels] = {};
  double* nlx[kMaxLevels] = {};
  double* nly[kMaxLevels] = {};
  double* out[kMaxLevels] = {};
};
int launch_nonlinear_rot_levels(const GridDims& g, const NlBatch& b, int nlev, cudaStream_t st);
// the same with the interior tiles' rows staged by bulk copies (the measured alternative)
int launch_nonlinear_rot_levels_bulk(const GridDims& g, const NlBatch& b, int nlev, int* err, cudaStream_t st);
int launch_apply_bc(const GridDims& g, double* v, const double* ring, double fac, cudaStream_t st);
int launch_rhsbc(const GridDims& g, double* v, const double* ra, const double* rb, double fac, cudaStream_t st);
int launch_axpby(int n, double a, const double* x, double b, const double* y, double* z, cudaStream_t st);
int launch_sub(int n, const double* x, const double* y, double* z, cudaStream_t st);
int launch_sub_scaled(int n, double d, const double* x, double* z, cudaStream_t st);
int launch_fill(int n, double v, double* z, cudaStream_t st);

// ibm.cu -- fsinterface.F90, grid.F90:459-528, operators_struct.F90:711-834
struct RegDev {
  // per unknown k (nf): component (1 = x, 2 = y), stencil origin, 49 weights
  const int* comp;
  int* ix;
  int* iy;
  double* w;        // nf*49, slot = (l+3)*7 + (p+3)
  // face-major contribution lists over the stencil bounding box, per component
  int* bbox;        // [0..3] = i0, j0, ni, nj (same box for u- and v-faces); [4..9] row ranges
  int* cnt_x;       // bbox faces + 1 (exclusive offsets after the scan)
  int* cnt_y;
  int* lst_x;       // contributions: k*49 + slot, ascending k per face
  int* lst_y;
  int max_faces;    // capacity of cnt_* (faces)
  int max_list;     // capacity of lst_*
  int* stale;       // set by the weights kernel when a stencil origin moved: lists to rebuild
};

int launch_reg_build(const GridDims& g, int nf, const double* xb, const double* yb, double delta, double offx,
                     double offy, RegDev& r, int* d_err, cudaStream_t st);
// The same in two parts: the origins and weights (and whether an origin moved), then the
// bounding box and the contribution lists, which only E^T (reg, redistribution) reads.
int launch_reg_weights(const GridDims& g, int nf, const double* xb, const double* yb, double delta, double offx,
                       double offy, RegDev& r, int* d_err, cudaStream_t st);
int launch_reg_lists(int nf, RegDev& r, const GridDims& g, cudaStream_t st);
// Copies of the origins and weights (ix_s, iy_s: nf ints; w_s: 49 nf doubles).
int launch_reg_snapshot(int nf, const RegDev& r, int* ix_s, int* iy_s, double* w_s, cudaStream_t st);
// hx, hy must be zero outside the stencil box; this writes every face in the box.
int launch_reg(const GridDims& g, int nf, const double* h0, const RegDev& r, double* hx, double* hy,
               cudaStream_t st);
// The same without clearing the fields: every face of the box is written (zero where no
// unknown contributes), the faces outside it are left as they are (read through the box only).
int launch_reg_box(const GridDims& g, int nf, const double* h0, const RegDev& r, double* hx, double* hy,
                   cudaStream_t st);
// h0 (+)= E q   (accumulate=1 keeps the incoming h0, fsinterface.F90:51-80)
int launch_regT(const GridDims& g, int nf, const double* qx, const double* qx0, const double* qy,
                const double* qy0, const RegDev& r, const double* h0_in, double* h0_out, cudaStream_t st);
// h0_out = h0_in + E curl(s) with s ghosts from the ring (curl fused into regT)
int launch_regT_s(const GridDims& g, int nf, const double* s, const double* ring, const RegDev& r,
                  const double* h0_in, double* h0_out, cudaStream_t st);
// finter = E^T f / E^T 1 on faces with weight > 1e-10 (operators_struct.F90:810-834)
int launch_redistribute_field(const GridDims& g, int nf, const double* f, const RegDev& r, double* fx,
                              double* fy, cudaStream_t st);
// mirror (optional): device address of pinned host memory that also receives the coefficients
// and, after them, the nt values of theta
int launch_force_coeffs(int nf, int nbody, const int* comp, const int* bid, const double* f, double dt,
                        double delta, double* out, cudaStream_t st, double* mirror = nullptr,
                        const double* theta = nullptr, int nt = 0);

// structure.cu -- operators_struct.F90 (family 2, torsional bodies)
struct TorsBody {
  int off, npts;
  double gamma0, itheta, ktheta, ctheta, deltas, xbf0, ybf0;
  // step constants of compute_dx (launch_tors_consts): 4/dt^2, 4/dt, 2/dt, the effective
  // stiffness 4/dt^2 I + 2/dt C + K and its reciprocal, deltas / (4/dt^2 I + K), delta/deltas/dt
  double a44, a4, a2, keff, keff_inv, bq, bs;
};
// A family-3 beam (beam.cu): offset and points of its unknowns, DOFs, the cosine and sine of
// its direction, the matrices (row-major) and the Newmark state with scratch vectors.
struct BeamDev {
  int off, npts, ndof;
  double sg, cg;
  double *M, *K, *Ke, *Ki, *Mi, *W, *phi, *B, *xy0;
  double *q, *qd, *qdd, *q0, *qd0, *qdd0, *t1, *t2, *t3, *t4;
};
struct TorsState {  // device arrays of length nt
  double *theta, *thetad, *thetadd, *theta0, *thetad0, *thetadd0;
  double *sinv, *cosv;  // sin, cos (gamma0 - theta) at the current theta, kept with theta
};
// BR_build (operators_struct.F90:319-338): x-rows (j-1) ds sin(g0-th),
// y-rows -(j-1) ds cos(g0-th).  sn, cs = sin, cos(g0-th), evaluated once per body.
__device__ __forceinline__ double br_val(const TorsBody& b, double sn, double cs, int j) {
  if (j < b.npts) return (double)j * b.deltas * sn;
  return -(double)(j - b.npts) * b.deltas * cs;
}
// effective stiffness of the Newmark update (operators_struct.F90:402-505)
__device__ __forceinline__ double keff(const TorsBody& b, double dt) {
  return 4.0 / (dt * dt) * b.itheta + 2.0 / dt * b.ctheta + b.ktheta;
}
// b_times2 scale (delta^2/ds/dt)(2 ds/dt), operators_struct.F90:14-127
__device__ __forceinline__ double btimes_scale(const TorsBody& b, double dt, double delta) {
  return (delta * delta / b.deltas / dt) * (2.0 * b.deltas / dt);
}
int launch_tors_btimes(int nt, const TorsBody* tb, const TorsState& s, double dt, double delta, const double* x,
                       double* y, cudaStream_t st);
int launch_tors_rhs(int nt, const TorsBody* tb, const TorsState& s, double dt, double delta, double* y,
                    cudaStream_t st);
int launch_tors_dx(int nt, const TorsBody* tb, const TorsState& s, double dt, double delta, const double* f,
                   double* xb, double* yb, double* err, cudaStream_t st);
// The end of one device FSI iteration in one kernel (fsi_update.cu): structure update,
// weights and influence patches at the new positions, and the loop condition.
struct FsiUpdateArgs {
  // structure: torsional bodies, the solved forces, positions, err[0] max and err[1..nt]
  const TorsBody* tb;
  TorsState ts;
  int nt;
  double dt, delta;
  const double* f;
  double *xb, *yb, *err;
  double *th_next, *sin_next, *cos_next;   // nt each: written before they are committed
  // weights (RegDev's origins and weights, the stale flag, the domain error)
  GridDims g;
  int nf;
  double ox, oy;
  const int* comp;
  int *ix, *iy;
  double* w;
  int *stale, *d_err;
  // patches: the band's tile map (tile x tile vertices), patch values and indices, flags
  const int* tile_of;
  int ntx, tile;
  double* pval;
  int *pidx, *used, *flag;
  // rows [rows[0], rows[1]) of the finest streamfunction and fluxes that are valid (null: all);
  // an unknown whose stencil needs others sets bit 4 of the band flag, which ends the loop
  const int* rows;
  // condition: counters ([0] iterations, [1] Krylov iterations, [2] operator applications,
  // [3] band flag), the cluster solver's counters, the ticket
  int* cnt;
  const int* ist;
  double tol;
  int max_it;
  cudaGraphConditionalHandle h;
  unsigned* done;
};
int launch_fsi_update(const FsiUpdateArgs& a, cudaStream_t st);
// The step constants of every torsional body record (set-up, after the records are uploaded).
int launch_tors_consts(int nt, TorsBody* tb, double dt, double delta, cudaStream_t st);
int launch_tors_initial_acc(int nt, const TorsBody* tb, const TorsState& s, double dt, double delta,
                            const double* f, cudaStream_t st);
int launch_tors_save(int nt, const TorsState& s, cudaStream_t st);
// recomputes sinv, cosv from theta (after theta is set other than by k_tors_dx)
int launch_tors_trig(int nt, const TorsBody* tb, const TorsState& s, cudaStream_t st);

// gmres.cu -- PETSc KSPGMRES as configured in variables.F90:565-574.  Every driver sums in
// one fixed order, so all produce the same iterates:
//   * a slice partial (kSlices contiguous slices of ceil(nf/kSlices) unknowns) takes the
//     rounded products in blocks of 4 consecutive rows, each block (p0+p1)+(p2+p3), and
//     the blocks by a pairwise tree over slice_blocks_p2(n) entries (missing rows and
//     blocks are 0);
//   * the kSlices slice partials are combined by the pairwise tree
//     ((p0+p1)+(p2+p3))+((p4+p5)+(p6+p7));
//   * w = Av - sum_j h_j v_j runs eight chains (j = g, g+8, ...; chain 0 starts at Av) joined
//     by the same pairwise tree;
//   * a dense row product splits the row into mv_segments(nf) column segments of
//     ceil(nf/S) columns, each summed as two chains (even and odd offsets) and e + o, the
//     segments joined by a pairwise tree (seg_tree).
constexpr int kSlices = 8;

// Blocks of 4 rows in a slice of n rows, rounded up to a power of two (at least 1).
__host__ __device__ inline int slice_blocks_p2(int n) {
  int p = 1;
  while (4 * p < n) p <<= 1;
  return p;
}

// Column segments per row of the dense product: the most (at most kSlices) for which the
// rows of one slice, in groups of S lanes that stay within a warp, fit in three warps.
__host__ __device__ inline int mv_segments(int nf) {
  const int nl = (nf + kSlices - 1) / kSlices;
  for (int S = kSlices; S > 1; --S)
    if (3 * (32 / S) >= nl) return S;
  return 1;
}

// One row segment of the dense product: two chains over even and odd offsets, e + o.
template <typename F>
__device__ __forceinline__ double seg_dot(int j0, int j1, F&& term_fma) {
  double e = 0.0, o = 0.0;
  int j = j0;
#pragma unroll 4
  for (; j + 1 < j1; j += 2) {
    e = term_fma(j, e);
    o = term_fma(j + 1, o);
  }
  if (j < j1) e = term_fma(j, e);
  return e + o;
}

// Pairwise tree over the S lanes of a row group (lane = group base + seg): at stride off,
// seg adds seg+off when seg is a multiple of 2*off.  The sum is valid at seg 0.  Every lane
// of the warp must call it.
__device__ __forceinline__ double seg_tree(double p, int seg, int S) {
  const int lane = threadIdx.x & 31;
  for (int off = 1; off < S; off <<= 1) {
    const double q = __shfl_sync(0xffffffffu, p, min(lane + off, 31));
    if ((seg & (2 * off - 1)) == 0 && seg + off < S) p += q;
  }
  return p;
}
struct GmresDev {
  int nf, restart;
  double* V;       // (restart+1) * nf
  double* H;       // (restart+1) * restart, column it at H + it*(restart+1)
  double* cs;
  double* sn;
  double* g;       // restart+1
  double* scal;    // [0]=ttol [1]=res [2]=bnorm [3]=rnorm
  int* ist;        // [0]=its [1]=reason [2]=it (inner) [3]=active [4]=restart cycles
  double* xin;     // matvec input
  double* Av;      // matvec output
};
int launch_gmres_init(const GmresDev& G, cudaStream_t st);
// The optional graph conditional handle is set by the kernel when use_cond != 0: start
// and arnoldi set the inner (Arnoldi) loop condition, update the outer (restart) one.
int launch_gmres_start(const GmresDev& G, const double* b, const double* x, double rtol, double atol, int max_it,
                       cudaStream_t st, cudaGraphConditionalHandle h = 0, int use_cond = 0);
int launch_gmres_arnoldi(const GmresDev& G, int max_it, cudaStream_t st, cudaGraphConditionalHandle h = 0,
                         int use_cond = 0);
int launch_gmres_update(const GmresDev& G, double* x, int max_it, cudaStream_t st, cudaGraphConditionalHandle h = 0,
                        int use_cond = 0);
int launch_copy(int n, const double* a, double* b, cudaStream_t st);
// Launch shape of the cluster solver, worked out on first use (state -1) and kept.
struct FusedPlan {
  int state = -1;   // 1 launchable, 0 not (the problem does not fit the cluster)
  int threads = 0, a_in = 0;
  size_t bytes = 0;
};
// The whole solve on a dense operator A, column-major (At[j*nf + r] = A[r][j]), as one
// cluster of kSlices CTAs: the operations of the start / arnoldi / update kernels in the same
// order, with A applied by the same segmented row products as k_dense_mv.  Writes G.ist like
// them.  Returns IB_ERR_ARG (nothing launched) when the problem does not fit the cluster.
int launch_gmres_fused(const GmresDev& G, FusedPlan* plan, const double* At, const double* b, double* x, double rtol,
                       double atol, int max_it, cudaStream_t st);

// dense symmetric positive definite solve (stationary-body path)
int launch_cholesky(int n, double* A, int* d_err, cudaStream_t st);
int launch_chol_solve(int n, const double* Lf, const double* b, double* x, cudaStream_t st);
int launch_copy_col(int n, const double* src, double* M, int col, cudaStream_t st);
int launch_unit(int n, int i, double* e, cudaStream_t st);

// fp64_peak.cu -- FP64 FMA throughput of the device (the FP64 roof of the DST kernels)
int probe_fp64(double* tflops);

}  // namespace ib
