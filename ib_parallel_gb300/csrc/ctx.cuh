// Device-resident simulation context: all state of variables.F90 for one rank,
// the spectral tables of myfft.F90, body data, Krylov workspace, and the stream
// every kernel of this simulation runs on.
#pragma once
#include <string>
#include <vector>

#include "../../include/ib_gpu.h"
#include "dst.cuh"
#include "kernels.cuh"
#include "tri.cuh"

namespace ib {

// Propagates a non-OK status to the caller.
#define RC(x)                     \
  do {                            \
    int _rc = (x);                \
    if (_rc != IB_OK) return _rc; \
  } while (0)

// Bump allocator over one device allocation made at ib_create.
struct DevPool {
  char* base = nullptr;
  size_t cap = 0, used = 0;
  template <typename T>
  T* take(size_t n) {
    size_t bytes = ((n * sizeof(T) + 255) / 256) * 256;
    if (used + bytes > cap) return nullptr;
    T* p = reinterpret_cast<T*>(base + used);
    used += bytes;
    return p;
  }
};

// Influence matrix of the fluid part of the Schur operator for moving bodies.  The band R
// is a set of 8 x 8 vertex tiles around the bodies' stencils; K[u][v] (column u contiguous,
// nR x nR) is the finest-level streamfunction at band vertex v for a unit vorticity at band
// vertex u, i.e. the map the matrix-free operator applies between rot and E curl.  Each
// unknown k owns the 8 x 8 vertex patch P_k = rot(E^T e_k) (values and band indices); the
// fluid Schur matrix is S_f = P^T K P (curl is the transpose of rot).
// Pressure recovery (pressure.cu): tables and fields, allocated on the first call.
struct PressureOp {
  bool ready = false, computed = false;
  double* mem = nullptr;
  double* W = nullptr;          // m x m DST-I matrix of the cell grid's x direction
  TriOp tri;                    // per-mode (lx(k) + T_y)^-1 of the n cell rows
  std::vector<double*> rhs, p, oqx, oqy, nlx, nly;   // per level
  double *y = nullptr, *tmp = nullptr, *hx = nullptr, *hy = nullptr, *fdt = nullptr;
  double *ubc = nullptr, *vbc = nullptr, *ring = nullptr;
};

// The buffers and the stream one application of the Schur operator's fluid part works in
// (schur_fluid): the context's own, or one of the band build's concurrent sets.
struct SchurScratch {
  double* vort = nullptr;     // input vorticity (a unit vector during the band build)
  double* specY = nullptr;    // ainv's modes
  double* spec1 = nullptr;    // a level's modes
  double* sbc = nullptr;      // ring
  double* s0 = nullptr;       // output streamfunction rows
  double* w[kMaxLevels] = {}; // ainv's vorticity and its coarsified levels (zero outside the centres)
  int* rr_in = nullptr;       // row range of the input (3 ints)
  int* prev = nullptr;        // the unit vector's last position (band build)
  // band build: per level l, rr_lv[3l..3l+2] = the rows [lo, hi) of ainv's vorticity (l = 0)
  // and of its coarsified levels that hold data, and the treatment of the other rows
  int* rr_lv = nullptr;
  // band build and sub-domain precompute: the finest-level box [box0, box1] x [box2, box3]
  // outside which ainv's response to the column's source is below 1e-18 of its peak, and the
  // coarse responses of level 1 (CoarseResp): with cr_R1 set the coarse levels' chain is the
  // sum of the responses over the level-1 vertices coarsify fills from that box
  int* box = nullptr;
  const double* cr_R1 = nullptr;
  const int* cr_idx1 = nullptr;
  // band build: the column's source vertex and the rows of ainv's modes it wrote last (4 ints:
  // a, b, the previous strip's rows [p0, p1)); with specY_ready the caller has formed ainv's
  // modes in specY (zero outside the strip) and schur_fluid starts from them
  int* strip = nullptr;
  bool specY_ready = false;
  cudaStream_t st = nullptr;
};

// The coarse levels' responses (coarse.cu).  For a level-k vertex v (k >= 1), R[k][slot(v)] is
// the ring level k hands level k-1 when level k's vorticity is the unit vector at v and the
// coarser levels hold its coarsified copies (the chain schur_fluid runs from level L-1 down to
// k).  They depend on the grid alone, so they are computed once per vertex and kept for the
// context's later builds.
struct CoarseResp {
  int* idx[kMaxLevels] = {};            // per level: slot of each vertex, -1 without a response
  std::vector<int> idx_h[kMaxLevels];
  double* R[kMaxLevels] = {};           // per level: slots x nbc ring values
  int cap[kMaxLevels] = {}, n[kMaxLevels] = {};
  int* items = nullptr;                 // the vertices one pass solves, level after level
  size_t items_cap = 0;
  int* err = nullptr;                   // a column's box met a level-1 vertex without a response
  bool enabled = true;                  // IB_COARSE_RESP=0 at creation: the per-column chain
  long long solves = 0;                 // level solves run
  double ms = 0.0;                      // host wall time of the passes
  size_t bytes = 0;
};

// The coarse-to-fine recursions of the predictor and of vort2flux with their chain of
// dependent solves collapsed (ringmap.cu).  Level k's solve depends on level k+1 only through
// its boundary data, which is linear in a short state of level k+1's modes: the two mode rows
// get_bc reads (J = n/4+1, 3n/4+1) and the values at the coarse vertices of the ring's left and
// right sides, as their sum and difference (vS, vA).  Laid out [s0 (N) | s1 (N) | vS | vA]
// (N = m-1 modes, NQ = n/2+1 vertices a side).  The state of level k's solution is that of its
// solution with zero boundary data plus G_k times its own boundary state, so the levels' solves
// with zero boundary data run as one batched launch, the states follow from L-2 dense products
// on the coarse-to-fine chain, and the final solves run as a second batched launch.  The DST's
// mirror symmetry in x splits G_k into two blocks (even modes with vS, odd modes with vA).
// Built only on request (IB_RING_MAPS=1): the twice-solved levels, the products and the
// batched boundary data take more FP64 issue than the chain's latency they remove.
struct RingMaps {
  bool on = false;
  int N = 0, NQ = 0, NS = 0;        // modes, coarse vertices a side, state length
  int nb[2] = {0, 0};               // block sizes: 2 * (modes of that parity) + NQ
  double* Gp[kMaxLevels] = {};      // the predictor's G_k, k = 1..L-2 (block 0 rows, then block 1)
  double* Gc = nullptr;             // vort2flux's (one operator and factor on every level)
  double* Z[kMaxLevels] = {};       // zero-boundary solutions, levels 1..L-2
  double* Ez[kMaxLevels] = {};      // their states
  double* R[kMaxLevels] = {};       // level k's boundary state, k = 0..L-2
  double* mem = nullptr;
  size_t bytes = 0;
  double ms = 0.0;                  // host wall time of the precomputation
};

struct Influence {
  static constexpr int kTile = 8;
  // the band's columns are computed on this many streams at once, each with its own scratch
#ifndef IB_BAND_STREAMS
#define IB_BAND_STREAMS 12
#endif
  static constexpr int kBuildStreams = IB_BAND_STREAMS;
  std::vector<SchurScratch> bscr;
  double* bmem = nullptr;
  int* bint = nullptr;
  static constexpr int kSetInts = 16 + 3 * kMaxLevels;   // prev, rr_in[3], column, box[4], strip[4], rr_lv
  // ainv's response to a unit vector on band row r in every x mode, rows r - trunc_rows ..
  // r + trunc_rows, for the rows [strip_r0, strip_r0 + strip_n) (the band build)
  double* strips = nullptr;
  int strip_r0 = 0, strip_n = 0;
  size_t strip_cap = 0;
  int trunc_rows = 0;   // rows of ainv's response kept on each side of a unit vector's row
  bool built = false;
  bool active = false;        // S holds the operator at the current positions
  bool patch_fresh = false;   // patches and flag match the current reg weights
  int flag_h = 0;             // 1: a patch leaves the band; 2: a patch touches the boundary
  int ntx = 0, nty = 0, ntile = 0, nR = 0;
  std::vector<int2> tiles_h;
  int* tile_of = nullptr;     // ntx*nty: tile index in the band or -1
  int2* tiles = nullptr;      // band tiles (tile coordinates)
  double* K = nullptr;
  size_t capK = 0, capR = 0;
  int* used = nullptr;        // nR: vertex touched by some patch
  int* ulist = nullptr;       // compacted band indices of the touched vertices
  int* upos = nullptr;        // nR: position in ulist or -1
  int* nu = nullptr;          // number of touched vertices
  double* T = nullptr;        // nf rows of nR: T[l][u] = (K P)[ulist[u]][l]
  double* pval = nullptr;     // nf*64 patch values
  int* pidx = nullptr;        // nf*64 patch band indices (-1: none)
  double* S = nullptr;        // nf x nf row-major fluid Schur matrix (P^T K P)
  double* St = nullptr;       // nf x nf column-major operator the solver applies: S + B
  double* brv = nullptr;      // nf: BR entry of each torsional unknown
  double* bco = nullptr;      // nf: b_times2 coefficient of the unknown's body
  int* bod = nullptr;         // nf: torsional body of the unknown, -1 for rigid ones
  int* flag = nullptr;
  int* h_flag = nullptr;      // pinned
  int* rr_in = nullptr;       // row ranges of the precompute (3 ints each)
  int* rr_out = nullptr;
  long long builds = 0, columns = 0, assemblies = 0, fallbacks = 0;
  double build_ms = 0.0;
  CoarseResp cr;
};

// A fixed phase of the time step replayed as one CUDA graph.
struct PhaseGraph {
  cudaGraphExec_t exec = nullptr;
  long long launches = 0;   // kernels in the graph
  long long passes[4] = {0, 0, 0, 0};   // DST passes by kind in the graph
  bool failed = false;
};
inline void drop_phase(PhaseGraph* ph) {
  if (ph->exec) cudaGraphExecDestroy(ph->exec);
  *ph = PhaseGraph{};
}

// The sub-domain precomputed-Schur method (sub_domain = T): a cloud of sub-domain points (the
// stationary rigid bodies' points, then a rectangle at spacing dsd), the fluid Schur operator B
// between them precomputed column by column on E E^T's sparsity and thinned by a drop
// tolerance, and per FSI iteration lumat = body + P B^T P^T with P bilinear interpolation from
// the sub-domain unknowns to the body unknowns.
struct SubDomain {
  bool on = false, ready = false, full_rect = true;
  double sdxi = 0, sdxe = 0, sdyi = 0, sdye = 0, dsd = 0;
  int nx = 0, ny = 0, nr_sd = 0, nb_sd = 0, nf_sd = 0;
  double* ux = nullptr;          // nf_sd positions (x components, then y components)
  double* uy = nullptr;
  int* ucomp = nullptr;
  RegDev reg{};                  // E_o: origins, weights, contribution lists of every unknown
  // candidate rows of each point's columns (point indices ascending, CSR over points), and the
  // point's own slot in its list
  int* cptr = nullptr;
  int* cidx = nullptr;
  int* cself = nullptr;
  int max_cand = 0;
  // B column-compressed after the drop: column j holds nz[j] rows (ascending) from colptr[j]
  long long* colptr = nullptr;
  int* nz = nullptr;
  int* rows = nullptr;
  double* vals = nullptr;
  // P of the body unknowns: 4 sub-domain unknowns and weights each; rigid[k] >= 0 maps a
  // stationary rigid body's unknown onto its own sub-domain point exactly
  int* rigid = nullptr;
  int* pidx = nullptr;
  double* pw = nullptr;
  double* fsd = nullptr;         // P^T f
  // precompute scratch per column set: the patch's 64 vertices, the candidate values
  int* pprev = nullptr;
  double* colbuf = nullptr;
  void* mem = nullptr;           // the fixed-size buffers above, one allocation
  long long candidates = 0, kept = 0, columns = 0;
  double precompute_ms = 0;
};

// The discrete adjoint (adjoint.cu): frame bases, checkpoints of the state every K steps and at
// the end, the tape of one segment's step inputs, the adjoint state and its scratch.
struct AdjointState {
  bool ready = false;
  int nsteps = 0, K = 0, nseg = 0;
  std::vector<double> frames;          // nsteps x (u, v, W)
  std::vector<long long> it_ckpt;      // itime at each checkpoint
  void* mem = nullptr;                 // the fixed-size buffers below
  double* ckpt = nullptr;              // (nseg + 1) states
  double* tape = nullptr;              // K x levels x (omega, qx, qy)
  double* bases = nullptr;             // 3 x levels x (u-faces, v-faces)
  double* q0 = nullptr;                // one step's frame flux, levels x (u-faces, v-faces)
  std::vector<double*> lom, lro, lqx, lqy, lom_n, lro_n, lqx_n, lqy_n, lw, lostar;
  double *t1 = nullptr, *t2 = nullptr, *t3 = nullptr, *zero_v = nullptr;
  double *hx = nullptr, *hy = nullptr, *ax = nullptr, *ay = nullptr;
  double *ring1 = nullptr, *ring2 = nullptr, *ring3 = nullptr;
  double *lf = nullptr, *lrhsf = nullptr, *dforce = nullptr, *dframe = nullptr, *dpart = nullptr;
  double* opT = nullptr;   // the sub-domain's lumat transposed (column-major), for the reverse solve
};

struct Ctx {
  IbParams p{};
  GridDims g{};
  int L = 0;
  double delta = 0, normalize = 0;
  cudaStream_t st = nullptr;
  DevPool pool;

  DstPlan px, py;
  DstLaunch lx, ly_none;
  DstLaunch lx_small;              // x passes over a few rows (latency-bound)
  DstLaunch lx_batch;              // x passes over every level at once

  // per-mode tridiagonal operators replacing the y-direction spectral solves
  TriOp tri_ctci, tri_ainv;
  std::vector<TriOp> tri_pred;     // per level
  TriLaunch tl;
  std::vector<double> vfac, con1, con2, cvis;   // cvis = dt/(2 Delta_k^2 Re)

  // state per level
  std::vector<double*> omega, s, qx, qy, q0x, q0y, rhs_old;
  std::vector<double*> rhs_lv;     // this step's nonlinear right-hand side per level
  // Schur-operator scratch per level
  std::vector<double*> mv_w, mv_s, mv_qx, mv_qy;
  // vort2flux: per-level mode-space fields and the ring each level receives
  std::vector<double*> hat, ringv;
  // vort2flux's modes of the coarser levels (k >= 1; hat[k] keeps the predictor's meanwhile)
  std::vector<double*> v2f_modes;
  unsigned char* rm_v2f = nullptr; // the rows coarsify writes: transformed; the others: ROW_SCALE
  // The step's first vort2flux transforms the finest level back only on the rows E(curl s)
  // reads (plus kFsiRowMargin) when the FSI iterations may run on the device; v2f_rows[0..1]
  // receives the rows, q0_partial says s and q of the finest level hold only those.
  static constexpr int kFsiRowMargin = 8;
  bool v2f_partial = false;
  bool q0_partial = false;
  int* v2f_rows = nullptr;
  double* v2f_f0 = nullptr;        // the finest level's solved modes of that call
  // per level: the boundary terms its solve adds (TriBc: ring end sums, edge-row transforms)
  std::vector<double*> sdv, edgev;
  double* emat = nullptr;          // edge matrix (dst_edge_matrix), its equal-parity entries: (m-1) x m/2
  // row treatments of the Schur operator's partial transforms (per vertex row)
  unsigned char *rm_top = nullptr, *rm_coarse = nullptr;
  double* wmat = nullptr;          // DST-I matrix of the x transform ((m-1) x (m-1))
  double* sk2 = nullptr;           // 2 sin(pi k/m), k = 1..m-1 (closed-form boundary-row modes)
  double* specY = nullptr;         // ainv's mode-space solution inside the Schur operator
  // work arrays
  double *spec1 = nullptr, *spec2 = nullptr, *rhs = nullptr, *rhsbc = nullptr;
  double *nlx = nullptr, *nly = nullptr, *hx = nullptr, *hy = nullptr, *vort = nullptr;
  std::vector<double*> lastbc;
  double *omegabc = nullptr, *sbc = nullptr, *zero_ring = nullptr;
  double* frame_lines = nullptr;   // ib_set_frame's per-row values (allocated on its first call)

  // bodies
  int nbody = 0, nb = 0, nf = 0, nt = 0;
  std::vector<IbBody> bodies_h;
  std::vector<int> comp_h, bid_h;
  std::vector<TorsBody> tb_h;
  double *f = nullptr, *f_rdst = nullptr, *xb = nullptr, *yb = nullptr;
  double *rhsf = nullptr, *tmpf = nullptr, *tmpf2 = nullptr, *forces = nullptr;
  // prescribed motion of rigid bodies (user.F90:137-174 compute_rhs_prescribed): the body
  // velocity u_B; once set, -delta u_B joins the right-hand side of every Schur solve
  double* ub = nullptr;
  bool ub_on = false;
  PressureOp pres;
  SubDomain sd;
  RingMaps rmap;
  AdjointState adj;
  // family-3 beams (beam.cu)
  int nbeam = 0;
  BeamDev* beams = nullptr;
  std::vector<BeamDev> beams_h;
  std::vector<double*> beam_mem;
  int *comp = nullptr, *bid = nullptr;
  RegDev reg{};
  TorsBody* tb = nullptr;
  TorsState ts{};
  double* err_fsi = nullptr;       // [0] max |dtheta|, [1..nt] per body
  GmresDev G{};
  // the whole Krylov solve as one CUDA graph: while(restart cycles){ matvec; start;
  // while(Arnoldi){ matvec; arnoldi } update } on the fixed buffers gm_b (rhs), gm_x (solution)
  double *gm_b = nullptr, *gm_x = nullptr;
  bool use_graph = true;
  bool use_fused = true;           // one-kernel GMRES on the assembled operator
  bool graph_failed = false;
  cudaGraphExec_t solve_exec = nullptr;         // matrix-free operator
  cudaGraph_t solve_graph = nullptr;
  cudaGraphExec_t solve_exec_dense = nullptr;   // assembled operator (Influence::S)
  cudaGraph_t solve_graph_dense = nullptr;
  long long kernels_per_matvec = 0, kernels_per_matvec_dense = 0;
  Influence inf;
  // predictor, first vort2flux and correction as graphs (from the second step on)
  bool use_step_graphs = true;
  PhaseGraph graph_pred, graph_v2f, graph_corr;
  // FSI iteration: right-hand side, Schur assembly, update (redistribute, structure, weights)
  PhaseGraph graph_fsi_rhs, graph_fsi_asm, graph_fsi_upd;
  // the FSI iterations of a step on the device (a while node around one iteration's common
  // path; counters [0] iterations [1] Krylov iterations [2] operator products [3] band flag)
  PhaseGraph graph_fsi_loop;
  long long fsi_body_launches = 0;
  // the whole step as one graph, from the second step on, where the forces come from the
  // device FSI loop (mode 1) or without host decisions (mode 2: no bodies, or the direct
  // solve): predictor, first vort2flux, forces, then the correction, in mode 1 under an if
  // node that a gate kernel opens when the host loop has no iteration left to run.  graph_step
  // counts what always runs (the FSI iterations come from fsi_body/post_launches), step_corr
  // the correction's kernels and DST passes.  IB_WHOLE_STEP=0 in the environment at creation
  // turns it off (the step then runs phase by phase with a host readback in the middle).
  PhaseGraph graph_step, step_corr;
  int step_mode = 0;
  bool use_whole_step = true;
  bool step_pending = false;       // graph_step launched: its counters arrive with the step
  long long n_step_graph = 0, n_step_gate_closed = 0, n_step_phased = 0;
  // origins and weights of the current positions, copied at the start of a device FSI
  // iteration for its redistribution (the weights are rebuilt meanwhile)
  int* reg_ix_s = nullptr;
  int* reg_iy_s = nullptr;
  double* reg_w_s = nullptr;
  // the device FSI loop's fused update: theta, sin, cos before they are committed, its ticket
  double* tors_next = nullptr;     // 3 x (nt + 1)
  unsigned* fsi_done = nullptr;
  long long fsi_post_launches = 0;
  int* fsi_cnt = nullptr;
  FusedPlan fused_plan;
  double* cholM = nullptr;         // nf x nf (num_stat)
  bool chol_ready = false;

  // host-visible status
  int* d_err = nullptr;
  int* h_ist = nullptr;            // pinned mirror of G.ist
  double* h_scal = nullptr;        // pinned mirror of err_fsi[0]
  // The step's outputs in mapped pinned memory: force coefficients (cx of every body, then cy)
  // and hinge angles.  Once the host has asked for them, every step's coefficient kernel writes
  // them there before the step finishes (want_out), and ib_get_forces / ib_get_body_state read
  // them without a device round trip while out_fresh (set by ib_advance when they were written,
  // cleared by every other entry point that may change the state).
  double* h_out = nullptr;
  double* d_out = nullptr;         // h_out's device address (mapped)
  bool want_out = false, out_queued = false, out_fresh = false;

  // staging for host pointers passed to operator entry points
  double* stage[8] = {nullptr};
  size_t stage_n = 0;

  int itime = 0, ksp_iter = 0, fsi_iter = 0;
  // outcome of the last step's solves: the most negative KSP reason of its Krylov solves (0
  // if none failed), and the FSI error when the loop stopped at fsi_max_it (else 0)
  int gmres_reason = 0;
  double fsi_err_capped = 0.0;
  // the parts of a step begun and not yet ended or finished (op_advance_begin/end/finish)
  bool loop_pending = false, end_pending = false, finish_pending = false;

  // work counters (host side): Schur matvecs and DST passes by kind
  long long n_matvec = 0;
  long long n_pass[4] = {0, 0, 0, 0};

  // optional stage timing of the Schur operator (ib_profile_schur): events at stage borders
  static constexpr int kStages = 8;
  bool stage_on = false;
  cudaEvent_t stage_ev[kStages + 1] = {};
  double stage_ms[kStages] = {0};

  // optional phase timing of the time step (ib_step_profile): 0 predictor, 1 vort2flux,
  // 2 FSI right-hand side, 3 Schur assembly, 4 GMRES, 5 FSI update (redistribute, structure,
  // weights, synchronisation), 6 correction, 7 the device FSI loop (its graph and the
  // synchronisation that reads its counters; step_prof_dev: the device loop stays on)
  static constexpr int kStepPhases = 8;
  bool step_prof = false;
  bool step_prof_dev = false;
  cudaEvent_t step_ev[10] = {};
  double step_ms[kStepPhases] = {0};
  long long step_n = 0;

  // optional CUDA-event timing of DST passes (ib_profile)
  static constexpr int kProfMax = 8192;
  bool prof_on = false;
  int prof_n = 0;
  std::vector<cudaEvent_t> prof_ev;     // 2 per record
  std::vector<int> prof_kind;
  std::vector<double> prof_bytes;
};

// Wraps one DST pass launch in an event pair when profiling is on.
struct ProfScope {
  Ctx* c;
  int slot = -1;
  ProfScope(Ctx* cc, int kind, double bytes);
  ~ProfScope();
};

// solver.cu
int ctx_create(const IbParams* p, const IbBody* bodies, int nbody, Ctx** out, std::string* msg);
void ctx_destroy(Ctx* c);
int op_ctci(Ctx* c, const double* in, double* out, const double* ring);  // ring: apply_bc(fac 1) on a copy
int op_ainv(Ctx* c, const double* in, double* out);
int op_dst(Ctx* c, const double* in, double* out);
int op_predictor(Ctx* c, int k, double* om, const double* rhs, const double* rhs_old, const double* rhsbc);
// coarse_modes_given: the coarser levels' vorticity outside the rows coarsify writes is the
// inverse x transform of the predictor's modes still in hat[k] (within a time step only)
// hat0_add (with hat0_given): the finest level's modes are hat[0] + hat0_add
int op_vort2flux(Ctx* c, double* const* w, double* const* s, double* const* qx, double* const* qy,
                 bool all_levels, bool hat0_given = false, bool coarse_modes_given = false,
                 const double* hat0_add = nullptr);
int op_schur(Ctx* c, const double* x, double* y, bool with_b);
int schur_fluid(Ctx* c, const double* vort, const int* rr_in, const int* rr_out, double* s_out,
                const double** ring0_out, const SchurScratch* sc = nullptr);
// influence.cu
int inf_alloc(Ctx* c);                 // fixed-size buffers (at ib_create)
void inf_free(Ctx* c);
// checkpoint.cu: the reference's restart file (variables.F90:709-913)
int op_write_variables(Ctx* c, const char* path, std::string* msg);
// beam.cu: family-3 bodies
int beam_build(Ctx* c, const IbBody* bodies, int nbody, std::string* msg);
void beam_free(Ctx* c);
int launch_beam_rhs(Ctx* c, double* y, cudaStream_t st);
int launch_beam_dx(Ctx* c, const double* f, cudaStream_t st);
int launch_beam_btimes(Ctx* c, const double* x, double* y, cudaStream_t st);
int launch_beam_add_b(Ctx* c, double* St, cudaStream_t st);
int launch_beam_initial_acc(Ctx* c, const double* f, cudaStream_t st);
int launch_beam_save(Ctx* c, cudaStream_t st);
// pressure.cu: calculate_pressure (operators_pressure.F90:110-437) into pres.p
int op_pressure(Ctx* c);
void pressure_free(Ctx* c);
int op_time_pressure_transform(Ctx* c, bool mma, int reps, double* avg_ms);
int op_write_pressure(Ctx* c, const char* path, std::string* msg);
// subdomain.cu: the sub-domain method (grid.F90:572-951, timestepper.F90:368-405, 602-770,
// operators_struct.F90:840-905)
int sd_setup(Ctx* c, int full_rectangular, double sdxi, double sdxe, double sdyi, double sdye, double dsd,
             std::string* msg);
int sd_precompute(Ctx* c);
int sd_assemble(Ctx* c, bool interp);                     // (P at the current positions,) lumat into inf.St
int launch_sd_lumat(Ctx* c, cudaStream_t st);             // lumat from P and the B rows already formed
// coarse.cu: the coarse responses of the level-1 vertices coarsify fills from the marked
// finest-level vertices (ns flags); IB_ERR_NOMEM when they would take more memory than allowed
// (the callers then run the per-column chain)
int cr_prepare(Ctx* c, const std::vector<unsigned char>& fine_mask);
// influence.cu: ainv's strips for the rows r_lo..r_hi (inf_strip_alloc first: false when the
// memory is not there)
bool inf_strip_alloc(Ctx* c, int n);
int inf_strip_table(Ctx* c, int r_lo, int r_hi);
int launch_cr_ring0(Ctx* c, const SchurScratch& sc, cudaStream_t st);
void cr_free(Ctx* c);
// ringmap.cu: the ring maps of a context (IB_RING_MAPS=1 at creation, from 3 levels on; else
// the per-level chain); rm_predict / rm_vort2flux run the recursions (the arguments as
// op_predict_levels and op_vort2flux hold them)
int rm_prepare(Ctx* c);
void rm_free(Ctx* c);
int rm_predict(Ctx* c);
int rm_vort2flux(Ctx* c, double* const* modes, double* F0, bool all_levels, double post0, const double* add0);
// the finest-level vertices within r of a marked one, in x and in y (the boxes of the sources)
void cr_dilate(const GridDims& g, std::vector<unsigned char>& mask, int r);
// rhsf = P E_o (q + q0) + rhsf (P formed first at the current positions unless interp is false)
int launch_sd_rhs(Ctx* c, double* rhsf, cudaStream_t st, bool interp = true);
int launch_sd_interp(Ctx* c, cudaStream_t st);            // P at the current positions
int launch_sd_ET(Ctx* c, const double* hx, const double* hy, double* out, cudaStream_t st);   // out = P E_o h
int launch_sd_spread(Ctx* c, const double* f, double* hx, double* hy, cudaStream_t st);   // E_o^T P^T f
int sd_write(Ctx* c, const char* path, std::string* msg);
int sd_read(Ctx* c, const char* path, std::string* msg);
void sd_free(Ctx* c);
int inf_build_scratch(Ctx* c);
// adjoint.cu: the discrete adjoint for stationary rigid bodies in a moving frame
int op_adjoint_forward(Ctx* c, int nsteps, int K, const double* frames, double* forces, std::string* msg);
int op_adjoint_backward(Ctx* c, const double* dforces, double* dframes, std::string* msg);
void adjoint_free(Ctx* c);
// solver.cu: a time step in three parts (op_advance runs them in a row)
int op_advance_begin(Ctx* c);
int op_advance_end(Ctx* c);
int op_advance_finish(Ctx* c);
int op_read_variables(Ctx* c, const char* path, int itime, std::string* msg);
// graph helpers (solver.cu): a while node after the capture position of st (its body graph
// returned), the graph st is capturing, and programmatic kernel-to-kernel edges
int add_while(cudaStream_t st, cudaGraphConditionalHandle h, cudaGraph_t* body);
cudaGraph_t capture_graph(cudaStream_t st);
void make_edges_programmatic(cudaGraph_t g);
// patches + flag for the current weights (async); cleared: the band flag and the touched-vertex
// flags are already zero (the device FSI loop clears them as it reads them)
int inf_patch(Ctx* c, bool cleared = false);
int inf_prepare(Ctx* c);               // build/rebuild the band if needed, assemble S
int inf_assemble(Ctx* c);              // the assembly kernels only
// the same in parts: K P on the touched vertices (clear_used: clear the touched-vertex flags
// as they are read), the B rows, P^T (K P) + B
int inf_assemble_kp(Ctx* c, cudaStream_t st, bool clear_used);
int inf_assemble_b(Ctx* c, cudaStream_t st);
int inf_assemble_ptk(Ctx* c, cudaStream_t st);
int inf_dense_mv(Ctx* c, const double* x, double* y);   // (S + B) x
int inf_build(Ctx* c);
int op_redistribute(Ctx* c, const double* f, double* frdst);
int op_reg_prep(Ctx* c);
int op_time_pass(Ctx* c, int kind, int reps, double* avg_ms);
int op_profile_schur(Ctx* c, int reps, double* ms);
int op_gmres(Ctx* c, const double* b, double* x, int* its, int* reason);
int op_advance(Ctx* c);
int op_step_profile(Ctx* c, int mode, double* ms, long long* nsteps);
int check_err(Ctx* c);

}  // namespace ib
