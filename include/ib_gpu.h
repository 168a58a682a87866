/*
 * C ABI of the GB300 immersed-boundary time step.
 *
 * Drop-in boundary for the Fortran modules of nirmaljp6/IB_Parallel
 * (src/timestepper.F90, src/operators_fluid.F90, src/myfft.F90,
 * src/fsinterface.F90, src/operators_struct.F90).  Every entry point returns an
 * int status (IB_OK = 0); the message of the last failure on the calling thread
 * is available from ib_last_error().
 *
 * Arrays cross the ABI in the reference's one-rank layout, x fastest:
 *   vertex field (omega, s):  (n-1) x (m-1)   element (I,J) at (J-2)*(m-1)+(I-2)
 *   u-face flux qx:           n x (m+1)       face (i,j) at (j-1)*(m+1)+(i-1)
 *   v-face flux qy:           (n+1) x m       face (i,j) at (j-1)*m+(i-1)
 *   boundary ring:            2(m+1)+2(n+1)   left[n+1] right[n+1] bottom[m+1] top[m+1]
 *   body vectors (f, xb, yb): nf = 2*nb       per body: x-unknowns then y-unknowns
 * Array pointers may be host or device memory: host arrays are staged through
 * the context's device buffers, device arrays are used in place.  Calls are
 * complete (the context's stream synchronised) when they return.
 */
#ifndef IB_GPU_H
#define IB_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define IB_OK 0
#define IB_ERR_ARG 1
#define IB_ERR_CUDA 2
#define IB_ERR_NOMEM 3
#define IB_ERR_GMRES 4
#define IB_ERR_FSI 5
#define IB_ERR_NONFINITE 6
#define IB_ERR_DOMAIN 7
#define IB_ERR_STATE 8

/* Namelist read_parameters of parameters.F90:55-59 (the sub-domain and pressure
 * keys are not part of this boundary).  motion = motion_grid of user.F90:13-31
 * (frame u, v, angular velocity, centre x, y), constant in time. */
typedef struct IbParams {
  int m, n, mgridlev;
  double dt, Re, len, offsetx, offsety;
  double fsi_tol, atol, rtol;
  int num_stat;
  double motion[5];
  int gmres_restart;  /* PETSc default 30 */
  int gmres_max_it;   /* PETSc default 10000 */
  int fsi_max_it;     /* timestepper.F90:318 iterates while fsi_count <= 1000 */
  int autotune;       /* pick DST launch shapes by timing at ib_create */
  /* How GMRES applies the Schur operator of moving (torsional) bodies.  0: through an
   * influence matrix -- the fluid's vorticity-to-streamfunction map restricted to a band of
   * vertices around the bodies, computed once and rebuilt when a body leaves the band -- from
   * which each FSI iteration assembles the dense nf x nf operator (same operator as the
   * matrix-free one up to round-off); solves whose stencils touch the domain boundary fall back
   * to the matrix-free operator; GMRES on the assembled matrix runs as one kernel.
   * 1: always matrix-free (a_times2 per Krylov iteration).  2: as 0, with GMRES as one
   * kernel per Krylov step (the graph the matrix-free operator uses), for comparisons. */
  int schur_mode;
  int influence_margin; /* vertices of slack around the stencils in the band (0: 8) */
} IbParams;

/* One input/body.NNN.inp (grid.F90:252-288).  fam: 1 rigid, 2 torsional, 3 Euler-Bernoulli
 * beam.  Rigid bodies must precede non-rigid ones (grid.F90:1226,1244).  Family 3 is declared
 * and left empty in the reference; here it is a linear beam clamped at its first point along the
 * line to its last point, nelem Hermite-cubic elements (0: (npts-1)/2), itheta = mass per unit
 * length, ktheta = bending stiffness EI (ib_get_beam_state gives its DOFs). */
typedef struct IbBody {
  int npts, fam;
  double gamma0_deg, alpha0_deg, itheta, ktheta, ctheta;
  const double* x;
  const double* y;
  int nelem;
} IbBody;

typedef struct IbCtx IbCtx;

enum { IB_FIELD_OMEGA = 0, IB_FIELD_S = 1, IB_FIELD_QX = 2, IB_FIELD_QY = 3, IB_FIELD_RHS_OLD = 4,
       IB_FIELD_Q0X = 5, IB_FIELD_Q0Y = 6 };
/* IB_VEC_UB: velocity u_B of prescribed rigid-body motion at the body points (nf, per body x then
 * y components; the reference's compute_rhs_prescribed, user.F90:137-174).  Once set it joins
 * every Schur right-hand side as -delta u_B (timestepper.F90:327-331, 479); a host moving a rigid
 * body sets IB_VEC_XB/YB (advance_rigidbody, user.F90:87-115) and IB_VEC_UB before each step. */
enum { IB_VEC_F = 0, IB_VEC_F_RDST = 1, IB_VEC_XB = 2, IB_VEC_YB = 3, IB_VEC_UB = 4 };

/* The namelist items of input/ib.inp that IbParams does not hold (parameters.F90:13-48). */
typedef struct IbRunControl {
  int istart, istop, isave, irestart;
  int compute_pressure, dimen, motion_prescribed;
  int sub_domain, sub_domain_full_rectangular, sub_domain_precomputed;
  double sdxi, sdxe, sdyi, sdye, delta_sd;
} IbRunControl;

const char* ib_last_error(void);
int ib_version(void);

/* setup: grid.F90:117-234 setup, variables.F90:84-257 setup_variables,
 * myfft.F90:96-157 setup_fft.  Initial condition variables.F90:262-295. */
int ib_create(const IbParams* p, const IbBody* bodies, int nbody, IbCtx** out);
int ib_destroy(IbCtx* ctx);
int ib_synchronize(IbCtx* ctx);

/* timestepper.F90:18-556 advance(itime): increments *itime and advances one step.
 * The reference never checks its solvers (KSP reasons are not read, timestepper.F90:363-366;
 * the FSI loop of timestepper.F90:318 ends silently after 1000 iterations).  Here the step is
 * always completed, and then IB_ERR_GMRES is returned if one of its Krylov solves stopped
 * without converging (iteration cap gmres_max_it or breakdown: a negative KSP reason), or
 * IB_ERR_FSI if the FSI iterations stopped at fsi_max_it + 1 without reaching fsi_tol;
 * ib_last_error() gives the reason or the final FSI error. */
int ib_advance(IbCtx* ctx, int* itime);

/* The frame's motion for the steps that follow: uvw = (u, v, angular velocity) of the grid
 * (host memory), the centre of rotation staying motion[3], motion[4] of ib_create.  Replaces the
 * reference's motion_potential + motion_rotation (variables.F90:299-360), which form the frame
 * fluxes q0 from motion_grid (user.F90:13-31); here they are formed on the device, stream-ordered
 * after the steps already launched (IB_ERR_STATE if a step is still in progress).  With
 * the motion given at ib_create the fluxes are those of creation bit for bit.  ib_write_variables
 * then records this motion, and the frame's angle as the reference integrates it (angular
 * velocity times time, exact for a constant one). */
int ib_set_frame(IbCtx* ctx, const double* uvw);

/* state access (the arrays of variables.F90:10-33) */
int ib_get_field(IbCtx* ctx, int field, int level, double* out);
int ib_set_field(IbCtx* ctx, int field, int level, const double* in);
int ib_get_vector(IbCtx* ctx, int which, double* out);
int ib_set_vector(IbCtx* ctx, int which, const double* in);
/* write_force2 (operators_struct.F90:711-731): cx[nbody], cy[nbody] */
int ib_get_forces(IbCtx* ctx, double* cx, double* cy);
/* torsional state of family-2 bodies in file order (variables.F90:31-32) */
int ib_get_body_state(IbCtx* ctx, double* theta, double* thetad, double* thetadd);
/* input (parameters.F90:51-78): the namelist group &read_parameters of the file at path (the
 * reference's input/ib.inp).  Items absent from the file keep the values p and rc hold on
 * entry, as a Fortran namelist read leaves them; an unknown item or a malformed value is an
 * error (IB_ERR_ARG). */
int ib_read_namelist(const char* path, IbParams* p, IbRunControl* rc);
/* setup_geometry (grid.F90:252-288): one body file input/body.NNN.inp (npts; fam; for fam 2 the
 * angles gamma0, alpha0 in degrees and itheta, ktheta, ctheta; for fam 3, which has no layout in
 * the reference, mass per length, EI and the element count; then npts lines of x y), read as
 * the reference's list-directed READs do.  x, y: arrays of capacity cap.  On return body holds
 * the header, npts and pointers to x, y; if cap < npts nothing is copied and IB_ERR_ARG is
 * returned with body->npts set, so a caller can size its arrays and call again. */
int ib_read_body(const char* path, IbBody* body, double* x, double* y, int cap);
/* The bodies of an input directory (grid.F90:252-260): body.001.inp, body.002.inp, ... up to the
 * first number that has no file. */
int ib_count_bodies(const char* dir, int* nbody);
/* The sub-domain precomputed-Schur method (sub_domain = T: grid.F90:320-352, 572-951;
 * timestepper.F90:79-97, 368-405, 500-516, 602-770; operators_struct.F90:840-980), switched on
 * for a context before its first step (and before ib_read_variables on a restart).  The cloud:
 * with full_rectangular = 0 the stationary rigid bodies' points first (point p of the rigid
 * bodies in file order is sub-domain point p; the reference assumes one such body), then the
 * rectangle [sdxi, sdxe] x [sdyi, sdye] at spacing delta_sd, nint((sdxe-sdxi)/delta_sd + 1)
 * points along x.  The fluid Schur operator between the cloud's unknowns, B, is computed at the
 * first step (or read by ib_read_subdomain_matrix) on E E^T's sparsity (21 x 21 face blocks that
 * meet) and thinned by the drop tolerance |B_ij| > 7.0e-3 B_jj; every FSI iteration then solves
 * with body + P B^T P^T, P bilinear interpolation from the cloud to the body points.  Every
 * cloud point's 21 x 21 block must lie inside the grid (the reference indexes it without bounds
 * checks), num_stat must be 0, and a body that leaves the cloud ends its step with
 * IB_ERR_DOMAIN (the reference stops). */
int ib_subdomain_setup(IbCtx* ctx, int full_rectangular, double sdxi, double sdxe, double sdyi, double sdye,
                       double delta_sd);
/* preprocess_sd's column loop now rather than at the first step. */
int ib_subdomain_precompute(IbCtx* ctx);
/* The thinned B in the reference's input/sd_precomputed.chd layout (Fortran unformatted
 * sequential, per column a record of its count, then one of its values and 1-based rows). */
int ib_write_subdomain_matrix(IbCtx* ctx, const char* path);
/* sub_domain_precomputed = T: B read from such a file (same cloud) instead of computed. */
int ib_read_subdomain_matrix(IbCtx* ctx, const char* path);
/* lumat = body_mat + P B^T P^T at the current body positions (nf x nf, row-major), the matrix
 * the FSI iteration solves with (computing B first if needed). */
int ib_subdomain_operator(IbCtx* ctx, double* lumat);
/* counts[4] = {cloud unknowns nf_sd, candidate entries of B (E E^T's sparsity), entries kept
 * after the drop tolerance, columns computed}; *precompute_ms = host wall time of the column
 * loops. */
int ib_get_subdomain_stats(IbCtx* ctx, long long* counts, double* precompute_ms);
/* The discrete adjoint of the step (no reference counterpart) for stationary rigid bodies in a
 * moving frame, their Schur system solved directly (num_stat = 1) or by GMRES on the assembled
 * operator or the sub-domain method's lumat (num_stat = 0, schur_mode 0; the reverse solves the
 * transposed system the same way and returns IB_ERR_GMRES if that solve stops without
 * converging).  The frame's flux
 * (motion_potential + motion_rotation, variables.F90:299-360) is linear in its velocity (u, v)
 * and angular velocity W about the centre (motion[3], motion[4]), so a body pitching or plunging
 * in its own frame is given by a triple (u, v, W) per step (the reference's motion_grid of
 * user.F90:13-31 as a function of the step).
 * ib_adjoint_forward: advances nsteps (<= 4096) from the current state with frames[3 n..3 n+2]
 * at step n, writes the force coefficients forces[(n nbody + b) 2 + {0, 1}] = (Cx, Cy) of body b
 * after step n, and keeps the state every K steps and at the end on the device.
 * ib_adjoint_backward: for J = sum dforces . forces (same layout), writes dJ/dframes (nsteps x
 * 3): each segment of K steps is recomputed from its checkpoint and run backwards through the
 * exact transpose of every operator of the step; the context is left as the forward left it. */
int ib_adjoint_forward(IbCtx* ctx, int nsteps, int K, const double* frames, double* forces);
int ib_adjoint_backward(IbCtx* ctx, const double* dforces, double* dframes);
/* write_variables (variables.F90:709-803): the restart file output/dataRR_IIIIIII.var of one
 * rank at path, in the reference's Fortran unformatted layout (4-byte record markers, 4-byte
 * integers, 8-byte reals; the layout output/getdata.m reads). */
int ib_write_variables(IbCtx* ctx, const char* path);
/* read_variables (variables.F90:807-913): restores omega, s, q, q0 (= q0p + q0r), rhs_old of
 * every level, f, xb, yb and the torsional state from a file of the same grid and bodies, and
 * sets the step counter to itime (the reference's istart), so the next ib_advance is step
 * itime + 1.  Like the reference it ignores the file's dt and f_rdst.  Unlike the reference
 * (timestepper.F90:76), a num_stat context factorises its Schur matrix on its first step
 * whatever itime is. */
int ib_read_variables(IbCtx* ctx, const char* path, int itime);
/* state of the family-3 beams in file order, each 2 nelem DOFs (w, dw/ds at nodes 1..nelem),
 * concatenated: deflections q, their rates and accelerations (any may be NULL) */
int ib_get_beam_state(IbCtx* ctx, double* q, double* qd, double* qdd);
/* ksp_iter, fsi_iter of the last step (timestepper.F90:365-366, 456) */
int ib_get_counters(IbCtx* ctx, int* ksp_iter, int* fsi_iter);
int ib_get_dims(IbCtx* ctx, int* nf, int* nbc, int* ns, int* nu, int* nv);

/* calculate_pressure (operators_pressure.F90:110-437, called every isave steps by main.F90:40-43
 * when compute_pressure is set): the pressure coefficient 2 (P - |u|^2/2) of the current state
 * at the cell centres of every level, solving D D^T P = D N(q) - D E^T f/dt coarse to fine.
 * p: mgridlev x n x m (levels contiguous, x fastest: cell (i, j) of level k at
 * (k*n + j-1)*m + i-1).  Zero user body forcing, as in the reference's user.F90. */
int ib_calculate_pressure(IbCtx* ctx, double* p);
/* write_pressure (operators_pressure.F90:857-879): the last pressure computed, written as
 * output/pressureRR_IIIIIII.var (index range record, then one record per level). */
int ib_write_pressure(IbCtx* ctx, const char* path);

/* ---- batches: many independent simulations advanced together (no counterpart in the
 * reference, which runs one simulation per job) ---- */
typedef struct IbBatch IbBatch;
/* nsim simulations, each with its own grid and bodies: params[i], and nbody[i] bodies taken in
 * order from `bodies` (the bodies of simulation 0, then of 1, ...).  Each is a context of its
 * own (its own device memory and stream); set autotune = 0 for large batches, since tuning
 * times every simulation's launch shapes at creation.  For the simulations' work to overlap on
 * the GPU, give the process CUDA_DEVICE_MAX_CONNECTIONS=32 before CUDA starts. */
int ib_batch_create(const IbParams* params, const IbBody* bodies, const int* nbody, int nsim, IbBatch** out);
int ib_batch_destroy(IbBatch* batch);
int ib_batch_size(IbBatch* batch, int* nsim);
/* simulation i as a context handle, for every per-context entry point (fields, forces,
 * counters, restart files); it stays the batch's: ib_destroy refuses it */
int ib_batch_context(IbBatch* batch, int i, IbCtx** ctx);
/* one time step of every simulation (timestepper.F90:18-556 each), with the same results as
 * ib_advance on each alone: each simulation's predictor, vort2flux and device FSI loop are
 * queued before the host waits on any, then their corrections, so the simulations' kernels run
 * side by side.  status[nsim] (may be NULL) gets each simulation's ib_advance code; the call
 * returns the first nonzero one (or IB_OK). */
int ib_batch_advance(IbBatch* batch, int* status);

/* ---- operator level (grid level 'level' is 0-based; tables of that level) ---- */
/* operators_fluid.F90:553-587; qx, qy are the total fluxes q+q0 */
int ib_nonlinear(IbCtx* ctx, const double* omega, const double* qx, const double* qy, const double* bc,
                 double* nlx, double* nly);
/* operators_fluid.F90:203-233 rot_int + rot_bc */
int ib_rot(IbCtx* ctx, const double* hx, const double* hy, double* vort);
/* operators_fluid.F90:423-471 curl_int + curl_bc */
int ib_curl(IbCtx* ctx, const double* s, const double* sbc, double* qx, double* qy);
/* operators_fluid.F90:381-419 (coarse modified in place, centre region only) */
int ib_coarsify(IbCtx* ctx, const double* fine, double* coarse);
/* operators_fluid.F90:475-535 */
int ib_get_bc(IbCtx* ctx, const double* s, double fac, double* ring);
/* operators_fluid.F90:539-549 (in place) */
int ib_apply_bc(IbCtx* ctx, double* vort, const double* ring, double fac);
/* myfft.F90:207-216 dst: unnormalised 2-D DST-I (FFTW RODFT00 x RODFT00) */
int ib_dst(IbCtx* ctx, const double* in, double* out);
/* myfft.F90:177-188 ctci */
int ib_ctci(IbCtx* ctx, const double* vort, double* s);
/* The same Poisson solve for an m x n grid without a context and without allocating device
 * memory.  It has no counterpart in the reference; it is for callers that may not allocate
 * when they need the solve: a host that reserves its device memory once at start-up, a time
 * loop that must not pay cudaFree's device-wide synchronisation, or code holding no IbCtx.
 * vort and s are DEVICE arrays of the current device ((n-1) x (m-1), x fastest); the kernels
 * run on `stream` (a cudaStream_t, NULL for the default stream) and the call returns without
 * waiting for them.  Scratch and tables live in one 16 MiB static device array that each GPU
 * loading the library keeps until the process exits: grids needing more ((m-1)(n-1) plus the
 * tables; 1200 x 600 fits, 1280 x 640 does not) fail with IB_ERR_ARG.  The first call on a
 * device, and the first after the grid size changes, does the set-up: it copies the tables and
 * waits for the whole device (cudaDeviceSynchronize), so make it before any stream capture.
 * All calls on a device share the array: calls whose kernels overlap on the GPU race and give
 * wrong results.  Errors are reported through ib_last_error(). */
int ib_ctci_static(int m, int n, const double* vort, double* s, void* stream);
/* myfft.F90:161-173 ainv (in place) */
int ib_ainv(IbCtx* ctx, double* vort);
/* operators_fluid.F90:649-663 fluid_predictor (omega in place) */
int ib_fluid_predictor(IbCtx* ctx, int level, double* omega, const double* rhs, const double* rhs_old,
                       const double* rhsbc);
/* operators_fluid.F90:237-377 vort2flux: omega, s: L*(n-1)(m-1); qx: L*n(m+1); qy: L*(n+1)m,
 * levels contiguous; omega's coarse centres are overwritten as in the reference */
int ib_vort2flux(IbCtx* ctx, double* omega, double* s, double* qx, double* qy);
/* grid.F90:459-528 setup_reg / variables.F90:364-373 reg_prep for positions xb, yb (nf each) */
int ib_reg_prep(IbCtx* ctx, const double* xb, const double* yb);
/* fsinterface.F90:14-47 reg: hx, hy = E^T h0 (fields overwritten) */
int ib_reg(IbCtx* ctx, const double* h0, double* hx, double* hy);
/* fsinterface.F90:51-80 regT: h0 += E (hx, hy) */
int ib_regT(IbCtx* ctx, const double* hx, const double* hy, double* h0);
/* operators_struct.F90:735-834 */
int ib_redistribute(IbCtx* ctx, const double* f, double* frdst);
/* timestepper.F90:774-782 ab_times = operators_fluid.F90:14-120 a_times2 (+ b_times2) */
int ib_schur_apply(IbCtx* ctx, const double* x, double* y);
/* operators_fluid.F90:1020-1105 a_times (fluid part only) */
int ib_schur_apply_fluid(IbCtx* ctx, const double* x, double* y);
/* operators_struct.F90:14-127 b_times2 */
int ib_struct_btimes(IbCtx* ctx, const double* x, double* y);
/* operators_struct.F90:342-398 compute_rhs: y (nf) gets the structural rhs, zero elsewhere */
int ib_struct_rhs(IbCtx* ctx, double* y);
/* operators_struct.F90:402-505 compute_dx: updates theta and body positions; *err = max |dtheta| */
int ib_struct_dx(IbCtx* ctx, const double* f, double* err);
/* GMRES on the Schur operator (timestepper.F90:363-366): f updated in place */
int ib_schur_solve(IbCtx* ctx, const double* rhs, double* f, int* iterations);

/* ---- instrumentation (no counterpart in the reference) ---- */
/* the cudaStream_t every kernel of this context runs on */
int ib_get_stream(IbCtx* ctx, void** stream);
/* average device time (ms) of `reps` back-to-back launches of one full pass over the finest
 * grid: kind 0 the DST-I x pass, 1 the per-mode tridiagonal solve; kinds 2 and 3 the pressure
 * grid's x transform (n x m cells times the m x m DST-I matrix) on the FP64 tensor cores (2) or
 * with FP64 FMAs (3).  The launches cycle over
 * pairs of temporary fields (allocated for the call) that together exceed twice the L2 size,
 * so each reads its input from HBM; the context's state is not touched.  Kinds 4 and 5: the
 * predictor's fused nonlinear + rot stencil of every level on the context's current fields
 * (operators_fluid.F90:553-587, 203-233), with plain loads (4) or with its tiles' rows staged by
 * bulk copies (5; IB_ERR_STATE if its output differs from kind 4's in any bit), each launch
 * after a write of twice the L2 size. */
int ib_time_pass(IbCtx* ctx, int kind, int reps, double* avg_ms);
/* device time (ms, summed over reps back-to-back applications) of the 8 stages of the Schur
 * operator: reg+rot, ainv, coarsify, coarse levels, finest forward, finest solve, finest
 * inverse rows, E curl + B */
int ib_profile_schur(IbCtx* ctx, int reps, double* stage_ms);
/* device time of the phases of ib_advance, summed over the steps since it was started:
 * mode 1 starts (clears) with the FSI iterations run from the host phase by phase, mode 3
 * starts with the device FSI loop kept, 0 stops, 2 only reads.  phase_ms[8] (may be NULL):
 * predictor, vort2flux, FSI right-hand side, Schur assembly, GMRES, FSI update (redistribute,
 * structure, weights, host synchronisation), correction, device FSI loop (mode 3: its graph and
 * the synchronisation that reads its counters); *nsteps (may be NULL): steps timed */
int ib_step_profile(IbCtx* ctx, int mode, double* phase_ms, long long* nsteps);
/* The launch shapes the context runs with (chosen by timing at ib_create when autotune is set):
 * shapes[0..12] = x pass of one level (lines per CTA, threads, one-warp scan), x pass over a few
 * rows (3), x pass over every level (3), y pass (3), modes per CTA of the tridiagonal solve */
int ib_get_launch_shapes(IbCtx* ctx, int* shapes);
/* Fluid part of the Schur matrix (a_times2 without B, operators_fluid.F90:14-120: the matrix
 * timestepper.F90:560-598 builds column by column for stationary bodies) at the current body
 * positions, assembled from the influence matrix (schur_mode 0; built on first use):
 * S[k*nf + l].  *status is 0 when S was assembled; nonzero when the stencils touch the domain
 * boundary or the band does not fit in memory (the solver then uses the matrix-free operator
 * and S is not written). */
int ib_schur_matrix(IbCtx* ctx, double* S, int* status);
/* influence-matrix work since creation: counts = {band builds, columns computed, assemblies,
 * matrix-free fallbacks, band vertices}, build_ms = host wall time of the builds */
int ib_get_influence_stats(IbCtx* ctx, long long* counts, double* build_ms);
/* The coarse levels' responses behind the influence-band build and the sub-domain precompute
 * (no reference counterpart: both evaluate the reference's a_times_sd / a_times2 chain,
 * operators_fluid.F90:14-199, column by column; here the coarse levels' part of every column is
 * a sum of per-vertex responses computed once).  counts[4] = {coarse level solves run, responses
 * held, bytes they take, 1 when enabled}, ms = host wall time of the passes that computed them.
 * The environment variable IB_COARSE_RESP=0 at ib_create runs the coarse chain per column. */
int ib_get_coarse_stats(IbCtx* ctx, long long* counts, double* ms);
/* The ring maps behind the coarse-to-fine recursions of the predictor and of vort2flux (no
 * reference counterpart: fluid_predictor's and vort2flux's level loops, timestepper.F90:103-236
 * and operators_fluid.F90:237-377, solve the levels one after another; here the levels with zero
 * boundary data are solved together, the boundary data follow from dense products precomputed at
 * ib_create, and the final solves again run together).  counts[2] = {1 when in use, bytes the
 * maps take}, ms = host wall time of their precomputation.  Used only when the environment
 * variable IB_RING_MAPS=1 at ib_create (from 3 levels on): at 800 x 400 x 5 they take more time
 * than the level-by-level chain they replace, which runs otherwise. */
int ib_get_ring_maps(IbCtx* ctx, long long* counts, double* ms);
/* How the steps since creation ran (no reference counterpart: the reference's advance,
 * timestepper.F90:18-556, is one host routine).  counts[3] = {steps launched as one CUDA graph
 * (predictor, first vort2flux, forces, correction: from the second step on, when the FSI
 * iterations run in the device loop, the forces come from the direct solve, or there is no
 * body), of those the steps whose device FSI loop left the influence band with iterations
 * still to run (the host took over the loop and ran the correction), steps run phase by
 * phase}.  The environment variable IB_WHOLE_STEP=0 at ib_create turns the one-graph step off. */
int ib_get_step_graph_stats(IbCtx* ctx, long long* counts);
/* enable (1) / disable (0) CUDA-event timing of each DST pass launch; enabling clears the totals */
int ib_profile(IbCtx* ctx, int enable);
/* work done since creation: Schur matvecs and DST passes by kind (0..3, see below) */
int ib_get_work(IbCtx* ctx, long long* matvecs, long long* passes4);
/* kernels launched by this library since it was loaded (all contexts) */
long long ib_launch_count(void);
/* measured FP64 FMA throughput of this GPU (TFLOP/s), from a register-resident FMA loop */
int ib_measure_fp64_peak(double* tflops);
/* kind 0: x pass, 1: y pass with diagonal, 2: y pass of the predictor, 3: plain y pass;
 * count of timed launches, their summed device time (ms) and summed algorithmic DRAM bytes */
int ib_profile_read(IbCtx* ctx, int kind, int* count, double* total_ms, double* bytes);

#ifdef __cplusplus
}
#endif
#endif /* IB_GPU_H */
