// The time step of timestepper.F90:18-556 and the composite operators it calls,
// orchestrated on one CUDA stream over device-resident state.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "ctx.cuh"

namespace ib {


static const double kPi = 4.0 * std::atan(1.0);  // parameters.F90:61

static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

ProfScope::ProfScope(Ctx* cc, int kind, double bytes) : c(cc) {
  c->n_pass[kind] += 1;
  if (!c->prof_on || c->prof_n >= Ctx::kProfMax) return;
  slot = c->prof_n++;
  c->prof_kind[slot] = kind;
  c->prof_bytes[slot] = bytes;
  cudaEventRecord(c->prof_ev[2 * slot], c->st);
}
ProfScope::~ProfScope() {
  if (slot >= 0) cudaEventRecord(c->prof_ev[2 * slot + 1], c->st);
}

// algorithmic DRAM bytes of one pass: each input field read once, the output written once
static double pass_bytes(const Ctx* c, int nin, int nout) { return 8.0 * c->g.ns * (nin + nout); }

// ------------------------------------------------------------- tuning
template <typename F>
static int time_it(Ctx* c, F run, float* ms) {
  // the least of three trials of three runs each, after a warm-up run: one slow trial (a clock
  // ramp, another context's work) must not decide a launch shape the whole run keeps
  cudaEvent_t e0, e1;
  IB_CUDA_CHECK(cudaEventCreate(&e0));
  IB_CUDA_CHECK(cudaEventCreate(&e1));
  int rc = run();
  *ms = 1e30f;
  for (int trial = 0; trial < 3 && rc == IB_OK; ++trial) {
    cudaEventRecord(e0, c->st);
    for (int r = 0; r < 3 && rc == IB_OK; ++r) rc = run();
    cudaEventRecord(e1, c->st);
    cudaEventSynchronize(e1);
    float t = 0.0f;
    cudaEventElapsedTime(&t, e0, e1);
    *ms = std::min(*ms, t);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

// Launch shapes of the x pass, the y pass and the tridiagonal solve, chosen by timing.  A
// shape replaces the default only when it is at least kTuneGain faster than the default timed
// the same way: near ties are left to the default, so that timing noise does not make one run's
// shapes differ from the next run's.
constexpr float kTuneGain = 0.97f;
static int tune(Ctx* c) {
  int dev = 0, smem_max = 0;
  IB_CUDA_CHECK(cudaGetDevice(&dev));
  IB_CUDA_CHECK(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  IB_CUDA_CHECK(cudaMemsetAsync(c->spec1, 0, sizeof(double) * c->g.ns, c->st));
  IB_CUDA_CHECK(cudaMemsetAsync(c->spec2, 0, sizeof(double) * c->g.ns, c->st));
  const int Bs[] = {1, 2, 3, 4, 5, 6, 8, 10, 12, 16};
  const int NTs[] = {32, 64, 96, 128, 160, 192, 256, 320, 384, 512};
  // 0: one level's x pass, 1: y pass, 2: x pass over a few rows, 3: x pass over every level
  for (int which = 0; which < 4; ++which) {
    if (which == 3 && c->L < 2) { c->lx_batch = c->lx; continue; }
    const DstPlan& pl = which != 1 ? c->px : c->py;
    DstLaunch* out = which == 0 ? &c->lx : (which == 1 ? &c->ly_none : (which == 2 ? &c->lx_small : &c->lx_batch));
    int nlines = which == 1 ? c->g.nsx : (which == 2 ? std::min(32, c->g.nsy) : c->g.nsy);
    float best = 1e30f, def_ms = 1e30f;
    DstLaunch bestL = *out;
    const DstLaunch defL = *out;
    for (int B : Bs) {
      size_t smem = which != 1 ? dst_smem_x(pl, B) : dst_smem_y(pl, B, YMODE_NONE);
      if ((long long)smem > smem_max || B > nlines) continue;
      for (int NT : NTs) {
        if (NT > 32 * B * 8) continue;
        for (int narrow = 0; narrow < 2; ++narrow) {
          DstLaunch L; L.B = B; L.NT = NT; L.narrow_scan = narrow;
          float ms = 0;
          auto run = [&]() -> int {
            if (which == 1) {
              DstYArgs a; a.a = c->spec1;
              return dst_pass_y(c->py, c->g.nsx, c->g.nsx, YMODE_NONE, a, L, c->st);
            }
            DstXArgs a; a.in = c->spec2; a.out = c->spec1;
            if (which == 2) { a.nlines = nlines; a.row0 = 0; a.row_step = 1; }
            if (which == 3) {   // every level: the per-level fields as inputs, the spectra as outputs
              a.nlev = c->L;
              for (int k = 0; k < c->L; ++k) { a.lin[k] = c->s[k]; a.lout[k] = c->hat[k]; }
            }
            return dst_pass_x(c->px, c->g.nsy, c->g.nsx, PRE_COPY, a, c->g, L, c->st);
          };
          if (time_it(c, run, &ms) != IB_OK) { cudaGetLastError(); continue; }
          if (ms < best) { best = ms; bestL = L; }
          if (L.B == defL.B && L.NT == defL.NT && L.narrow_scan == defL.narrow_scan) def_ms = ms;
        }
      }
    }
    *out = best < kTuneGain * def_ms ? bestL : defL;
  }
  {
    float best = 1e30f, def_ms = 1e30f;
    TriLaunch bestT = c->tl;
    const TriLaunch defT = c->tl;
    for (int Mb : {1, 2, 4, 8, 16, 32}) {
      if (Mb * c->tri_ctci.C > 1024 || (long long)tri_smem(c->tri_ctci, Mb) > smem_max) continue;
      TriLaunch T; T.Mb = Mb;
      float ms = 0;
      auto run = [&]() -> int { return tri_solve(c->tri_ctci, c->spec1, c->spec1, c->g.nsx, T, c->st); };
      if (time_it(c, run, &ms) != IB_OK) { cudaGetLastError(); continue; }
      if (ms < best) { best = ms; bestT = T; }
      if (Mb == defT.Mb) def_ms = ms;
    }
    c->tl = best < kTuneGain * def_ms ? bestT : defT;
  }
  return IB_OK;
}

// ------------------------------------------------------------- create
int ctx_create(const IbParams* pin, const IbBody* bodies, int nbody, Ctx** out, std::string* msg) {
  const IbParams& p = *pin;
  if (p.m < 8 || p.n < 8 || p.m % 4 || p.n % 4) { *msg = "grid must be divisible by 4 (grid.F90:135)"; return IB_ERR_ARG; }
  if (p.mgridlev < 1 || p.mgridlev > 16) { *msg = "mgridlev out of range"; return IB_ERR_ARG; }
  if (!(p.dt > 0) || !(p.Re > 0) || !(p.len > 0)) { *msg = "dt, Re, len must be positive"; return IB_ERR_ARG; }
  if (nbody < 0 || (nbody > 0 && !bodies)) { *msg = "bad body list"; return IB_ERR_ARG; }
  bool seen_nonrigid = false;
  for (int i = 0; i < nbody; ++i) {
    const IbBody& b = bodies[i];
    if (b.npts < 2 || !b.x || !b.y) { *msg = "body needs >= 2 points"; return IB_ERR_ARG; }
    if (b.fam < 1 || b.fam > 3) { *msg = "body family must be 1 (rigid), 2 (torsional) or 3 (beam)"; return IB_ERR_ARG; }
    if (b.fam == 2 && !(b.itheta > 0)) { *msg = "torsional body needs itheta > 0"; return IB_ERR_ARG; }
    if (b.fam == 3 && (!(b.itheta > 0) || !(b.ktheta > 0))) {
      *msg = "a beam needs mass per length (itheta) and EI (ktheta) > 0"; return IB_ERR_ARG;
    }
    if (b.fam == 3 && (b.nelem < 0 || (b.nelem == 0 && b.npts < 3))) {
      *msg = "a beam needs nelem >= 1 (or at least 3 points)"; return IB_ERR_ARG;
    }
    if (b.fam != 1) seen_nonrigid = true;
    else if (seen_nonrigid) { *msg = "rigid bodies must precede non-rigid ones (grid.F90:1226)"; return IB_ERR_ARG; }
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { *msg = "no CUDA device"; return IB_ERR_CUDA; }

  Ctx* c = new Ctx();
  c->p = p;
  if (c->p.gmres_restart <= 0) c->p.gmres_restart = 30;
  if (c->p.gmres_restart > 60) c->p.gmres_restart = 60;
  if (c->p.gmres_max_it <= 0) c->p.gmres_max_it = 10000;
  if (c->p.fsi_max_it <= 0) c->p.fsi_max_it = 1000;
  c->g.init(p.m, p.n);
  c->L = p.mgridlev;
  c->delta = p.len / (double)p.m;                    // grid.F90:131
  c->normalize = 4.0 * (double)((long long)p.m * p.n);  // myfft.F90:122
  const GridDims& g = c->g;
  const int L = c->L;
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) {
    delete c; *msg = "stream creation failed"; return IB_ERR_CUDA;
  }
  int rc = dst_plan_create(&c->px, g.nsx);
  if (rc == IB_OK) rc = dst_plan_create(&c->py, g.nsy);
  if (rc != IB_OK) { *msg = "unsupported DST size (m, n must be 2^a 3^b 5^c)"; ctx_destroy(c); return rc; }

  // bodies (grid.F90:403-433 collect_bodies)
  c->nbody = nbody;
  for (int i = 0; i < nbody; ++i) c->nb += bodies[i].npts;
  c->nf = 2 * c->nb;
  std::vector<double> xb_h(c->nf), yb_h(c->nf);
  c->comp_h.resize(c->nf);
  c->bid_h.resize(c->nf);
  {
    int off = 0;
    for (int i = 0; i < nbody; ++i) {
      const IbBody& b = bodies[i];
      for (int j = 0; j < b.npts; ++j) {
        xb_h[off + j] = b.x[j]; yb_h[off + j] = b.y[j];
        xb_h[off + b.npts + j] = b.x[j]; yb_h[off + b.npts + j] = b.y[j];
        c->comp_h[off + j] = 1; c->comp_h[off + b.npts + j] = 2;
        c->bid_h[off + j] = i; c->bid_h[off + b.npts + j] = i;
      }
      if (b.fam == 2) {
        TorsBody t;
        t.off = off; t.npts = b.npts;
        t.gamma0 = b.gamma0_deg * kPi / 180.0;
        t.itheta = b.itheta; t.ktheta = b.ktheta; t.ctheta = b.ctheta;
        t.deltas = std::sqrt((b.x[1] - b.x[0]) * (b.x[1] - b.x[0]) + (b.y[1] - b.y[0]) * (b.y[1] - b.y[0]));
        t.xbf0 = b.x[0]; t.ybf0 = b.y[0];
        c->tb_h.push_back(t);
      }
      off += 2 * b.npts;
    }
  }
  c->nt = (int)c->tb_h.size();
  const int nf = c->nf, nt = c->nt, R = c->p.gmres_restart;

  // one device allocation for everything
  size_t ns = g.ns, nu = g.nu, nv = g.nv, nbc = g.nbc;
  int max_faces = (g.m + 3) * (g.n + 3) + 1;
  size_t stage_n = std::max(std::max((size_t)L * ns, (size_t)L * nu), std::max((size_t)L * nv, (size_t)nf));
  stage_n = std::max(stage_n, nbc);
  size_t dbl = 0;
  dbl += (size_t)L * (3 * ns + 2 * nu + 2 * nv);         // state
  dbl += (size_t)L * ns;                                 // per-level predictor right-hand sides
  dbl += (size_t)L * (2 * ns + nu + nv);                 // Schur scratch
  int tri_s = 0, tri_C = 0;
  tri_chunking(g.n, g.nsx, &tri_s, &tri_C);
  size_t tri_n = tri_table_doubles(g.nsx, tri_s, tri_C);
  dbl += (size_t)(2 + L) * tri_n;                        // tridiagonal tables
  dbl += 6 * ns + 2 * nu + 2 * nv;                       // work (+ ainv mode-space copy)
  dbl += (size_t)g.nsx * g.nsx + (size_t)g.nsy;          // DST matrix, row treatments
  dbl += (size_t)g.nsx;                                  // 2 sin(pi k/m) table
  dbl += (size_t)(L + 3) * nbc;                          // rings
  dbl += (size_t)L * ns + (size_t)L * nbc + 2 * L;       // per-level spectra and rings (vort2flux)
  dbl += (size_t)g.nsx * g.nsx + (size_t)L * (2 * (size_t)g.nsy + 2 * (size_t)g.nsx);   // edge matrix, terms
  dbl += (size_t)(L - 1) * ns + (size_t)g.nsy;           // vort2flux's coarse-level modes, row modes
  dbl += 8 * (size_t)nf + 2 * (size_t)nbody + 49 * (size_t)nf;
  dbl += 49 * (size_t)nf + (size_t)nf + 1;               // weights snapshot (+ its origins, as doubles)
  dbl += 3 * ((size_t)nt + 1) + 1;                       // fused FSI update: theta, sin, cos; ticket
  dbl += 8 * (size_t)nt + nt + 3;
  dbl += (size_t)(R + 1) * nf + (size_t)(R + 1) * R + 3 * (R + 1) + 4 + 4 * (size_t)nf + 2;
  if (p.num_stat) dbl += (size_t)nf * nf;
  dbl += 8 * stage_n;
  size_t ints = 2 * (size_t)nf + 2 * (size_t)nf + 16 + 2 * (size_t)max_faces + 2 * 49 * (size_t)nf + 4 + 2 + 8;
  size_t bytes = dbl * 8 + ints * 4 + (size_t)nt * sizeof(TorsBody) + 256 * 400;
  if (cudaMalloc(&c->pool.base, bytes) != cudaSuccess) {
    *msg = "device allocation failed"; ctx_destroy(c); return IB_ERR_NOMEM;
  }
  c->pool.cap = bytes;
  IB_CUDA_CHECK(cudaMemset(c->pool.base, 0, bytes));
  DevPool& P = c->pool;
  auto lv = [&](std::vector<double*>& v, size_t n) {
    v.resize(L);
    for (int k = 0; k < L; ++k) v[k] = P.take<double>(n);
  };
  lv(c->omega, ns); lv(c->s, ns); lv(c->rhs_old, ns); lv(c->rhs_lv, ns);
  lv(c->qx, nu); lv(c->q0x, nu); lv(c->qy, nv); lv(c->q0y, nv);
  lv(c->mv_w, ns); lv(c->mv_s, ns); lv(c->mv_qx, nu); lv(c->mv_qy, nv);
  double* tri_mem = P.take<double>((2 + L) * tri_n);
  c->spec1 = P.take<double>(ns); c->spec2 = P.take<double>(ns); c->rhs = P.take<double>(ns);
  c->rhsbc = P.take<double>(ns); c->vort = P.take<double>(ns); c->specY = P.take<double>(ns);
  c->wmat = P.take<double>((size_t)g.nsx * g.nsx);
  c->sk2 = P.take<double>(g.nsx);
  c->rm_top = P.take<unsigned char>(g.nsy); c->rm_coarse = P.take<unsigned char>(g.nsy);
  c->nlx = P.take<double>(nu); c->hx = P.take<double>(nu);
  c->nly = P.take<double>(nv); c->hy = P.take<double>(nv);
  lv(c->lastbc, nbc);
  c->omegabc = P.take<double>(nbc); c->sbc = P.take<double>(nbc); c->zero_ring = P.take<double>(nbc);
  c->hat.resize(L); c->ringv.resize(L);
  for (int k = 0; k < L; ++k) { c->hat[k] = P.take<double>(ns); c->ringv[k] = P.take<double>(nbc); }
  c->emat = P.take<double>((size_t)g.nsx * g.nsx);
  c->v2f_modes.assign(L, nullptr);
  for (int k = 1; k < L; ++k) c->v2f_modes[k] = P.take<double>(ns);
  c->rm_v2f = P.take<unsigned char>(g.nsy);
  c->v2f_rows = P.take<int>(4);
  c->v2f_partial = nf > 0 && nt > 0 && !p.num_stat;
  c->sdv.resize(L); c->edgev.resize(L);
  for (int k = 0; k < L; ++k) { c->sdv[k] = P.take<double>(2 * (size_t)g.nsy); c->edgev[k] = P.take<double>(2 * (size_t)g.nsx); }
  c->f = P.take<double>(nf); c->f_rdst = P.take<double>(nf); c->xb = P.take<double>(nf);
  c->yb = P.take<double>(nf); c->rhsf = P.take<double>(nf); c->tmpf = P.take<double>(nf);
  c->tmpf2 = P.take<double>(nf); c->forces = P.take<double>(2 * nbody + 1); c->ub = P.take<double>(nf);
  c->comp = P.take<int>(nf); c->bid = P.take<int>(nf);
  c->reg.comp = c->comp; c->reg.ix = P.take<int>(nf); c->reg.iy = P.take<int>(nf);
  c->reg.w = P.take<double>(49 * (size_t)nf); c->reg.bbox = P.take<int>(16);
  c->reg.cnt_x = P.take<int>(max_faces); c->reg.cnt_y = P.take<int>(max_faces);
  c->reg.lst_x = P.take<int>(49 * (size_t)nf + 1); c->reg.lst_y = P.take<int>(49 * (size_t)nf + 1);
  c->reg.stale = P.take<int>(1);
  c->reg_w_s = P.take<double>(49 * (size_t)nf + 1);
  c->reg_ix_s = P.take<int>(nf + 1);
  c->reg_iy_s = P.take<int>(nf + 1);
  c->tors_next = P.take<double>(3 * ((size_t)nt + 1));
  c->fsi_done = P.take<unsigned>(2);
  c->reg.max_faces = max_faces; c->reg.max_list = 49 * nf;
  c->tb = P.take<TorsBody>(nt + 1);
  c->ts.theta = P.take<double>(nt + 1); c->ts.thetad = P.take<double>(nt + 1);
  c->ts.thetadd = P.take<double>(nt + 1); c->ts.theta0 = P.take<double>(nt + 1);
  c->ts.thetad0 = P.take<double>(nt + 1); c->ts.thetadd0 = P.take<double>(nt + 1);
  c->ts.sinv = P.take<double>(nt + 1); c->ts.cosv = P.take<double>(nt + 1);
  c->err_fsi = P.take<double>(nt + 1);
  c->fsi_cnt = P.take<int>(8);
  c->G.nf = nf; c->G.restart = R;
  c->G.V = P.take<double>((size_t)(R + 1) * nf); c->G.H = P.take<double>((size_t)(R + 1) * R);
  c->G.cs = P.take<double>(R + 1); c->G.sn = P.take<double>(R + 1); c->G.g = P.take<double>(R + 1);
  c->G.scal = P.take<double>(4); c->G.ist = P.take<int>(8);
  c->gm_b = P.take<double>(nf + 1); c->gm_x = P.take<double>(nf + 1);
  c->G.xin = P.take<double>(nf); c->G.Av = P.take<double>(nf);
  if (p.num_stat) c->cholM = P.take<double>((size_t)nf * nf);
  c->d_err = P.take<int>(1);
  c->stage_n = stage_n;
  for (int i = 0; i < 8; ++i) c->stage[i] = P.take<double>(stage_n);
  if (!c->stage[7] || !c->d_err) { *msg = "internal pool overflow"; ctx_destroy(c); return IB_ERR_NOMEM; }
  if (cudaMallocHost(&c->h_ist, 16 * sizeof(int)) != cudaSuccess ||   // [12]: the step's error word
      cudaMallocHost(&c->h_scal, 4 * sizeof(double)) != cudaSuccess ||
      cudaHostAlloc(&c->h_out, sizeof(double) * (2 * (size_t)nbody + (size_t)nt + 1), cudaHostAllocMapped) !=
          cudaSuccess ||
      cudaHostGetDevicePointer(&c->d_out, c->h_out, 0) != cudaSuccess) {
    *msg = "pinned allocation failed"; ctx_destroy(c); return IB_ERR_NOMEM;
  }

  c->prof_ev.resize(2 * Ctx::kProfMax);
  c->prof_kind.resize(Ctx::kProfMax);
  c->prof_bytes.resize(Ctx::kProfMax);
  for (auto& e : c->prof_ev) IB_CUDA_CHECK(cudaEventCreate(&e));

  // spectral operators (myfft.F90:125-148) as per-mode tridiagonal systems
  {
    double del2 = c->delta * c->delta;
    std::vector<double> lamx(g.nsx), shift(g.nsx);
    for (int k = 1; k <= g.nsx; ++k) {
      double sn = std::sin(kPi * (double)k / (2.0 * g.m));
      lamx[k - 1] = 4.0 * sn * sn;  // 2 - 2 cos(pi k/m) without cancellation
    }
    for (int k = 1; k <= L; ++k) {
      double del22 = del2 * std::pow(4.0, k - 1);
      c->vfac.push_back(0.5 * p.dt / p.Re / del22 / c->normalize);
      c->con1.push_back(1.5 * p.dt / del22 / c->normalize);
      c->con2.push_back(-0.5 * p.dt / del22 / c->normalize);
      c->cvis.push_back(0.5 * p.dt / del22 / p.Re);
    }
    int rc2 = tri_build(&c->tri_ctci, g.nsx, g.nsy, lamx.data(), 1.0 / (2.0 * g.m), tri_mem);
    double c1 = c->cvis[0];
    for (int k = 0; k < g.nsx; ++k) shift[k] = lamx[k] + 1.0 / c1;
    if (rc2 == IB_OK) rc2 = tri_build(&c->tri_ainv, g.nsx, g.nsy, shift.data(), 1.0 / (2.0 * g.m * c1), tri_mem + tri_n);
    c->tri_pred.resize(L);
    for (int k = 0; k < L && rc2 == IB_OK; ++k) {
      double ck = c->cvis[k];
      for (int q = 0; q < g.nsx; ++q) shift[q] = lamx[q] + 1.0 / ck;
      rc2 = tri_build(&c->tri_pred[k], g.nsx, g.nsy, shift.data(), 2.0 * g.n / ck, tri_mem + (2 + k) * tri_n);
    }
    if (rc2 != IB_OK) { *msg = "tridiagonal table upload failed"; ctx_destroy(c); return rc2; }
  }
  // row treatments of the partial transforms (vertex row r = J-2): coarsify fills coarse rows
  // J = n/4+2 .. 3n/4; apply_bc fills rows J = 2, n wholly and the first/last sample of every
  // other row
  {
    std::vector<unsigned char> top(g.nsy), coarse(g.nsy), v2f(g.nsy);
    for (int r = 0; r < g.nsy; ++r) {
      bool centre = r >= g.n / 4 && r <= 3 * g.n / 4 - 2;
      bool edge = r == 0 || r == g.nsy - 1;
      v2f[r] = centre ? ROW_FFT : ROW_SCALE;
      top[r] = centre ? ROW_FFT : ROW_ZERO;
      coarse[r] = (centre || edge) ? ROW_FFT : ROW_EDGES;
    }
    IB_CUDA_CHECK(cudaMemcpy(c->rm_top, top.data(), g.nsy, cudaMemcpyHostToDevice));
    IB_CUDA_CHECK(cudaMemcpy(c->rm_coarse, coarse.data(), g.nsy, cudaMemcpyHostToDevice));
    IB_CUDA_CHECK(cudaMemcpy(c->rm_v2f, v2f.data(), g.nsy, cudaMemcpyHostToDevice));
    int rc3 = dst_matrix_table(c->px, c->wmat);
    if (rc3 == IB_OK) rc3 = dst_sin2_table(c->px, c->sk2);
    if (rc3 == IB_OK && L > 1) rc3 = dst_edge_matrix(c->px, g, c->wmat, c->emat);
    if (rc3 != IB_OK) { *msg = "DST matrix upload failed"; ctx_destroy(c); return rc3; }
  }

  // frame fluxes q0 = q0p + q0r (variables.F90:299-360), constant in time
  {
    const double* uv = p.motion;
    std::vector<double> ax(nu), ay(nv);
    for (int k = 1; k <= L; ++k) {
      double fac = c->delta * std::pow(2.0, k - 1);
      for (int j = 1; j <= g.n; ++j)
        for (int i = 1; i <= g.m + 1; ++i) {
          double yy = ((double)j - 0.5 - g.n / 2) * c->delta * std::pow(2.0, k - 1) + (g.n / 2) * c->delta - p.offsety;
          ax[(size_t)(j - 1) * g.nux + (i - 1)] = -fac * uv[0] + fac * (0.0 + uv[2] * (yy - uv[4]));
        }
      for (int j = 1; j <= g.n + 1; ++j)
        for (int i = 1; i <= g.m; ++i) {
          double xx = ((double)i - 0.5 - g.m / 2) * c->delta * std::pow(2.0, k - 1) + (g.m / 2) * c->delta - p.offsetx;
          ay[(size_t)(j - 1) * g.nvx + (i - 1)] = -fac * uv[1] + fac * (0.0 - uv[2] * (xx - uv[3]));
        }
      IB_CUDA_CHECK(cudaMemcpy(c->q0x[k - 1], ax.data(), 8 * nu, cudaMemcpyHostToDevice));
      IB_CUDA_CHECK(cudaMemcpy(c->q0y[k - 1], ay.data(), 8 * nv, cudaMemcpyHostToDevice));
    }
  }
  if (nf > 0) {
    IB_CUDA_CHECK(cudaMemcpy(c->xb, xb_h.data(), 8 * (size_t)nf, cudaMemcpyHostToDevice));
    IB_CUDA_CHECK(cudaMemcpy(c->yb, yb_h.data(), 8 * (size_t)nf, cudaMemcpyHostToDevice));
    IB_CUDA_CHECK(cudaMemcpy(c->comp, c->comp_h.data(), 4 * (size_t)nf, cudaMemcpyHostToDevice));
    IB_CUDA_CHECK(cudaMemcpy(c->bid, c->bid_h.data(), 4 * (size_t)nf, cudaMemcpyHostToDevice));
  }
  if (nt > 0) IB_CUDA_CHECK(cudaMemcpy(c->tb, c->tb_h.data(), sizeof(TorsBody) * nt, cudaMemcpyHostToDevice));
  rc = launch_tors_consts(nt, c->tb, p.dt, c->delta, c->st);
  if (rc == IB_OK) rc = launch_tors_trig(nt, c->tb, c->ts, c->st);
  if (rc != IB_OK) { *msg = "device initialisation failed"; ctx_destroy(c); return rc; }
  for (int i = 0; i < nbody; ++i) c->bodies_h.push_back(bodies[i]);

  // default launch shapes, then tuned by timing
  c->lx.B = 1; c->lx.NT = 256; c->lx.narrow_scan = 1;
  c->lx_small.B = 1; c->lx_small.NT = 256;
  c->lx_batch.B = 2; c->lx_batch.NT = 256;
  c->lx_batch.narrow_scan = 1;   // the throughput-bound batched passes scan with one warp
  c->ly_none.B = 3; c->ly_none.NT = 384; c->ly_none.narrow_scan = 1;
  c->tl.Mb = 4;
  c->use_fused = p.schur_mode != 2;
  if (const char* w = std::getenv("IB_WHOLE_STEP")) c->use_whole_step = std::atoi(w) != 0;
  if (const char* w = std::getenv("IB_COARSE_RESP")) c->inf.cr.enabled = std::atoi(w) != 0;
  if (p.autotune) {
    rc = tune(c);
    if (rc != IB_OK) { *msg = "DST tuning failed"; ctx_destroy(c); return rc; }
  }
  rc = rm_prepare(c);
  if (rc != IB_OK) { *msg = "ring map precomputation failed"; ctx_destroy(c); return rc; }
  if (nf > 0 && inf_alloc(c) != IB_OK) { *msg = "device allocation failed"; ctx_destroy(c); return IB_ERR_NOMEM; }
  {
    const int rcb = beam_build(c, bodies, nbody, msg);
    if (rcb != IB_OK) { ctx_destroy(c); return rcb; }
  }
  rc = op_reg_prep(c);
  if (rc == IB_OK) rc = check_err(c);
  if (rc != IB_OK) { *msg = "body stencil outside the grid"; ctx_destroy(c); return rc; }
  *out = c;
  return IB_OK;
}

void ctx_destroy(Ctx* c) {
  if (!c) return;
  if (c->st) cudaStreamSynchronize(c->st);
  dst_plan_destroy(&c->px);
  dst_plan_destroy(&c->py);
  if (c->solve_exec) cudaGraphExecDestroy(c->solve_exec);
  if (c->solve_graph) cudaGraphDestroy(c->solve_graph);
  if (c->solve_exec_dense) cudaGraphExecDestroy(c->solve_exec_dense);
  for (PhaseGraph* ph : {&c->graph_pred, &c->graph_v2f, &c->graph_corr, &c->graph_fsi_rhs, &c->graph_fsi_asm,
                         &c->graph_fsi_upd, &c->graph_fsi_loop, &c->graph_step})
    drop_phase(ph);
  if (c->solve_graph_dense) cudaGraphDestroy(c->solve_graph_dense);
  inf_free(c);
  pressure_free(c);
  beam_free(c);
  sd_free(c);
  rm_free(c);
  if (c->frame_lines) cudaFree(c->frame_lines);
  adjoint_free(c);
  if (c->pool.base) cudaFree(c->pool.base);
  if (c->h_ist) cudaFreeHost(c->h_ist);
  if (c->h_scal) cudaFreeHost(c->h_scal);
  if (c->h_out) cudaFreeHost(c->h_out);
  for (auto& e : c->prof_ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : c->stage_ev)
    if (e) cudaEventDestroy(e);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
}

int check_err(Ctx* c) {
  int e = 0;
  IB_CUDA_CHECK(cudaMemcpyAsync(c->h_ist, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  IB_CUDA_CHECK(cudaStreamSynchronize(c->st));
  e = c->h_ist[0];
  if (e) {
    IB_CUDA_CHECK(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->st));
    return e;
  }
  return IB_OK;
}

// ------------------------------------------------------------- operators
// x transform -> per-mode tridiagonal solve along y -> x transform
static int spectral_solve(Ctx* c, DstPre pre, const DstXArgs& a_in, const TriOp& op, double* out) {
  DstXArgs a = a_in;
  a.out = c->spec1;
  {
    ProfScope ps(c, 0, pass_bytes(c, pre == PRE_PRED ? 4 : 1, 1));
    RC(dst_pass_x(c->px, c->g.nsy, c->g.nsx, pre, a, c->g, c->lx, c->st));
  }
  {
    ProfScope ps(c, 1, pass_bytes(c, 1, 1));
    RC(tri_solve(op, c->spec1, c->spec1, c->g.nsx, c->tl, c->st));
  }
  DstXArgs b;
  b.in = c->spec1; b.out = out;
  ProfScope ps(c, 0, pass_bytes(c, 1, 1));
  return dst_pass_x(c->px, c->g.nsy, c->g.nsx, PRE_COPY, b, c->g, c->lx, c->st);
}

// ctci (myfft.F90:177-188); ring != null applies apply_bc(fac 1) to a copy of the input
int op_ctci(Ctx* c, const double* in, double* out, const double* ring) {
  DstXArgs a;
  a.in = in; a.ring = ring; a.fac = 1.0;
  return spectral_solve(c, ring ? PRE_APPLYBC : PRE_COPY, a, c->tri_ctci, out);
}

// ainv (myfft.F90:161-173)
int op_ainv(Ctx* c, const double* in, double* out) {
  DstXArgs a;
  a.in = in;
  return spectral_solve(c, PRE_COPY, a, c->tri_ainv, out);
}

int op_dst(Ctx* c, const double* in, double* out) {
  DstXArgs a;
  a.in = in; a.out = out;
  {
    ProfScope ps(c, 0, pass_bytes(c, 1, 1));
    RC(dst_pass_x(c->px, c->g.nsy, c->g.nsx, PRE_COPY, a, c->g, c->lx, c->st));
  }
  DstYArgs y;
  y.a = out;
  ProfScope ps(c, 3, pass_bytes(c, 1, 1));
  return dst_pass_y(c->py, c->g.nsx, c->g.nsx, YMODE_NONE, y, c->ly_none, c->st);
}

// fluid_predictor (operators_fluid.F90:649-663):
// omega = dst(lam1i*(dst(con1 rhs + con2 rhs_old + rhsbc) + lam1*dst(omega)))
//       = S_x (2n/c)(1/c + lam_x + T_y)^-1 S_x[con1 rhs + con2 rhs_old + rhsbc + (omega - c L omega)/normalize]
int op_predictor(Ctx* c, int k, double* om, const double* rhs, const double* rhs_old, const double* rhsbc) {
  DstXArgs a;
  a.in = rhs; a.in2 = rhs_old; a.in3 = rhsbc; a.in4 = om;
  a.ca = c->con1[k]; a.cb = c->con2[k];
  double cv = c->cvis[k];
  a.alpha = (1.0 - 4.0 * cv) / c->normalize;
  a.beta = cv / c->normalize;
  return spectral_solve(c, PRE_PRED, a, c->tri_pred[k], om);
}

static int ring_from_modes(Ctx* c, const double* spec, double* s, double* ring, double fac = 1.0);

// The boundary terms level k's solve adds: from its ring, left by level k+1.
static TriBc level_bc(Ctx* c, int k, double post_scale) {
  TriBc bc;
  bc.sk2 = c->sk2;
  bc.sd = c->sdv[k];
  bc.edge = c->edgev[k];
  bc.post_scale = post_scale;
  return bc;
}

// Level k's ring (fac * get_bc of the coarser level's streamfunction or vorticity, from its
// modes spec) and the boundary terms of its solve.
static int ring_edge_from_modes(Ctx* c, const double* spec, int k, double fac) {
  return dst_ring_edge_from_modes(c->px, c->g, spec, c->g.nsx, c->wmat, c->emat, fac, c->ringv[k], c->sdv[k],
                                  c->edgev[k], c->st);
}

// vort2flux (operators_fluid.F90:237-377).  all_levels=false writes the streamfunction and the
// fluxes of the finest level only (the coarser levels' vorticity is still coarsified and their
// modes still give the finest level its boundary values).
//
// Only the boundary values a level receives from the next coarser one depend on the
// coarse-to-fine recursion, and they enter through apply_bc on the boundary rows and
// columns.  So the x transforms of every level's vorticity run as one batched pass; then,
// coarse to fine in mode space, each level adds the transform of its boundary terms
// (closed form on interior rows, dot products on the two edge rows), solves its per-mode
// tridiagonal systems and evaluates the next finer level's ring from its modes at the few
// points get_bc reads; one batched inverse pass and the curls finish.
int op_vort2flux(Ctx* c, double* const* w, double* const* s, double* const* qx, double* const* qy, bool all_levels,
                 bool hat0_given, bool coarse_modes_given, const double* hat0_add) {
  const int L = c->L;
  const GridDims& g = c->g;
  cudaStream_t st = c->st;
  if (L > kMaxBatch) return IB_ERR_ARG;
  // hat0_given: hat[0] holds modes Y with w[0] = S_x Y, so S_x w[0] = 2m Y and the finest level
  // skips its forward transform (its boundary terms scale Y by 2m).  With all_levels false the
  // finest level is then solved in spec2, leaving Y in hat[0] for the correction.
  const bool skip0 = hat0_given && L >= 2;
  double* F0 = skip0 && !all_levels ? c->spec2 : c->hat[0];
  // The coarser levels are transformed and solved in v2f_modes[k].  coarse_modes_given: their
  // vorticity is S_x Y_k, Y_k the predictor's modes still in hat[k], except on the rows
  // coarsify writes, so only those rows are transformed and the others take 2m Y_k.
  const bool cm = coarse_modes_given && skip0;
  auto modes = [&](int k) -> double* { return k == 0 ? c->hat[0] : c->v2f_modes[k]; };
  for (int k = 1; k < L; ++k) RC(launch_coarsify(g, w[k - 1], w[k], st));
  {
    DstXArgs a;
    const int k0 = skip0 ? 1 : 0;
    a.nlev = L - k0;
    for (int k = k0; k < L; ++k) {
      a.lin[k - k0] = w[k];
      a.lout[k - k0] = modes(k);
      if (cm) a.lin2[k - k0] = c->hat[k];
    }
    if (cm) {
      a.rowmode = c->rm_v2f;
      a.row_scale = 2.0 * g.m;
    }
    ProfScope ps(c, 0, pass_bytes(c, L - k0, L - k0));
    RC(dst_pass_x(c->px, g.nsy, g.nsx, PRE_COPY, a, g, c->lx_batch, st));
  }
  if (c->rmap.on) {
    // the same recursion with the chain of level solves collapsed (with all_levels false the
    // coarser levels' final solves are not needed: only their boundary data is)
    double* mk[kMaxLevels];
    for (int k = 0; k < L; ++k) mk[k] = modes(k);
    RC(rm_vort2flux(c, mk, F0, all_levels, skip0 ? 2.0 * g.m : 1.0, skip0 ? hat0_add : nullptr));
  } else {
    for (int k = L - 1; k >= 0; --k) {
      double* F = k == 0 ? F0 : modes(k);
      // boundary terms of the ring of level k (get_bc of level k+1), apply_bc with fac 1, added
      // by the solve as it loads its right-hand side
      TriBc bc;
      if (k < L - 1) bc = level_bc(c, k, k == 0 && skip0 ? 2.0 * g.m : 1.0);
      if (k == 0 && skip0) bc.add2 = hat0_add;
      {
        ProfScope ps(c, 1, pass_bytes(c, 1, 1));
        RC(tri_solve(c->tri_ctci, modes(k), F, g.nsx, c->tl, st, bc));
      }
      if (k > 0) RC(ring_edge_from_modes(c, F, k - 1, 1.0));
    }
  }
  if (!all_levels) {
    DstXArgs a;
    a.in = F0; a.out = s[0];
    c->v2f_f0 = F0;
    if (c->v2f_partial) {   // the rows E(curl s) reads, widened; the others are left as they are
      a.rowrange = c->reg.bbox + 7;
      a.row_margin = Ctx::kFsiRowMargin;
      a.rows_used = c->v2f_rows;
    }
    {
      ProfScope ps(c, 0, pass_bytes(c, 1, 1));
      RC(dst_pass_x(c->px, g.nsy, g.nsx, PRE_COPY, a, g, c->lx, st));
    }
    return launch_curl(g, s[0], L == 1 ? c->zero_ring : c->ringv[0], qx[0], qy[0], st);
  }
  {
    DstXArgs a;
    a.nlev = L;
    for (int k = 0; k < L; ++k) { a.lin[k] = modes(k); a.lout[k] = s[k]; }
    ProfScope ps(c, 0, pass_bytes(c, L, L));
    RC(dst_pass_x(c->px, g.nsy, g.nsx, PRE_COPY, a, g, c->lx_batch, st));
  }
  CurlBatch cb;
  for (int k = 0; k < L; ++k) {
    cb.s[k] = s[k];
    cb.sbc[k] = k == L - 1 ? c->zero_ring : c->ringv[k];
    cb.qx[k] = qx[k];
    cb.qy[k] = qy[k];
  }
  return launch_curl_levels(g, cb, L, st);
}

// s on the next finer level's boundary only: the points get_bc reads, each an inverse x
// transform evaluated as a dot product (spread over all SMs), then get_bc
// (operators_fluid.F90:475-535) into the ring.
static int ring_from_modes(Ctx* c, const double* spec, double* s, double* ring, double fac) {
  (void)s;   // the field itself is not needed: the ring comes straight from the modes
  return dst_ring_from_modes(c->px, c->g, spec, c->g.nsx, c->wmat, fac, ring, c->st);
}

// The fluid part of the Schur operator between rot and E curl: the finest-level
// streamfunction s_out = (vort2flux(ainv(vort)))_1 on the rows rr_out selects, and the ring
// of level 1 in *ring0.  vort must be zero outside the rows rr_in selects.
//  * ainv: x transform of the rows rr_in selects, tridiagonal solve (Y), full inverse
//    transform (the vorticity every coarser level is coarsified from).
//  * coarse levels: inputs are the coarsified centre rows plus the boundary values of
//    apply_bc (closed-form transforms); outputs are needed on the finer boundary only.
//  * finest level: its forward transform is 2m Y plus the boundary terms; its inverse is
//    needed only on the rows rr_out selects.
int schur_fluid(Ctx* c, const double* vort, const int* rr_in, const int* rr_out, double* s_out,
                const double** ring0_out, const SchurScratch* sc) {
  const GridDims& g = c->g;
  const int L = c->L;
  // the context's own buffers unless a scratch set (and its stream) is given
  SchurScratch own;
  if (!sc) {
    own.specY = c->specY; own.spec1 = c->spec1; own.sbc = c->sbc; own.st = c->st;
    for (int k = 0; k < L; ++k) own.w[k] = c->mv_w[k];
    sc = &own;
  }
  cudaStream_t st = sc->st;
  double* specY = sc->specY;
  double* spec1 = sc->spec1;
  auto mark = [&](int i) { if (c->stage_on) cudaEventRecord(c->stage_ev[i], st); };
  if (!sc->specY_ready) {   // else the band build has formed ainv's modes of its unit vector
    {
      DstXArgs a;
      a.in = vort; a.out = specY; a.rowrange = rr_in;
      ProfScope ps(c, 0, pass_bytes(c, 1, 1));
      RC(dst_pass_x(c->px, g.nsy, g.nsx, PRE_COPY, a, g, c->lx_small, st));
    }
    {
      ProfScope ps(c, 1, pass_bytes(c, 1, 1));
      RC(tri_solve(c->tri_ainv, specY, specY, g.nsx, c->tl, st));
    }
  }
  {
    DstXArgs a;
    a.in = specY; a.out = sc->w[0];
    if (sc->rr_lv) a.rowrange = sc->rr_lv;   // band build: the rows of ainv's response
    ProfScope ps(c, 0, pass_bytes(c, 1, 1));
    RC(dst_pass_x(c->px, g.nsy, g.nsx, PRE_COPY, a, g, c->lx, st));
  }
  mark(2);
  const double* ring0 = c->zero_ring;
  if (L > 1 && sc->cr_R1) {
    // the coarse levels by superposition of their responses (coarse.cu)
    mark(3);
    RC(launch_cr_ring0(c, *sc, st));
    ring0 = sc->sbc;
  } else if (L > 1) {
    // outside their centres the coarse vorticities of the operator stay zero
    for (int k = 1; k < L; ++k) RC(launch_coarsify(g, sc->w[k - 1], sc->w[k], st));
    mark(3);
    for (int k = L - 1; k >= 1; --k) {
      DstXArgs a;
      a.in = sc->w[k]; a.out = spec1;
      a.ring = sc->sbc; a.fac = 1.0;
      if (sc->rr_lv) {   // band build: the coarsified rows holding data (and the edge rows)
        a.rowrange = sc->rr_lv + 3 * k;
        a.fft_edge_rows = k == L - 1 ? 0 : 1;
      } else {
        a.rowmode = k == L - 1 ? c->rm_top : c->rm_coarse;
      }
      {
        ProfScope ps(c, 0, pass_bytes(c, 1, 1));
        RC(dst_pass_x(c->px, g.nsy, g.nsx, k == L - 1 ? PRE_COPY : PRE_APPLYBC, a, g, c->lx, st));
      }
      {
        ProfScope ps(c, 1, pass_bytes(c, 1, 1));
        RC(tri_solve(c->tri_ctci, spec1, spec1, g.nsx, c->tl, st));
      }
      RC(dst_ring_from_modes(c->px, g, spec1, g.nsx, c->wmat, 1.0, sc->sbc, st));
    }
    ring0 = sc->sbc;
  } else {
    mark(3);
  }
  mark(4);
  {
    // S_x(vort1 + apply_bc(ring0)) = 2m Y + transform of the boundary terms: the two full
    // boundary rows by dot products, the others in closed form (two nonzero samples)
    ProfScope ps(c, 0, pass_bytes(c, 1, 1));
    RC(dst_x_bc_modes(c->px, g, ring0, c->wmat, c->sk2, specY, 2.0 * g.m, spec1, st, sc != &own));
  }
  mark(5);
  {
    ProfScope ps(c, 1, pass_bytes(c, 1, 1));
    RC(tri_solve(c->tri_ctci, spec1, spec1, g.nsx, c->tl, st));
  }
  mark(6);
  {
    DstXArgs a;
    a.in = spec1; a.out = s_out; a.rowrange = rr_out;
    ProfScope ps(c, 0, pass_bytes(c, 1, 1));
    RC(dst_pass_x(c->px, g.nsy, g.nsx, PRE_COPY, a, g, c->lx_small, st));
  }
  *ring0_out = ring0;
  return IB_OK;
}

// ab_times / a_times2 (timestepper.F90:774-782, operators_fluid.F90:14-120):
// y = E (vort2flux(ainv(rot(E^T x))))_1 + B x, evaluating only what E reads: the rows
// rot(E^T x) can touch go in, the rows E (curl s) reads come out, and curl is fused into E.
int op_schur(Ctx* c, const double* x, double* y, bool with_b) {
  const GridDims& g = c->g;
  cudaStream_t st = c->st;
  c->n_matvec += 1;
  auto mark = [&](int i) { if (c->stage_on) cudaEventRecord(c->stage_ev[i], st); };
  mark(0);
  RC(launch_reg(g, c->nf, x, c->reg, c->hx, c->hy, st));
  RC(launch_rot(g, c->hx, c->hy, c->vort, st));
  mark(1);
  const double* ring0 = nullptr;
  RC(schur_fluid(c, c->vort, c->reg.bbox + 4, c->reg.bbox + 7, c->mv_s[0], &ring0));
  mark(7);
  RC(launch_regT_s(g, c->nf, c->mv_s[0], ring0, c->reg, nullptr, y, st));
  if (with_b) RC(launch_tors_btimes(c->nt, c->tb, c->ts, c->p.dt, c->delta, x, y, st));
  if (with_b) RC(launch_beam_btimes(c, x, y, st));
  mark(8);
  return IB_OK;
}

// Device time of each stage of the Schur operator, summed over `reps` back-to-back
// applications: 0 reg+rot, 1 ainv, 2 coarsify, 3 coarse levels, 4 finest forward,
// 5 finest solve, 6 finest inverse rows, 7 E curl + B.
int op_profile_schur(Ctx* c, int reps, double* ms) {
  for (int i = 0; i <= Ctx::kStages; ++i)
    if (!c->stage_ev[i]) IB_CUDA_CHECK(cudaEventCreate(&c->stage_ev[i]));
  for (int i = 0; i < Ctx::kStages; ++i) ms[i] = 0.0;
  RC(op_schur(c, c->G.xin, c->G.Av, true));
  c->stage_on = true;
  for (int r = 0; r < reps; ++r) {
    int rc = op_schur(c, c->G.xin, c->G.Av, true);
    if (rc != IB_OK) { c->stage_on = false; return rc; }
    IB_CUDA_CHECK(cudaEventSynchronize(c->stage_ev[Ctx::kStages]));
    for (int i = 0; i < Ctx::kStages; ++i) {
      float t = 0.f;
      cudaEventElapsedTime(&t, c->stage_ev[i], c->stage_ev[i + 1]);
      ms[i] += t;
    }
  }
  c->stage_on = false;
  c->n_matvec -= reps + 1;
  return IB_OK;
}

static int redistribute_with(Ctx* c, const RegDev& r, const double* f, double* frdst) {
  RC(launch_redistribute_field(c->g, c->nf, f, r, c->nlx, c->nly, c->st));
  return launch_regT(c->g, c->nf, c->nlx, nullptr, c->nly, nullptr, r, nullptr, frdst, c->st);
}

int op_redistribute(Ctx* c, const double* f, double* frdst) { return redistribute_with(c, c->reg, f, frdst); }

// Kinds 4 and 5: the predictor's nonlinear-and-rot stencil over every level on the context's
// current fields, with plain loads (4) or with the interior tiles' rows staged by bulk copies
// (5), each launch after a write of twice the L2 size (so its inputs come from HBM).  Kind 5
// first checks that both give the same bits.
static int time_nonlinear(Ctx* c, bool bulk, int reps, double* avg_ms) {
  const GridDims& g = c->g;
  const int L = c->L;
  cudaStream_t st = c->st;
  int dev = 0, l2 = 0;
  IB_CUDA_CHECK(cudaGetDevice(&dev));
  IB_CUDA_CHECK(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev));
  double* out = nullptr;
  void* flush = nullptr;
  const size_t fbytes = 2 * (size_t)l2;
  IB_CUDA_CHECK(cudaMalloc(&out, 16 * (size_t)g.ns * L));
  if (cudaMalloc(&flush, fbytes) != cudaSuccess) {
    cudaFree(out);
    return IB_ERR_NOMEM;
  }
  NlBatch b[2];
  for (int v = 0; v < 2; ++v)
    for (int k = 0; k < L; ++k) {
      b[v].om[k] = c->omega[k];
      b[v].bc[k] = c->lastbc[k];
      b[v].qx[k] = c->qx[k];
      b[v].q0x[k] = c->q0x[k];
      b[v].qy[k] = c->qy[k];
      b[v].q0y[k] = c->q0y[k];
      b[v].out[k] = out + ((size_t)v * L + k) * g.ns;
    }
  int rc = IB_OK;
  auto launch = [&](bool use_bulk, int v) {
    return use_bulk ? launch_nonlinear_rot_levels_bulk(g, b[v], L, c->d_err, st)
                    : launch_nonlinear_rot_levels(g, b[v], L, st);
  };
  if (bulk) {   // the two kernels' outputs, bit for bit
    rc = launch(false, 0);
    if (rc == IB_OK) rc = launch(true, 1);
    if (rc == IB_OK) {
      std::vector<double> h(2 * (size_t)g.ns * L);
      if (cudaMemcpyAsync(h.data(), out, 8 * h.size(), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess)
        rc = IB_ERR_CUDA;
      else if (std::memcmp(h.data(), h.data() + (size_t)g.ns * L, 8 * (size_t)g.ns * L) != 0)
        rc = IB_ERR_STATE;
    }
    if (rc == IB_OK) rc = check_err(c);
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (rc == IB_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) rc = IB_ERR_CUDA;
  double total = 0.0;
  for (int r = 0; r < reps && rc == IB_OK; ++r) {
    if (cudaMemsetAsync(flush, r & 0xff, fbytes, st) != cudaSuccess) rc = IB_ERR_CUDA;
    if (rc == IB_OK && cudaEventRecord(e0, st) != cudaSuccess) rc = IB_ERR_CUDA;
    if (rc == IB_OK) rc = launch(bulk, 0);
    if (rc == IB_OK && cudaEventRecord(e1, st) != cudaSuccess) rc = IB_ERR_CUDA;
    if (rc == IB_OK && cudaEventSynchronize(e1) != cudaSuccess) rc = IB_ERR_CUDA;
    float ms = 0.f;
    if (rc == IB_OK) cudaEventElapsedTime(&ms, e0, e1);
    total += ms;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamSynchronize(st);
  cudaFree(out);
  cudaFree(flush);
  if (rc == IB_OK) rc = check_err(c);
  RC(rc);
  *avg_ms = total / reps;
  return IB_OK;
}

// Device time of `reps` back-to-back launches of one full pass over the finest grid
// (kind 0: x pass, 1: tridiagonal solve), for the roofline of a kernel timed alone; kinds 4
// and 5: time_nonlinear.
int op_time_pass(Ctx* c, int kind, int reps, double* avg_ms) {
  if (kind == 4 || kind == 5) return time_nonlinear(c, kind == 5, reps, avg_ms);
  // Each launch reads and writes its own pair of fields, and the pairs together are more than
  // twice L2, so every pass starts with its input in HBM, as in a step.
  cudaStream_t st = c->st;
  int dev = 0, l2 = 0;
  IB_CUDA_CHECK(cudaGetDevice(&dev));
  IB_CUDA_CHECK(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev));
  const size_t field = 8 * (size_t)c->g.ns;
  const int nbuf = std::max(2, (int)((2 * (size_t)l2 + field - 1) / field));
  double* buf = nullptr;
  IB_CUDA_CHECK(cudaMalloc(&buf, 2 * field * nbuf));
  // nonzero inputs (every byte 0x3f: about 4.8e-4 in each double)
  int rc = cudaMemsetAsync(buf, 0x3f, 2 * field * nbuf, st) == cudaSuccess ? IB_OK : IB_ERR_CUDA;
  auto run = [&](int i) -> int {
    double* in = buf + (size_t)(2 * (i % nbuf)) * c->g.ns;
    double* out = in + c->g.ns;
    if (kind == 0) {
      DstXArgs a; a.in = in; a.out = out;
      return dst_pass_x(c->px, c->g.nsy, c->g.nsx, PRE_COPY, a, c->g, c->lx, st);
    }
    return tri_solve(c->tri_ctci, in, out, c->g.nsx, c->tl, st);
  };
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (rc == IB_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) rc = IB_ERR_CUDA;
  for (int i = 0; i < nbuf && rc == IB_OK; ++i) rc = run(i);   // warm-up over every pair
  if (rc == IB_OK && cudaEventRecord(e0, st) != cudaSuccess) rc = IB_ERR_CUDA;
  for (int r = 0; r < reps && rc == IB_OK; ++r) rc = run(r);
  if (rc == IB_OK && cudaEventRecord(e1, st) != cudaSuccess) rc = IB_ERR_CUDA;
  if (rc == IB_OK && cudaEventSynchronize(e1) != cudaSuccess) rc = IB_ERR_CUDA;
  float ms = 0.f;
  if (rc == IB_OK) cudaEventElapsedTime(&ms, e0, e1);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamSynchronize(st);
  cudaFree(buf);
  RC(rc);
  *avg_ms = ms / reps;
  return IB_OK;
}

int op_reg_prep(Ctx* c) {
  c->inf.patch_fresh = false;
  c->inf.active = false;
  return launch_reg_build(c->g, c->nf, c->xb, c->yb, c->delta, c->p.offsetx, c->p.offsety, c->reg, c->d_err, c->st);
}

static int read_ist(Ctx* c) {
  IB_CUDA_CHECK(cudaMemcpyAsync(c->h_ist, c->G.ist, 8 * sizeof(int), cudaMemcpyDeviceToHost, c->st));
  IB_CUDA_CHECK(cudaStreamSynchronize(c->st));
  return IB_OK;
}

// Adds a conditional node of the given type (while, if) after the current capture position of
// `st` and returns its body graph.
static int add_conditional(cudaStream_t st, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                           cudaGraph_t* body) {
  cudaStreamCaptureStatus stat;
  cudaGraph_t capg;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  IB_CUDA_CHECK(cudaStreamGetCaptureInfo(st, &stat, nullptr, &capg, &deps, nullptr, &ndeps));
  cudaGraphNodeParams pr = {};
  pr.type = cudaGraphNodeTypeConditional;
  pr.conditional.handle = h;
  pr.conditional.type = type;
  pr.conditional.size = 1;
  cudaGraphNode_t node;
  IB_CUDA_CHECK(cudaGraphAddNode(&node, capg, deps, nullptr, ndeps, &pr));
  IB_CUDA_CHECK(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  *body = pr.conditional.phGraph_out[0];
  return IB_OK;
}

int add_while(cudaStream_t st, cudaGraphConditionalHandle h, cudaGraph_t* body) {
  return add_conditional(st, h, cudaGraphCondTypeWhile, body);
}

cudaGraph_t capture_graph(cudaStream_t st) {
  cudaStreamCaptureStatus stat;
  cudaGraph_t g = nullptr;
  cudaStreamGetCaptureInfo(st, &stat, nullptr, &g, nullptr, nullptr, nullptr);
  return g;
}

// The Schur operator the Krylov solver applies: the assembled matrix when the influence
// matrix is active, else the matrix-free operator.
static int schur_mv(Ctx* c, bool dense, const double* x, double* y) {
  return dense ? inf_dense_mv(c, x, y) : op_schur(c, x, y, true);
}

// Builds the graph of a whole GMRES solve (KSPSolve, timestepper.F90:363-366) on gm_b/gm_x.
static int build_solve_graph(Ctx* c, bool dense) {
  const GmresDev& G = c->G;
  const int max_it = c->p.gmres_max_it;
  const double rtol = c->p.rtol, atol = c->p.atol;
  cudaStream_t st = c->st, s1 = nullptr, s2 = nullptr;
  IB_CUDA_CHECK(cudaStreamCreateWithFlags(&s1, cudaStreamNonBlocking));
  IB_CUDA_CHECK(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
  const bool prof = c->prof_on;
  c->prof_on = false;
  int rc = IB_OK;
  cudaGraph_t graph = nullptr;
  do {
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) != cudaSuccess) { rc = IB_ERR_CUDA; break; }
    rc = launch_gmres_init(G, st);
    cudaGraphConditionalHandle h_out = 0, h_in = 0;
    cudaGraph_t outer = nullptr, inner = nullptr;
    if (rc == IB_OK && cudaGraphConditionalHandleCreate(&h_out, capture_graph(st), 1, cudaGraphCondAssignDefault) != cudaSuccess)
      rc = IB_ERR_CUDA;
    if (rc == IB_OK) rc = add_while(st, h_out, &outer);
    // restart cycle: r = b - A x, V0, then the Arnoldi loop, then x += V y
    if (rc == IB_OK && cudaStreamBeginCaptureToGraph(s1, outer, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess)
      rc = IB_ERR_CUDA;
    if (rc == IB_OK && cudaGraphConditionalHandleCreate(&h_in, outer, 0, 0) != cudaSuccess) rc = IB_ERR_CUDA;
    if (rc == IB_OK) {
      c->st = s1;
      rc = launch_copy(c->nf, c->gm_x, G.xin, s1);
      long long l0 = launch_count();
      if (rc == IB_OK) rc = schur_mv(c, dense, G.xin, G.Av);
      (dense ? c->kernels_per_matvec_dense : c->kernels_per_matvec) = launch_count() - l0;
      c->n_matvec -= 1;  // capture only
      if (rc == IB_OK) rc = launch_gmres_start(G, c->gm_b, c->gm_x, rtol, atol, max_it, s1, h_in, 1);
      if (rc == IB_OK) rc = add_while(s1, h_in, &inner);
      if (rc == IB_OK && cudaStreamBeginCaptureToGraph(s2, inner, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess)
        rc = IB_ERR_CUDA;
      if (rc == IB_OK) {
        c->st = s2;
        rc = schur_mv(c, dense, G.xin, G.Av);
        c->n_matvec -= 1;
        if (rc == IB_OK) rc = launch_gmres_arnoldi(G, max_it, s2, h_in, 1);
        cudaGraph_t tmp;
        if (cudaStreamEndCapture(s2, &tmp) != cudaSuccess && rc == IB_OK) rc = IB_ERR_CUDA;
      }
      c->st = s1;
      if (rc == IB_OK) rc = launch_gmres_update(G, c->gm_x, max_it, s1, h_out, 1);
      cudaGraph_t tmp;
      if (cudaStreamEndCapture(s1, &tmp) != cudaSuccess && rc == IB_OK) rc = IB_ERR_CUDA;
    }
    c->st = st;
    if (cudaStreamEndCapture(st, &graph) != cudaSuccess && rc == IB_OK) rc = IB_ERR_CUDA;
    if (rc == IB_OK && cudaGraphInstantiate(dense ? &c->solve_exec_dense : &c->solve_exec, graph, 0) != cudaSuccess)
      rc = IB_ERR_CUDA;
  } while (false);
  c->st = st;
  c->prof_on = prof;
  cudaGetLastError();
  if (rc == IB_OK) (dense ? c->solve_graph_dense : c->solve_graph) = graph;
  else if (graph) cudaGraphDestroy(graph);
  cudaStreamDestroy(s1);
  cudaStreamDestroy(s2);
  return rc;
}

// KSPSolve with KSPGMRES (timestepper.F90:363-366); x is the initial guess.
int op_gmres(Ctx* c, const double* b, double* x, int* its, int* reason) {
  const GmresDev& G = c->G;
  const int max_it = c->p.gmres_max_it;
  const bool dense = c->inf.active;
  if (dense && c->use_fused) {
    // the whole solve in one kernel on the assembled matrix
    int rc = launch_gmres_fused(G, &c->fused_plan, c->inf.St, b, x, c->p.rtol, c->p.atol, max_it, c->st);
    if (rc == IB_OK) {
      RC(read_ist(c));
      c->n_matvec += c->h_ist[0] + c->h_ist[4];
      *its = c->h_ist[0];
      *reason = c->h_ist[1];
      return IB_OK;
    }
    if (rc != IB_ERR_ARG) return rc;
  }
  if (c->use_graph && !c->prof_on && !c->graph_failed) {
    cudaGraphExec_t& exec = dense ? c->solve_exec_dense : c->solve_exec;
    if (!exec && build_solve_graph(c, dense) != IB_OK) c->graph_failed = true;
    if (exec) {
      if (b != c->gm_b) IB_CUDA_CHECK(cudaMemcpyAsync(c->gm_b, b, 8 * (size_t)c->nf, cudaMemcpyDeviceToDevice, c->st));
      if (x != c->gm_x) IB_CUDA_CHECK(cudaMemcpyAsync(c->gm_x, x, 8 * (size_t)c->nf, cudaMemcpyDeviceToDevice, c->st));
      IB_CUDA_CHECK(cudaGraphLaunch(exec, c->st));
      if (x != c->gm_x) IB_CUDA_CHECK(cudaMemcpyAsync(x, c->gm_x, 8 * (size_t)c->nf, cudaMemcpyDeviceToDevice, c->st));
      RC(read_ist(c));
      long long it = c->h_ist[0], cycles = c->h_ist[4];
      c->n_matvec += it + cycles;
      count_launches((it + cycles) * (dense ? c->kernels_per_matvec_dense : c->kernels_per_matvec) + it +
                     3 * cycles + 1);
      *its = (int)it;
      *reason = c->h_ist[1];
      return IB_OK;
    }
  }
  RC(launch_gmres_init(G, c->st));
  for (;;) {
    IB_CUDA_CHECK(cudaMemcpyAsync(G.xin, x, 8 * (size_t)c->nf, cudaMemcpyDeviceToDevice, c->st));
    RC(schur_mv(c, dense, G.xin, G.Av));
    RC(launch_gmres_start(G, b, x, c->p.rtol, c->p.atol, max_it, c->st));
    RC(read_ist(c));
    if (c->h_ist[1] != 0) break;
    for (;;) {
      RC(schur_mv(c, dense, G.xin, G.Av));
      RC(launch_gmres_arnoldi(G, max_it, c->st));
      RC(read_ist(c));
      if (!c->h_ist[3]) break;
    }
    RC(launch_gmres_update(G, x, max_it, c->st));
    RC(read_ist(c));
    if (c->h_ist[1] != 0 || c->h_ist[0] >= max_it) break;
  }
  *its = c->h_ist[0];
  *reason = c->h_ist[1];
  return IB_OK;
}

static int preprocess_chol(Ctx* c) {
  // timestepper.F90:560-598: column i of the Schur matrix is a_times(e_i)
  const int nf = c->nf;
  for (int i = 0; i < nf; ++i) {
    RC(launch_unit(nf, i, c->tmpf, c->st));
    RC(op_schur(c, c->tmpf, c->tmpf2, false));
    RC(launch_copy_col(nf, c->tmpf2, c->cholM, i, c->st));
  }
  RC(launch_cholesky(nf, c->cholM, c->d_err, c->st));
  int e = check_err(c);
  if (e) return IB_ERR_ARG;
  c->chol_ready = true;
  return IB_OK;
}

// mode 1: start (totals cleared) with the FSI iterations run from the host, phase by phase;
// 3: start with the device FSI loop kept (timed as one phase); 0: stop; 2: read only.
// ms[8] totals, *nsteps steps timed.
int op_step_profile(Ctx* c, int mode, double* ms, long long* nsteps) {
  if (mode == 1 || mode == 3) {
    for (auto& e : c->step_ev)
      if (!e) IB_CUDA_CHECK(cudaEventCreate(&e));
    for (double& v : c->step_ms) v = 0.0;
    c->step_n = 0;
    c->step_prof = true;
    c->step_prof_dev = mode == 3;
  } else if (mode == 0) {
    c->step_prof = false;
  }
  if (ms)
    for (int i = 0; i < Ctx::kStepPhases; ++i) ms[i] = c->step_ms[i];
  if (nsteps) *nsteps = c->step_n;
  return IB_OK;
}

static void step_mark(Ctx* c, int i) {
  if (c->step_prof) cudaEventRecord(c->step_ev[i], c->st);
}

// adds the time between events a and b (both complete) to phase ph
static void step_acc(Ctx* c, int ph, int a, int b) {
  if (!c->step_prof) return;
  float t = 0.f;
  if (cudaEventElapsedTime(&t, c->step_ev[a], c->step_ev[b]) == cudaSuccess) c->step_ms[ph] += t;
}

// Turns every ordinary kernel-to-kernel edge of a captured graph into a programmatic one: the
// dependent kernel may be scheduled while its predecessor finishes (every kernel here starts
// with IB_GRID_DEP_WAIT).  Edges to or from other nodes keep full serialisation.  An edge the
// driver refuses to convert is put back as it was.
void make_edges_programmatic(cudaGraph_t g) {
  size_t n = 0;
  if (cudaGraphGetEdges(g, nullptr, nullptr, nullptr, &n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return;
  }
  std::vector<cudaGraphNode_t> from(n), to(n);
  std::vector<cudaGraphEdgeData> ed(n);
  if (cudaGraphGetEdges(g, from.data(), to.data(), ed.data(), &n) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  for (size_t i = 0; i < n; ++i) {
    cudaGraphNodeType ta, tb;
    if (cudaGraphNodeGetType(from[i], &ta) != cudaSuccess || cudaGraphNodeGetType(to[i], &tb) != cudaSuccess) continue;
    if (ta != cudaGraphNodeTypeKernel || tb != cudaGraphNodeTypeKernel) continue;
    if (ed[i].type != cudaGraphDependencyTypeDefault || ed[i].from_port != cudaGraphKernelNodePortDefault) continue;
    cudaGraphEdgeData e = {};
    e.from_port = cudaGraphKernelNodePortProgrammatic;
    e.type = cudaGraphDependencyTypeProgrammatic;
    if (cudaGraphRemoveDependencies(g, &from[i], &to[i], &ed[i], 1) != cudaSuccess) continue;
    if (cudaGraphAddDependencies(g, &from[i], &to[i], &e, 1) != cudaSuccess)
      cudaGraphAddDependencies(g, &from[i], &to[i], &ed[i], 1);
  }
  cudaGetLastError();
}

// Runs one fixed phase of the step (the same kernels on the same buffers every step) through a
// CUDA graph captured on first use, which removes the gaps between its dependent launches.
// If capture fails the phase runs directly from then on.
template <typename F>
static int run_phase(Ctx* c, PhaseGraph& ph, F&& fn) {
  if (!c->use_step_graphs || c->prof_on || c->stage_on || ph.failed) return fn();
  if (!ph.exec) {
    const long long l0 = launch_count();
    long long p0[4];
    for (int i = 0; i < 4; ++i) p0[i] = c->n_pass[i];
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(c->st, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
      cudaGetLastError();
      ph.failed = true;
      return fn();
    }
    const int rc = fn();
    const cudaError_t e = cudaStreamEndCapture(c->st, &graph);
    ph.launches = launch_count() - l0;
    count_launches(-ph.launches);   // captured, not run
    for (int i = 0; i < 4; ++i) {
      ph.passes[i] = c->n_pass[i] - p0[i];
      c->n_pass[i] = p0[i];
    }
    if (rc == IB_OK && e == cudaSuccess) make_edges_programmatic(graph);
    if (rc != IB_OK || e != cudaSuccess || cudaGraphInstantiate(&ph.exec, graph, 0) != cudaSuccess) {
      cudaGetLastError();
      if (graph) cudaGraphDestroy(graph);
      ph.exec = nullptr;
      ph.failed = true;
      return fn();
    }
    cudaGraphDestroy(graph);
  }
  IB_CUDA_CHECK(cudaGraphLaunch(ph.exec, c->st));
  count_launches(ph.launches);
  for (int i = 0; i < 4; ++i) c->n_pass[i] += ph.passes[i];
  return IB_OK;
}

// ------------------------------------------------------------- FSI iterations on the device
__global__ void k_fsi_loop_init(int* cnt, int* band_flag, unsigned* done) {
  IB_GRID_DEP_WAIT();
  if (threadIdx.x < 8) cnt[threadIdx.x] = 0;
  if (threadIdx.x == 0) {
    *band_flag = 0;
    *done = 0u;
  }
}

// Captures the graph of a step's FSI iterations: the counters reset, then a while node whose
// body is one iteration on the assembled operator, and after it the contribution lists of the
// final positions.  The body runs its independent parts side by side:
//     s1: K P ---------> P^T K P + B -> Krylov solve -> structure update, weights, patches, condition
//     s2: B rows, right-hand side --^                \-> redistribution ----------------------------->|
//     s3: copy of the current weights, their contribution lists -----------^
// The lists (read only by E^T, i.e. the redistribution, and after the loop by the
// correction) are rebuilt at the start of the iteration after the weights they belong to,
// and the redistribution reads the copy, so neither is on the chain from one solve to the
// next.  The band flag and the touched-vertex flags are cleared by the kernels that read
// them (the condition, the compaction), so the patches need no memsets; the end of the
// iteration is one kernel (k_fsi_update).  The body's launches are counted once
// (fsi_body_launches), the lists after the loop in fsi_post_launches.
// Adds the FSI iterations to the graph `st` is capturing (see build_fsi_loop).
static int capture_fsi_loop(Ctx* c, cudaStream_t st) {
  const GridDims& g = c->g;
  const IbParams& p = c->p;
  Influence& I = c->inf;
  cudaStream_t s1 = nullptr, s2 = nullptr, s3 = nullptr;
  cudaEvent_t ev[7] = {};
  int rc = IB_OK;
  if (cudaStreamCreateWithFlags(&s1, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s3, cudaStreamNonBlocking) != cudaSuccess)
    rc = IB_ERR_CUDA;
  for (int i = 0; i < 7 && rc == IB_OK; ++i)
    if (cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming) != cudaSuccess) rc = IB_ERR_CUDA;
  cudaEvent_t ev_fork = ev[0], ev_rhs = ev[1], ev_lists = ev[2], ev_f = ev[3], ev_rd = ev[4];
  cudaEvent_t ev_p = ev[5], ev_b = ev[6];   // the sub-domain's P, and the body block's rows
  do {
    if (rc != IB_OK) break;
    count_launch();
    k_fsi_loop_init<<<1, 32, 0, st>>>(c->fsi_cnt, I.flag, c->fsi_done);
    cudaGraphConditionalHandle h = 0;
    cudaGraph_t body = nullptr;
    if (cudaGraphConditionalHandleCreate(&h, capture_graph(st), 1, cudaGraphCondAssignDefault) != cudaSuccess)
      rc = IB_ERR_CUDA;
    if (rc == IB_OK) rc = add_while(st, h, &body);
    if (rc == IB_OK && cudaStreamBeginCaptureToGraph(s1, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) !=
                           cudaSuccess)
      rc = IB_ERR_CUDA;
    if (rc == IB_OK) {
      c->st = s1;
      const long long b0 = launch_count();
      auto iteration = [&]() -> int {
        IB_CUDA_CHECK(cudaEventRecord(ev_fork, s1));
        IB_CUDA_CHECK(cudaStreamWaitEvent(s2, ev_fork, 0));
        IB_CUDA_CHECK(cudaStreamWaitEvent(s3, ev_fork, 0));
        // s1 (sub-domain): P at these positions, beside the B rows
        if (c->sd.on) {
          RC(launch_sd_interp(c, s1));
          IB_CUDA_CHECK(cudaEventRecord(ev_p, s1));
        }
        // s2: the B rows and the right-hand side
        RC(inf_assemble_b(c, s2));
        IB_CUDA_CHECK(cudaEventRecord(ev_b, s2));
        if (c->nt < c->nbody) IB_CUDA_CHECK(cudaMemsetAsync(c->rhsf, 0, 8 * (size_t)c->nf, s2));
        RC(launch_tors_rhs(c->nt, c->tb, c->ts, p.dt, c->delta, c->rhsf, s2));
        if (c->ub_on) RC(launch_sub_scaled(c->nf, c->delta, c->ub, c->rhsf, s2));
        if (c->sd.on) {   // P E_o (q + q0), P from s1
          IB_CUDA_CHECK(cudaStreamWaitEvent(s2, ev_p, 0));
          RC(launch_sd_rhs(c, c->rhsf, s2, false));
        } else {
          RC(launch_regT(g, c->nf, c->qx[0], c->q0x[0], c->qy[0], c->q0y[0], c->reg, c->rhsf, c->rhsf, s2));
        }
        IB_CUDA_CHECK(cudaEventRecord(ev_rhs, s2));
        // s3: a copy of the current origins and weights and their contribution lists
        RC(launch_reg_snapshot(c->nf, c->reg, c->reg_ix_s, c->reg_iy_s, c->reg_w_s, s3));
        RC(launch_reg_lists(c->nf, c->reg, g, s3));
        IB_CUDA_CHECK(cudaMemsetAsync(c->reg.stale, 0, sizeof(int), s3));   // for the weights below
        IB_CUDA_CHECK(cudaEventRecord(ev_lists, s3));
        // s1: assembly (the sub-domain's lumat from P and the B rows of s2) and solve
        if (c->sd.on) {   // lumat from P and the B rows, beside the right-hand side
          IB_CUDA_CHECK(cudaStreamWaitEvent(s1, ev_b, 0));
          RC(launch_sd_lumat(c, s1));
          IB_CUDA_CHECK(cudaStreamWaitEvent(s1, ev_rhs, 0));
        } else {
          RC(inf_assemble_kp(c, s1, true));
          IB_CUDA_CHECK(cudaStreamWaitEvent(s1, ev_rhs, 0));
          RC(inf_assemble_ptk(c, s1));
        }
        RC(launch_gmres_fused(c->G, &c->fused_plan, I.St, c->rhsf, c->f, p.rtol, p.atol, p.gmres_max_it, s1));
        // s2: redistribution with the copy, beside the structure update and the weights and
        // patches at the new positions on s1
        IB_CUDA_CHECK(cudaEventRecord(ev_f, s1));
        IB_CUDA_CHECK(cudaStreamWaitEvent(s2, ev_f, 0));
        IB_CUDA_CHECK(cudaStreamWaitEvent(s2, ev_lists, 0));
        RegDev snap = c->reg;
        snap.ix = c->reg_ix_s;
        snap.iy = c->reg_iy_s;
        snap.w = c->reg_w_s;
        c->st = s2;
        const int rrd = redistribute_with(c, snap, c->f, c->f_rdst);
        c->st = s1;
        RC(rrd);
        IB_CUDA_CHECK(cudaEventRecord(ev_rd, s2));
        // structure update, weights and patches at the new positions, the condition (after the
        // copy and the lists of the current weights are taken)
        IB_CUDA_CHECK(cudaStreamWaitEvent(s1, ev_lists, 0));
        I.patch_fresh = false;
        I.active = false;
        FsiUpdateArgs u;
        u.tb = c->tb; u.ts = c->ts; u.nt = c->nt; u.dt = p.dt; u.delta = c->delta; u.f = c->f;
        u.xb = c->xb; u.yb = c->yb; u.err = c->err_fsi;
        u.th_next = c->tors_next; u.sin_next = c->tors_next + (c->nt + 1); u.cos_next = c->tors_next + 2 * (c->nt + 1);
        u.g = g; u.nf = c->nf; u.ox = p.offsetx; u.oy = p.offsety; u.comp = c->reg.comp;
        u.ix = c->reg.ix; u.iy = c->reg.iy; u.w = c->reg.w; u.stale = c->reg.stale; u.d_err = c->d_err;
        u.tile_of = I.tile_of; u.ntx = I.ntx; u.tile = Influence::kTile;
        u.pval = c->sd.on ? nullptr : I.pval; u.pidx = I.pidx; u.used = I.used; u.flag = I.flag;
        u.rows = c->v2f_partial ? c->v2f_rows : nullptr;
        u.cnt = c->fsi_cnt; u.ist = c->G.ist; u.tol = p.fsi_tol; u.max_it = p.fsi_max_it; u.h = h;
        u.done = c->fsi_done;
        RC(launch_fsi_update(u, s1));
        IB_CUDA_CHECK(cudaStreamWaitEvent(s1, ev_rd, 0));   // the body ends with the redistribution
        return IB_OK;
      };
      rc = iteration();
      c->fsi_body_launches = launch_count() - b0;
      cudaGraph_t tmp;
      if (cudaStreamEndCapture(s1, &tmp) != cudaSuccess && rc == IB_OK) rc = IB_ERR_CUDA;
      c->st = st;
    }
    if (rc == IB_OK) {
      const long long a0 = launch_count();
      rc = launch_reg_lists(c->nf, c->reg, g, st);
      c->fsi_post_launches = launch_count() - a0;
    }
    if (rc == IB_OK) make_edges_programmatic(body);
  } while (false);
  c->st = st;
  for (cudaEvent_t e : ev)
    if (e) cudaEventDestroy(e);
  if (s3) cudaStreamDestroy(s3);
  if (s2) cudaStreamDestroy(s2);
  if (s1) cudaStreamDestroy(s1);
  return rc;
}

// The FSI iterations of a step as a graph of their own.
static int build_fsi_loop(Ctx* c) {
  cudaStream_t st = c->st;
  cudaGraph_t graph = nullptr;
  const long long l0 = launch_count();
  int rc = IB_OK;
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) != cudaSuccess) rc = IB_ERR_CUDA;
  if (rc == IB_OK) {
    rc = capture_fsi_loop(c, st);
    if (cudaStreamEndCapture(st, &graph) != cudaSuccess && rc == IB_OK) rc = IB_ERR_CUDA;
  }
  if (rc == IB_OK) make_edges_programmatic(graph);
  if (rc == IB_OK && cudaGraphInstantiate(&c->graph_fsi_loop.exec, graph, 0) != cudaSuccess) rc = IB_ERR_CUDA;
  count_launches(-(launch_count() - l0));   // captured, not run
  cudaGetLastError();
  if (graph) cudaGraphDestroy(graph);
  if (rc != IB_OK) {
    if (c->graph_fsi_loop.exec) cudaGraphExecDestroy(c->graph_fsi_loop.exec);
    c->graph_fsi_loop.exec = nullptr;
    c->graph_fsi_loop.failed = true;
  }
  return rc;
}

// The predictor of every level (timestepper.F90:103-236), coarse to fine.  Level k's solve
// depends on the coarser levels only through rhsbc's second ring, 0.25 get_bc(omega_{k+1})
// of the updated coarser vorticity, which enters on the boundary rows and columns.  So the
// nonlinear terms and the forward transforms (with the combine, the stencil, lastbc's part of
// rhsbc, and the copy of rhs into rhs_old) run as batched launches over all levels; then,
// coarse to fine in mode space, each level adds the transform of its second ring (closed form
// on interior rows, dot products on the two edge rows), solves its per-mode tridiagonal
// systems and evaluates the next finer level's ring from its modes at the points get_bc
// reads; one batched inverse pass writes every level's vorticity.
static int op_predict_levels(Ctx* c, bool seed_rhs_old) {
  const GridDims& g = c->g;
  const int L = c->L;
  cudaStream_t st = c->st;
  if (L > kMaxBatch) return IB_ERR_ARG;
  // lastbc from the vorticity before the update (zero on the coarsest level)
  RingBatch rb;
  for (int k = 0; k < L; ++k) {
    rb.src[k] = k < L - 1 ? c->omega[k + 1] : nullptr;
    rb.dst[k] = c->lastbc[k];
  }
  RC(launch_get_bc_levels(g, rb, L, 0.25, st));
  // nonlinear terms (operators_fluid.F90:553-587) and their rot, into rhs_lv
  NlBatch nb;
  for (int k = 0; k < L; ++k) {
    nb.om[k] = c->omega[k]; nb.bc[k] = c->lastbc[k];
    nb.qx[k] = c->qx[k]; nb.q0x[k] = c->q0x[k]; nb.qy[k] = c->qy[k]; nb.q0y[k] = c->q0y[k];
    nb.nlx[k] = c->mv_qx[k]; nb.nly[k] = c->mv_qy[k];
    nb.out[k] = c->rhs_lv[k];
  }
  RC(launch_nonlinear_rot_levels(g, nb, L, st));
  if (seed_rhs_old)   // the first step: rhs_old = rhs
    for (int k = 0; k < L; ++k)
      IB_CUDA_CHECK(cudaMemcpyAsync(c->rhs_old[k], c->rhs_lv[k], 8 * (size_t)g.ns, cudaMemcpyDeviceToDevice, st));
  {
    DstXArgs a;
    a.nlev = L;
    for (int k = 0; k < L; ++k) {
      const double cv = c->cvis[k];
      a.lin[k] = c->rhs_lv[k]; a.lin2[k] = c->rhs_old[k]; a.lsave[k] = c->rhs_old[k]; a.lin4[k] = c->omega[k];
      a.lring[k] = c->lastbc[k]; a.lfac[k] = c->vfac[k];
      a.lca[k] = c->con1[k]; a.lcb[k] = c->con2[k];
      a.lalpha[k] = (1.0 - 4.0 * cv) / c->normalize;
      a.lbeta[k] = cv / c->normalize;
      a.lout[k] = c->hat[k];
    }
    ProfScope ps(c, 0, pass_bytes(c, 4 * L, L));
    RC(dst_pass_x(c->px, g.nsy, g.nsx, PRE_PRED, a, g, c->lx_batch, st));
  }
  if (c->rmap.on) {
    RC(rm_predict(c));   // the same recursion with the chain of level solves collapsed
  } else {
    for (int k = L - 1; k >= 0; --k) {
      double* F = c->hat[k];
      // the second ring: ringv[k] = vfac[k] * 0.25 get_bc(omega_{k+1}), left by level k+1 with
      // its boundary terms, added by the solve
      TriBc bc;
      if (k < L - 1) bc = level_bc(c, k, 1.0);
      {
        ProfScope ps(c, 1, pass_bytes(c, 1, 1));
        RC(tri_solve(c->tri_pred[k], F, F, g.nsx, c->tl, st, bc));
      }
      if (k > 0) RC(ring_edge_from_modes(c, F, k - 1, 0.25 * c->vfac[k - 1]));
    }
  }
  // every row of every level back: coarsify rewrites only the centre columns of a coarser
  // level's centre rows, the rest of those rows (the coarse grid beside the finer one) is the
  // predictor's, read by the next step's nonlinear terms and get_bc and by vort2flux
  DstXArgs b;
  b.nlev = L;
  for (int k = 0; k < L; ++k) { b.lin[k] = c->hat[k]; b.lout[k] = c->omega[k]; }
  ProfScope ps(c, 0, pass_bytes(c, L, L));
  return dst_pass_x(c->px, g.nsy, g.nsx, PRE_COPY, b, g, c->lx_batch, st);
}

// timestepper.F90:18-556, in three parts so that a batch of contexts can put every context's
// work on the GPU before it waits for any (op_batch_advance):
//   begin:  predictor, vort2flux and, when the FSI iterations can run on the device, their
//           captured loop, launched without waiting;
//   end:    the loop's counters (the first wait), the host FSI iterations when needed, the
//           correction, and the error word's copy, launched without waiting;
//   finish: the error word and the solvers' status (the second wait).
int op_advance(Ctx* c) {
  RC(op_advance_begin(c));
  RC(op_advance_end(c));
  return op_advance_finish(c);
}

// The correction on the finest grid (timestepper.F90:488-553) after the forces are known.
static int op_correction(Ctx* c) {
  const GridDims& g = c->g;
  const int L = c->L;
  if (c->nf > 0) {
    // ainv of rot(E^T f): rot is formed as the x pass loads its rows (the face fields are
    // read inside the stencil box only, which E^T writes wholly), and the input is zero
    // outside the rows the stencils touch, so the forward transform runs on those rows
    // only (the others' modes are zero).  The solve negates its right-hand side on load, so
    // spec1 = -Y' (ainv's modes) exactly, and the inverse pass adds S_x(-Y') to omega_1 as
    // it stores: omega_1 - vort in one pass.
    // the sub-domain method spreads E_o^T P^T f instead (timestepper.F90:500-516)
    const int* box = c->sd.on ? c->sd.reg.bbox : c->reg.bbox;
    if (c->sd.on) RC(launch_sd_spread(c, c->f, c->hx, c->hy, c->st));
    else RC(launch_reg_box(g, c->nf, c->f, c->reg, c->hx, c->hy, c->st));
    DstXArgs a;
    a.in = c->hx; a.in2 = c->hy; a.box = box; a.out = c->spec1; a.rowrange = box + 4;
    RC(dst_pass_x(c->px, g.nsy, g.nsx, PRE_ROT, a, g, c->lx_small, c->st));
    TriBc neg;
    neg.post_scale = -1.0;
    RC(tri_solve(c->tri_ainv, c->spec1, c->spec1, g.nsx, c->tl, c->st, neg));
    DstXArgs b;
    b.in = c->spec1; b.out = c->omega[0]; b.post_add = c->omega[0]; b.post_scale = 1.0;
    RC(dst_pass_x(c->px, g.nsy, g.nsx, PRE_COPY, b, g, c->lx, c->st));
    // omega_1 was S_x Y (the predictor's modes, still in hat[0]): the corrected omega_1 has
    // modes Y - Y' = hat[0] + spec1, which the finest level's solve forms as it loads them
    return op_vort2flux(c, c->omega.data(), c->s.data(), c->qx.data(), c->qy.data(), true, L >= 2, true,
                        L >= 2 ? c->spec1 : nullptr);
  }
  RC(launch_reg(g, c->nf, c->f, c->reg, c->hx, c->hy, c->st));
  RC(launch_rot(g, c->hx, c->hy, c->vort, c->st));
  RC(op_ainv(c, c->vort, c->vort));
  RC(launch_sub(g.ns, c->omega[0], c->vort, c->omega[0], c->st));
  if (L >= 2) RC(launch_sub(g.ns, c->hat[0], c->spec1, c->hat[0], c->st));
  return op_vort2flux(c, c->omega.data(), c->s.data(), c->qx.data(), c->qy.data(), true, L >= 2, true);
}

// The stationary-body direct solve (timestepper.F90:457-490, num_stat): E q (less delta u_B
// of a prescribed motion), the Cholesky solve and the redistribution.
static int op_direct_solve(Ctx* c) {
  const GridDims& g = c->g;
  cudaStream_t st = c->st;
  if (c->ub_on) {   // -delta u_B of a prescribed motion, then E q accumulated onto it
    RC(launch_fill(c->nf, 0.0, c->rhsf, st));
    RC(launch_sub_scaled(c->nf, c->delta, c->ub, c->rhsf, st));
    RC(launch_regT(g, c->nf, c->qx[0], c->q0x[0], c->qy[0], c->q0y[0], c->reg, c->rhsf, c->rhsf, st));
  } else {
    RC(launch_regT(g, c->nf, c->qx[0], c->q0x[0], c->qy[0], c->q0y[0], c->reg, nullptr, c->rhsf, st));
  }
  RC(launch_chol_solve(c->nf, c->cholM, c->rhsf, c->f, st));
  return op_redistribute(c, c->f, c->f_rdst);
}

// ------------------------------------------------------------------ the step as one graph
// Opens the correction of a whole-step graph when the host FSI loop would add no iteration:
// the device loop stopped at the tolerance or at the cap (timestepper.F90:318), not at a band
// exit, and its residual is finite.  cnt[5] records the decision for the host.
__global__ void k_step_gate(int* cnt, const double* err, double tol, int max_it, cudaGraphConditionalHandle h) {
  IB_GRID_DEP_WAIT();
  const double e = err[0];
  const bool open = isfinite(e) && !(e >= tol && cnt[0] <= max_it);
  cnt[5] = open ? 1 : 0;
  cudaGraphSetConditional(h, open ? 1u : 0u);
}

// Which whole-step graph this step can run (0: none, the step runs phase by phase).  Mode 1
// needs every condition of the device FSI loop; mode 2 is a step with no host decision in it.
static int whole_step_mode(Ctx* c) {
  const IbParams& p = c->p;
  if (!c->use_whole_step || !c->use_step_graphs || c->prof_on || c->stage_on || c->step_prof ||
      c->graph_step.failed || c->itime < 2)
    return 0;
  if (c->nf == 0 || (p.num_stat && c->chol_ready)) return 2;
  if (p.num_stat) return 0;
  const Influence& I = c->inf;
  const bool operator_ready = c->sd.on ? c->sd.ready : (I.built && I.patch_fresh && I.flag_h == 0);
  const bool loop = (c->nt > 0) && c->nbeam == 0 && p.schur_mode != 1 && c->use_fused &&
                    !c->graph_fsi_loop.failed && c->fused_plan.state == 1 && operator_ready;
  return loop ? 1 : 0;
}

// Captures graph_step for `mode`: the predictor and first vort2flux of a step after the
// first (as graph_pred and graph_v2f), the forces, the correction (as graph_corr), and the
// copies the host reads when the step ends: in mode 1 the FSI loop's counters, its residual
// and the gate's decision, and the error word.
static int build_step_graph(Ctx* c, int mode) {
  const IbParams& p = c->p;
  cudaStream_t st = c->st, sc = nullptr;
  drop_phase(&c->graph_step);
  c->step_corr = PhaseGraph{};
  c->step_mode = mode;
  int rc = cudaStreamCreateWithFlags(&sc, cudaStreamNonBlocking) == cudaSuccess ? IB_OK : IB_ERR_CUDA;
  cudaGraph_t graph = nullptr;
  const long long l0 = launch_count();
  long long p0[4], p1[4], l1 = l0, loop_launches = 0;
  for (int i = 0; i < 4; ++i) p1[i] = p0[i] = c->n_pass[i];
  const bool prof = c->prof_on;
  do {
    if (rc != IB_OK) break;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) != cudaSuccess) { rc = IB_ERR_CUDA; break; }
    rc = op_predict_levels(c, false);
    if (rc == IB_OK)
      rc = op_vort2flux(c, c->omega.data(), c->s.data(), c->qx.data(), c->qy.data(), false, true, true);
    cudaGraphConditionalHandle h = 0;
    if (rc == IB_OK && mode == 1) {
      rc = launch_tors_save(c->nt, c->ts, st);
      const long long b0 = launch_count();
      Influence& I = c->inf;
      const bool fresh = I.patch_fresh, active = I.active;
      if (rc == IB_OK) rc = capture_fsi_loop(c, st);
      I.patch_fresh = fresh;   // what the capture recorded on the host for an iteration it did not run
      I.active = active;
      loop_launches = launch_count() - b0;
      if (rc == IB_OK &&
          cudaGraphConditionalHandleCreate(&h, capture_graph(st), 0, cudaGraphCondAssignDefault) != cudaSuccess)
        rc = IB_ERR_CUDA;
      if (rc == IB_OK) {
        count_launch();
        k_step_gate<<<1, 1, 0, st>>>(c->fsi_cnt, c->err_fsi, p.fsi_tol, p.fsi_max_it, h);
        if (cudaGetLastError() != cudaSuccess) rc = IB_ERR_CUDA;
      }
      if (rc == IB_OK &&
          (cudaMemcpyAsync(c->h_ist, c->fsi_cnt, 6 * sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
           cudaMemcpyAsync(c->h_scal, c->err_fsi, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess))
        rc = IB_ERR_CUDA;
    } else if (rc == IB_OK && c->nf > 0) {
      rc = op_direct_solve(c);
    }
    l1 = launch_count();
    for (int i = 0; i < 4; ++i) p1[i] = c->n_pass[i];
    if (rc == IB_OK && mode == 1) {
      cudaGraph_t body = nullptr;
      rc = add_conditional(st, h, cudaGraphCondTypeIf, &body);
      if (rc == IB_OK && cudaStreamBeginCaptureToGraph(sc, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) !=
                             cudaSuccess)
        rc = IB_ERR_CUDA;
      if (rc == IB_OK) {
        c->st = sc;
        rc = op_correction(c);
        c->st = st;
        cudaGraph_t tmp;
        if (cudaStreamEndCapture(sc, &tmp) != cudaSuccess && rc == IB_OK) rc = IB_ERR_CUDA;
        if (rc == IB_OK) make_edges_programmatic(body);
      }
    } else if (rc == IB_OK) {
      rc = op_correction(c);
    }
    c->step_corr.launches = launch_count() - l1;
    for (int i = 0; i < 4; ++i) c->step_corr.passes[i] = c->n_pass[i] - p1[i];
    if (rc == IB_OK &&
        cudaMemcpyAsync(c->h_ist + 12, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
      rc = IB_ERR_CUDA;
    if (cudaStreamEndCapture(st, &graph) != cudaSuccess && rc == IB_OK) rc = IB_ERR_CUDA;
    if (rc == IB_OK) make_edges_programmatic(graph);
    if (rc == IB_OK && cudaGraphInstantiate(&c->graph_step.exec, graph, 0) != cudaSuccess) rc = IB_ERR_CUDA;
  } while (false);
  c->st = st;
  c->prof_on = prof;
  c->graph_step.launches = (l1 - l0) - loop_launches;
  for (int i = 0; i < 4; ++i) {
    c->graph_step.passes[i] = p1[i] - p0[i];
    c->n_pass[i] = p0[i];   // captured, not run
  }
  count_launches(-(launch_count() - l0));
  cudaGetLastError();
  if (graph) cudaGraphDestroy(graph);
  if (sc) cudaStreamDestroy(sc);
  if (rc != IB_OK) {
    drop_phase(&c->graph_step);
    c->graph_step.failed = true;
  }
  return rc;
}

// Launches graph_step when this step can run as one graph; false leaves the step to the phases.
static bool launch_whole_step(Ctx* c) {
  const int mode = whole_step_mode(c);
  if (mode == 0) return false;
  if ((!c->graph_step.exec || c->step_mode != mode) && build_step_graph(c, mode) != IB_OK) return false;
  if (cudaGraphLaunch(c->graph_step.exec, c->st) != cudaSuccess) {
    cudaGetLastError();
    drop_phase(&c->graph_step);
    c->graph_step.failed = true;
    return false;
  }
  count_launches(c->graph_step.launches);
  for (int i = 0; i < 4; ++i) c->n_pass[i] += c->graph_step.passes[i];
  c->q0_partial = c->v2f_partial;
  if (mode == 1) {
    c->ksp_iter = 0;
    c->gmres_reason = 0;
    c->loop_pending = true;
  }
  c->step_pending = true;
  return true;
}

int op_advance_begin(Ctx* c) {
  const GridDims& g = c->g;
  const int L = c->L;
  const IbParams& p = c->p;
  cudaStream_t st = c->st;
  c->gmres_reason = 0;
  c->fsi_err_capped = 0.0;
  c->itime += 1;
  const int it = c->itime;
  // timestepper.F90:76 factorises at it == 1 only, so a num_stat restart (istart > 0) would
  // solve with a matrix never factorised; here the first step of a context factorises.
  if (p.num_stat && c->nf > 0 && !c->chol_ready) RC(preprocess_chol(c));
  // preprocess_sd (timestepper.F90:79-97): B at the first step unless it was read from a file
  if (c->sd.on && !c->sd.ready) RC(sd_precompute(c));
  if (launch_whole_step(c)) {
    c->n_step_graph += 1;
    c->end_pending = true;
    return IB_OK;
  }
  c->n_step_phased += 1;
  step_mark(c, 0);
  // boundary values of the previous step (timestepper.F90:103-117) and the predictor, coarse
  // to fine (timestepper.F90:121-236)
  auto predictor = [&]() -> int { return op_predict_levels(c, it == 1); };
  if (it == 1) RC(predictor());   // the first step also seeds rhs_old
  else RC(run_phase(c, c->graph_pred, predictor));
  step_mark(c, 1);
  // the FSI iterations read the finest level's fluxes only (timestepper.F90:240-245), and the
  // correction's vort2flux rewrites every level's streamfunction and fluxes before they are
  // read again: here the coarser levels are coarsified and solved in mode space only
  RC(run_phase(c, c->graph_v2f, [&]() {
    return op_vort2flux(c, c->omega.data(), c->s.data(), c->qx.data(), c->qy.data(), false, true, true);
  }));
  c->q0_partial = c->v2f_partial;
  step_mark(c, 2);
  // forces (timestepper.F90:249-486)
  if (c->nf > 0) {
    if (!p.num_stat) {
      if (it == 1) RC(launch_tors_initial_acc(c->nt, c->tb, c->ts, p.dt, c->delta, c->f, st));
      if (it == 1) RC(launch_beam_initial_acc(c, c->f, st));
      RC(launch_tors_save(c->nt, c->ts, st));
      RC(launch_beam_save(c, st));
      c->ksp_iter = 0;
      c->gmres_reason = 0;
      const bool moved = c->nt > 0 || c->nbeam > 0;
      // the iterations on the device while the operator stays assembled on a valid band (the
      // host loop below takes over when a patch leaves it, and runs every step that needs the
      // band built, the matrix-free operator or per-phase timing)
      {
        Influence& I = c->inf;
        const bool operator_ready = c->sd.on ? c->sd.ready : (I.built && I.patch_fresh && I.flag_h == 0);
        const bool device_loop = moved && p.schur_mode != 1 && c->use_step_graphs && c->use_fused && !c->prof_on &&
                                 !c->stage_on && (!c->step_prof || c->step_prof_dev) && c->nbeam == 0 &&
                                 !c->graph_fsi_loop.failed && c->fused_plan.state == 1 && operator_ready;
        if (device_loop && (c->graph_fsi_loop.exec || build_fsi_loop(c) == IB_OK)) {
          IB_CUDA_CHECK(cudaGraphLaunch(c->graph_fsi_loop.exec, st));
          IB_CUDA_CHECK(cudaMemcpyAsync(c->h_ist, c->fsi_cnt, 5 * sizeof(int), cudaMemcpyDeviceToHost, st));
          IB_CUDA_CHECK(cudaMemcpyAsync(c->h_scal, c->err_fsi, sizeof(double), cudaMemcpyDeviceToHost, st));
          c->loop_pending = true;
        }
      }
    }
  }
  c->end_pending = true;
  return IB_OK;
}

static int advance_end(Ctx* c);

// The step's end, then (once the host has asked for them) the copies of its outputs into
// pinned memory, queued before the step finishes (write_force2's values, operators_struct.F90:
// 711-731, and the hinge angles).
int op_advance_end(Ctx* c) {
  c->out_queued = false;
  RC(advance_end(c));
  if (!c->want_out) return IB_OK;
  // the coefficient kernel writes them, and the hinge angles, straight into the mapped buffer
  if (c->nbody > 0)
    RC(launch_force_coeffs(c->nf, c->nbody, c->comp, c->bid, c->f, c->p.dt, c->delta, c->forces, c->st, c->d_out,
                           c->ts.theta, c->nt));
  c->out_queued = true;
  return IB_OK;
}

static int advance_end(Ctx* c) {
  if (!c->end_pending) return IB_ERR_STATE;
  c->end_pending = false;
  const GridDims& g = c->g;
  const IbParams& p = c->p;
  cudaStream_t st = c->st;
  const int L = c->L;
  const bool whole = c->step_pending;
  c->step_pending = false;
  bool corr_done = false;
  if (whole && c->step_mode == 2) {   // the whole step is on the stream: its error word comes at the finish
    count_launches(c->step_corr.launches);
    for (int i = 0; i < 4; ++i) c->n_pass[i] += c->step_corr.passes[i];
    c->finish_pending = true;
    return IB_OK;
  }
  if (c->nf > 0) {
    if (!p.num_stat) {
      double err = 10.0;
      int fsi_count = 0;
      const bool moved = c->nt > 0 || c->nbeam > 0;
      {
        Influence& I = c->inf;
        if (c->loop_pending) {
          c->loop_pending = false;
          IB_CUDA_CHECK(cudaStreamSynchronize(st));
          if (c->step_prof) {
            step_mark(c, 3);
            cudaEventSynchronize(c->step_ev[3]);
            step_acc(c, 7, 2, 3);
          }
          fsi_count = c->h_ist[0];
          c->ksp_iter += c->h_ist[1];
          c->n_matvec += c->h_ist[2];
          count_launches(1 + c->fsi_body_launches * (long long)fsi_count + c->fsi_post_launches);
          I.assemblies += fsi_count;
          I.flag_h = c->h_ist[3] & 3;   // bit 4: a stencil left the rows of s computed (below)
          c->gmres_reason = std::min(c->gmres_reason, c->h_ist[4]);
          corr_done = whole && c->h_ist[5] != 0;   // the gate opened the correction in graph_step
          if (whole && !corr_done) c->n_step_gate_closed += 1;
          I.patch_fresh = true;
          I.active = false;
          err = c->h_scal[0];
          if (!std::isfinite(err)) return IB_ERR_NONFINITE;
        }
      }
      while (err >= p.fsi_tol && fsi_count <= p.fsi_max_it) {
        if (c->q0_partial) {
          // the host iterations read the finest fluxes at any stencil: complete s and q
          DstXArgs a;
          a.in = c->v2f_f0; a.out = c->s[0];
          RC(dst_pass_x(c->px, g.nsy, g.nsx, PRE_COPY, a, g, c->lx, st));
          RC(launch_curl(g, c->s[0], L == 1 ? c->zero_ring : c->ringv[0], c->qx[0], c->qy[0], st));
          c->q0_partial = false;
        }
        fsi_count += 1;
        step_mark(c, 3);
        RC(run_phase(c, c->graph_fsi_rhs, [&]() -> int {
          // k_tors_rhs writes every unknown of a torsional body: rigid bodies' start at zero
          if (c->nt < c->nbody) IB_CUDA_CHECK(cudaMemsetAsync(c->rhsf, 0, 8 * (size_t)c->nf, c->st));
          RC(launch_tors_rhs(c->nt, c->tb, c->ts, p.dt, c->delta, c->rhsf, c->st));
          RC(launch_beam_rhs(c, c->rhsf, c->st));
          // prescribed rigid-body motion (timestepper.F90:327-331): rhsf - delta u_B
          if (c->ub_on) RC(launch_sub_scaled(c->nf, c->delta, c->ub, c->rhsf, c->st));
          // sub-domain method (timestepper.F90:371-395): P E_o (q + q0) added to the structure's
          if (c->sd.on) return launch_sd_rhs(c, c->rhsf, c->st);
          return launch_regT(g, c->nf, c->qx[0], c->q0x[0], c->qy[0], c->q0y[0], c->reg, c->rhsf, c->rhsf, c->st);
        }));
        step_mark(c, 4);
        // Schur operator at the current positions: the band is valid and every patch lies in
        // it (checked at the end of the previous iteration) -> the captured assembly; else
        // the host path (build / rebuild / matrix-free fallback)
        Influence& I = c->inf;
        if (c->sd.on) {
          // compute_operator (timestepper.F90:377): lumat = body_mat + P B^T P^T, P as the
          // right-hand side formed it (the same positions)
          RC(sd_assemble(c, false));
          I.active = true;
        } else if (p.schur_mode != 1 && I.built && I.patch_fresh && I.flag_h == 0) {
          RC(run_phase(c, c->graph_fsi_asm, [&]() { return inf_assemble(c); }));
          I.assemblies += 1;
          I.active = true;
        } else {
          RC(inf_prepare(c));
        }
        step_mark(c, 5);
        // the cluster solver's counters come back with this iteration's synchronisation
        bool async = false;
        if (I.active && c->use_fused) {
          int rc = launch_gmres_fused(c->G, &c->fused_plan, I.St, c->rhsf, c->f, p.rtol, p.atol, p.gmres_max_it,
                                      c->st);
          if (rc == IB_OK) {
            IB_CUDA_CHECK(cudaMemcpyAsync(c->h_ist, c->G.ist, 8 * sizeof(int), cudaMemcpyDeviceToHost, st));
            async = true;
          } else if (rc != IB_ERR_ARG) {
            return rc;
          }
        }
        if (!async) {
          int its = 0, reason = 0;
          RC(op_gmres(c, c->rhsf, c->f, &its, &reason));
          c->ksp_iter += its;
          c->gmres_reason = std::min(c->gmres_reason, reason);
        }
        step_mark(c, 6);
        // redistribute, structure update, weights at the new positions and the next solve's
        // patches (checked against the band with the same synchronisation)
        const bool patch = moved && p.schur_mode != 1 && I.built;
        RC(run_phase(c, c->graph_fsi_upd, [&]() -> int {
          RC(op_redistribute(c, c->f, c->f_rdst));
          RC(launch_tors_dx(c->nt, c->tb, c->ts, p.dt, c->delta, c->f, c->xb, c->yb, c->err_fsi, c->st));
          RC(launch_beam_dx(c, c->f, c->st));
          if (moved) RC(op_reg_prep(c));
          if (patch) {
            RC(inf_patch(c));
            IB_CUDA_CHECK(cudaMemcpyAsync(I.h_flag, I.flag, sizeof(int), cudaMemcpyDeviceToHost, c->st));
          }
          IB_CUDA_CHECK(cudaMemcpyAsync(c->h_scal, c->err_fsi, sizeof(double), cudaMemcpyDeviceToHost, c->st));
          return IB_OK;
        }));
        if (moved) {   // what op_reg_prep records on the host (not replayed by the graph)
          I.patch_fresh = false;
          I.active = false;
        }
        step_mark(c, 7);
        IB_CUDA_CHECK(cudaStreamSynchronize(st));
        step_acc(c, 2, 3, 4);
        step_acc(c, 3, 4, 5);
        step_acc(c, 4, 5, 6);
        step_acc(c, 5, 6, 7);
        if (async) {
          c->ksp_iter += c->h_ist[0];
          c->n_matvec += c->h_ist[0] + c->h_ist[4];
          c->gmres_reason = std::min(c->gmres_reason, c->h_ist[1]);
        }
        if (patch) {
          I.flag_h = I.h_flag[0];
          I.patch_fresh = true;
        }
        err = c->h_scal[0];
        if (!std::isfinite(err)) return IB_ERR_NONFINITE;
      }
      c->fsi_iter = fsi_count;
      // the loop of timestepper.F90:318 ends at fsi_max_it + 1 iterations without reaching
      // fsi_tol; the reference carries on silently, this step reports it (after finishing)
      c->fsi_err_capped = err >= p.fsi_tol ? err : 0.0;
    } else {
      RC(op_direct_solve(c));
    }
  }
  // correction on the finest grid (timestepper.F90:488-553)
  step_mark(c, 8);
  if (corr_done) {   // graph_step has run it and copied the error word
    count_launches(c->step_corr.launches);
    for (int i = 0; i < 4; ++i) c->n_pass[i] += c->step_corr.passes[i];
  } else {
    RC(run_phase(c, c->graph_corr, [&]() { return op_correction(c); }));
    step_mark(c, 9);
    IB_CUDA_CHECK(cudaMemcpyAsync(c->h_ist + 12, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  }
  c->finish_pending = true;
  return IB_OK;
}

int op_advance_finish(Ctx* c) {
  if (!c->finish_pending) return IB_ERR_STATE;
  c->finish_pending = false;
  IB_CUDA_CHECK(cudaStreamSynchronize(c->st));
  int rc = c->h_ist[12];
  if (rc) IB_CUDA_CHECK(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->st));
  // the step is complete either way; a Krylov solve that stopped without converging, or an
  // FSI loop that stopped at its cap, is reported once the state is consistent
  if (rc == IB_OK && c->gmres_reason < 0) rc = IB_ERR_GMRES;
  else if (rc == IB_OK && c->fsi_err_capped > 0.0) rc = IB_ERR_FSI;
  if (c->step_prof) {
    step_acc(c, 0, 0, 1);
    step_acc(c, 1, 1, 2);
    step_acc(c, 6, 8, 9);
    c->step_n += 1;
  }
  return rc;
}

}  // namespace ib
