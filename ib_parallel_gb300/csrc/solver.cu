// The time step of timestepper.F90:18-556 and the composite operators it calls,
// orchestrated on one CUDA stream over device-resident state.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>

#include "ctx.cuh"

namespace ib {

#define RC(x)                   \
  do {                          \
    int _rc = (x);              \
    if (_rc != IB_OK) return _rc; \
  } while (0)

static const double kPi = 4.0 * std::atan(1.0);  // parameters.F90:61

static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
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

// ------------------------------------------------------------- DST tuning
static int time_pass(Ctx* c, int which, const DstLaunch& L, float* ms) {
  cudaEvent_t e0, e1;
  IB_CUDA_CHECK(cudaEventCreate(&e0));
  IB_CUDA_CHECK(cudaEventCreate(&e1));
  auto run = [&]() -> int {
    if (which == 0) {
      DstXArgs a; a.in = c->spec2; a.out = c->spec1;
      return dst_pass_x(c->px, c->g.nsy, c->g.nsx, PRE_COPY, a, c->g, L, c->st);
    }
    DstYArgs a; a.a = c->spec1; a.b = c->spec2; a.t1 = c->laminv; a.t2 = c->laminv;
    DstYMode m = which == 1 ? YMODE_DIAG : (which == 2 ? YMODE_PRED : YMODE_NONE);
    return dst_pass_y(c->py, c->g.nsx, c->g.nsx, m, a, L, c->st);
  };
  RC(run());
  IB_CUDA_CHECK(cudaEventRecord(e0, c->st));
  for (int r = 0; r < 3; ++r) RC(run());
  IB_CUDA_CHECK(cudaEventRecord(e1, c->st));
  IB_CUDA_CHECK(cudaEventSynchronize(e1));
  IB_CUDA_CHECK(cudaEventElapsedTime(ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return IB_OK;
}

static int tune_dst(Ctx* c) {
  int dev = 0, smem_max = 0;
  IB_CUDA_CHECK(cudaGetDevice(&dev));
  IB_CUDA_CHECK(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  IB_CUDA_CHECK(cudaMemsetAsync(c->spec1, 0, sizeof(double) * c->g.ns, c->st));
  IB_CUDA_CHECK(cudaMemsetAsync(c->spec2, 0, sizeof(double) * c->g.ns, c->st));
  const int Bs[] = {1, 2, 3, 4, 5, 6, 8, 10, 12, 16};
  const int NTs[] = {32, 64, 96, 128, 160, 192, 256, 320, 384, 512};
  DstLaunch* outs[4] = {&c->lx, &c->ly_diag, &c->ly_pred, &c->ly_none};
  for (int which = 0; which < 4; ++which) {
    const DstPlan& pl = which == 0 ? c->px : c->py;
    float best = 1e30f;
    DstLaunch bestL = *outs[which];
    for (int B : Bs) {
      size_t smem = which == 0 ? dst_smem_x(pl, B)
                               : dst_smem_y(pl, B, which == 2 ? YMODE_PRED : YMODE_DIAG);
      if ((long long)smem > smem_max) continue;
      int nlines = which == 0 ? c->g.nsy : c->g.nsx;
      if (B > nlines) continue;
      for (int NT : NTs) {
        if (NT > 32 * B * 8) continue;  // more than 8 warps per line never helps
        DstLaunch L; L.B = B; L.NT = NT;
        float ms = 0;
        if (time_pass(c, which, L, &ms) != IB_OK) { cudaGetLastError(); continue; }
        if (ms < best) { best = ms; bestL = L; }
      }
    }
    *outs[which] = bestL;
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
    if (b.fam != 1 && b.fam != 2) { *msg = "body family must be 1 (rigid) or 2 (torsional)"; return IB_ERR_ARG; }
    if (b.fam == 2 && !(b.itheta > 0)) { *msg = "torsional body needs itheta > 0"; return IB_ERR_ARG; }
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
  dbl += (size_t)L * (2 * ns + nu + nv);                 // Schur scratch
  dbl += (size_t)(2 + 2 * L) * ns;                       // tables
  dbl += 5 * ns + 2 * nu + 2 * nv;                       // work
  dbl += (size_t)(L + 3) * nbc;                          // rings
  dbl += 7 * (size_t)nf + 2 * (size_t)nbody + 49 * (size_t)nf;
  dbl += 6 * (size_t)nt + nt + 1;
  dbl += (size_t)(R + 1) * nf + (size_t)(R + 1) * R + 3 * (R + 1) + 4 + 2 * (size_t)nf;
  if (p.num_stat) dbl += (size_t)nf * nf;
  dbl += 8 * stage_n;
  size_t ints = 2 * (size_t)nf + 2 * (size_t)nf + 4 + 2 * (size_t)max_faces + 2 * 49 * (size_t)nf + 4 + 1;
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
  lv(c->omega, ns); lv(c->s, ns); lv(c->rhs_old, ns);
  lv(c->qx, nu); lv(c->q0x, nu); lv(c->qy, nv); lv(c->q0y, nv);
  lv(c->mv_w, ns); lv(c->mv_s, ns); lv(c->mv_qx, nu); lv(c->mv_qy, nv);
  c->laminv = P.take<double>(ns); c->lam1i_n = P.take<double>(ns);
  lv(c->lam1, ns); lv(c->lam1i, ns);
  c->spec1 = P.take<double>(ns); c->spec2 = P.take<double>(ns); c->rhs = P.take<double>(ns);
  c->rhsbc = P.take<double>(ns); c->vort = P.take<double>(ns);
  c->nlx = P.take<double>(nu); c->hx = P.take<double>(nu);
  c->nly = P.take<double>(nv); c->hy = P.take<double>(nv);
  lv(c->lastbc, nbc);
  c->omegabc = P.take<double>(nbc); c->sbc = P.take<double>(nbc); c->zero_ring = P.take<double>(nbc);
  c->f = P.take<double>(nf); c->f_rdst = P.take<double>(nf); c->xb = P.take<double>(nf);
  c->yb = P.take<double>(nf); c->rhsf = P.take<double>(nf); c->tmpf = P.take<double>(nf);
  c->tmpf2 = P.take<double>(nf); c->forces = P.take<double>(2 * nbody + 1);
  c->comp = P.take<int>(nf); c->bid = P.take<int>(nf);
  c->reg.comp = c->comp; c->reg.ix = P.take<int>(nf); c->reg.iy = P.take<int>(nf);
  c->reg.w = P.take<double>(49 * (size_t)nf); c->reg.bbox = P.take<int>(4);
  c->reg.cnt_x = P.take<int>(max_faces); c->reg.cnt_y = P.take<int>(max_faces);
  c->reg.lst_x = P.take<int>(49 * (size_t)nf + 1); c->reg.lst_y = P.take<int>(49 * (size_t)nf + 1);
  c->reg.max_faces = max_faces; c->reg.max_list = 49 * nf;
  c->tb = P.take<TorsBody>(nt + 1);
  c->ts.theta = P.take<double>(nt + 1); c->ts.thetad = P.take<double>(nt + 1);
  c->ts.thetadd = P.take<double>(nt + 1); c->ts.theta0 = P.take<double>(nt + 1);
  c->ts.thetad0 = P.take<double>(nt + 1); c->ts.thetadd0 = P.take<double>(nt + 1);
  c->err_fsi = P.take<double>(nt + 1);
  c->G.nf = nf; c->G.restart = R;
  c->G.V = P.take<double>((size_t)(R + 1) * nf); c->G.H = P.take<double>((size_t)(R + 1) * R);
  c->G.cs = P.take<double>(R + 1); c->G.sn = P.take<double>(R + 1); c->G.g = P.take<double>(R + 1);
  c->G.scal = P.take<double>(4); c->G.ist = P.take<int>(4);
  c->G.xin = P.take<double>(nf); c->G.Av = P.take<double>(nf);
  if (p.num_stat) c->cholM = P.take<double>((size_t)nf * nf);
  c->d_err = P.take<int>(1);
  c->stage_n = stage_n;
  for (int i = 0; i < 8; ++i) c->stage[i] = P.take<double>(stage_n);
  if (!c->stage[7] || !c->d_err) { *msg = "internal pool overflow"; ctx_destroy(c); return IB_ERR_NOMEM; }
  if (cudaMallocHost(&c->h_ist, 4 * sizeof(int)) != cudaSuccess ||
      cudaMallocHost(&c->h_scal, 4 * sizeof(double)) != cudaSuccess) {
    *msg = "pinned allocation failed"; ctx_destroy(c); return IB_ERR_NOMEM;
  }

  c->prof_ev.resize(2 * Ctx::kProfMax);
  c->prof_kind.resize(Ctx::kProfMax);
  c->prof_bytes.resize(Ctx::kProfMax);
  for (auto& e : c->prof_ev) IB_CUDA_CHECK(cudaEventCreate(&e));

  // spectral tables (myfft.F90:125-148)
  {
    std::vector<double> lam(ns), t1(ns), t2(ns);
    for (int J = 2; J <= g.n; ++J)
      for (int I = 2; I <= g.m; ++I) {
        size_t q = (size_t)(J - 2) * g.nsx + (I - 2);
        lam[q] = -2.0 * (std::cos(kPi * (double)(I - 1) / (double)g.m) + std::cos(kPi * (double)(J - 1) / (double)g.n) - 2.0);
        t1[q] = 1.0 / lam[q] / c->normalize;
      }
    IB_CUDA_CHECK(cudaMemcpy(c->laminv, t1.data(), 8 * ns, cudaMemcpyHostToDevice));
    double del2 = c->delta * c->delta;
    for (int k = 1; k <= L; ++k) {
      double del22 = del2 * std::pow(4.0, k - 1);
      c->vfac.push_back(0.5 * p.dt / p.Re / del22 / c->normalize);
      c->con1.push_back(1.5 * p.dt / del22 / c->normalize);
      c->con2.push_back(-0.5 * p.dt / del22 / c->normalize);
      for (size_t q = 0; q < ns; ++q) {
        t1[q] = (1.0 - 0.5 * p.dt * lam[q] / del22 / p.Re) / c->normalize;
        t2[q] = 1.0 / (1.0 + 0.5 * p.dt * lam[q] / del22 / p.Re);
      }
      IB_CUDA_CHECK(cudaMemcpy(c->lam1[k - 1], t1.data(), 8 * ns, cudaMemcpyHostToDevice));
      IB_CUDA_CHECK(cudaMemcpy(c->lam1i[k - 1], t2.data(), 8 * ns, cudaMemcpyHostToDevice));
      if (k == 1) {
        for (size_t q = 0; q < ns; ++q) t1[q] = t2[q] / c->normalize;
        IB_CUDA_CHECK(cudaMemcpy(c->lam1i_n, t1.data(), 8 * ns, cudaMemcpyHostToDevice));
      }
    }
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
  for (int i = 0; i < nbody; ++i) c->bodies_h.push_back(bodies[i]);

  // default launch shapes, then tuned by timing
  c->lx.B = 2; c->lx.NT = 160;
  c->ly_none.B = 8; c->ly_none.NT = 160;
  c->ly_diag.B = 8; c->ly_diag.NT = 160;
  c->ly_pred.B = 4; c->ly_pred.NT = 160;
  if (p.autotune) {
    rc = tune_dst(c);
    if (rc != IB_OK) { *msg = "DST tuning failed"; ctx_destroy(c); return rc; }
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
  if (c->pool.base) cudaFree(c->pool.base);
  if (c->h_ist) cudaFreeHost(c->h_ist);
  if (c->h_scal) cudaFreeHost(c->h_scal);
  for (auto& e : c->prof_ev)
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
static int ctci_like(Ctx* c, const double* in, double* out, const double* ring, const double* table) {
  DstXArgs a;
  a.in = in; a.out = c->spec1; a.ring = ring; a.fac = 1.0;
  {
    ProfScope ps(c, 0, pass_bytes(c, 1, 1));
    RC(dst_pass_x(c->px, c->g.nsy, c->g.nsx, ring ? PRE_APPLYBC : PRE_COPY, a, c->g, c->lx, c->st));
  }
  DstYArgs y;
  y.a = c->spec1; y.t1 = table;
  {
    ProfScope ps(c, 1, pass_bytes(c, 2, 1));
    RC(dst_pass_y(c->py, c->g.nsx, c->g.nsx, YMODE_DIAG, y, c->ly_diag, c->st));
  }
  DstXArgs b;
  b.in = c->spec1; b.out = out;
  ProfScope ps(c, 0, pass_bytes(c, 1, 1));
  return dst_pass_x(c->px, c->g.nsy, c->g.nsx, PRE_COPY, b, c->g, c->lx, c->st);
}

int op_ctci(Ctx* c, const double* in, double* out, const double* ring) { return ctci_like(c, in, out, ring, c->laminv); }
int op_ainv(Ctx* c, const double* in, double* out) { return ctci_like(c, in, out, nullptr, c->lam1i_n); }

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

// omega = dst(lam1i*(dst(con1 rhs + con2 rhs_old + rhsbc) + lam1*dst(omega)))  (operators_fluid.F90:649-663)
int op_predictor(Ctx* c, int k, double* om, const double* rhs, const double* rhs_old, const double* rhsbc) {
  DstXArgs a;
  a.in = rhs; a.in2 = rhs_old; a.in3 = rhsbc; a.ca = c->con1[k]; a.cb = c->con2[k]; a.out = c->spec1;
  {
    ProfScope ps(c, 0, pass_bytes(c, 3, 1));
    RC(dst_pass_x(c->px, c->g.nsy, c->g.nsx, PRE_COMBINE, a, c->g, c->lx, c->st));
  }
  DstXArgs b;
  b.in = om; b.out = c->spec2;
  {
    ProfScope ps(c, 0, pass_bytes(c, 1, 1));
    RC(dst_pass_x(c->px, c->g.nsy, c->g.nsx, PRE_COPY, b, c->g, c->lx, c->st));
  }
  DstYArgs y;
  y.a = c->spec1; y.b = c->spec2; y.t1 = c->lam1i[k]; y.t2 = c->lam1[k];
  {
    ProfScope ps(c, 2, pass_bytes(c, 4, 1));
    RC(dst_pass_y(c->py, c->g.nsx, c->g.nsx, YMODE_PRED, y, c->ly_pred, c->st));
  }
  DstXArgs d;
  d.in = c->spec1; d.out = om;
  ProfScope ps(c, 0, pass_bytes(c, 1, 1));
  return dst_pass_x(c->px, c->g.nsy, c->g.nsx, PRE_COPY, d, c->g, c->lx, c->st);
}

// vort2flux (operators_fluid.F90:237-377).  all_curls=false computes the fluxes
// of the finest level only (the Schur operator reads nothing else).
int op_vort2flux(Ctx* c, double* const* w, double* const* s, double* const* qx, double* const* qy, bool all_curls) {
  const int L = c->L;
  const GridDims& g = c->g;
  for (int k = 1; k < L; ++k) RC(launch_coarsify(g, w[k - 1], w[k], c->st));
  RC(op_ctci(c, w[L - 1], s[L - 1], nullptr));
  if (all_curls || L == 1) RC(launch_curl(g, s[L - 1], c->zero_ring, qx[L - 1], qy[L - 1], c->st));
  if (L > 1) RC(launch_get_bc(g, s[L - 1], 1.0, c->sbc, c->st));
  for (int k = L - 2; k >= 0; --k) {
    RC(op_ctci(c, w[k], s[k], c->sbc));
    if (all_curls || k == 0) RC(launch_curl(g, s[k], c->sbc, qx[k], qy[k], c->st));
    if (k > 0) RC(launch_get_bc(g, s[k], 1.0, c->sbc, c->st));
  }
  return IB_OK;
}

// ab_times / a_times2 (timestepper.F90:774-782, operators_fluid.F90:14-120)
int op_schur(Ctx* c, const double* x, double* y, bool with_b) {
  const GridDims& g = c->g;
  c->n_matvec += 1;
  RC(launch_reg(g, c->nf, x, c->reg, c->hx, c->hy, c->st));
  RC(launch_rot(g, c->hx, c->hy, c->mv_w[0], c->st));
  RC(op_ainv(c, c->mv_w[0], c->mv_w[0]));
  for (int k = 1; k < c->L; ++k) IB_CUDA_CHECK(cudaMemsetAsync(c->mv_w[k], 0, 8 * (size_t)g.ns, c->st));
  RC(op_vort2flux(c, c->mv_w.data(), c->mv_s.data(), c->mv_qx.data(), c->mv_qy.data(), false));
  RC(launch_regT(g, c->nf, c->mv_qx[0], nullptr, c->mv_qy[0], nullptr, c->reg, nullptr, y, c->st));
  if (with_b) RC(launch_tors_btimes(c->nt, c->tb, c->ts, c->p.dt, c->delta, x, y, c->st));
  return IB_OK;
}

int op_redistribute(Ctx* c, const double* f, double* frdst) {
  RC(launch_redistribute_field(c->g, c->nf, f, c->reg, c->nlx, c->nly, c->st));
  return launch_regT(c->g, c->nf, c->nlx, nullptr, c->nly, nullptr, c->reg, nullptr, frdst, c->st);
}

int op_reg_prep(Ctx* c) {
  return launch_reg_build(c->g, c->nf, c->xb, c->yb, c->delta, c->p.offsetx, c->p.offsety, c->reg, c->d_err, c->st);
}

static int read_ist(Ctx* c) {
  IB_CUDA_CHECK(cudaMemcpyAsync(c->h_ist, c->G.ist, 4 * sizeof(int), cudaMemcpyDeviceToHost, c->st));
  IB_CUDA_CHECK(cudaStreamSynchronize(c->st));
  return IB_OK;
}

// KSPSolve with KSPGMRES (timestepper.F90:363-366); x is the initial guess.
int op_gmres(Ctx* c, const double* b, double* x, int* its, int* reason) {
  const GmresDev& G = c->G;
  const int max_it = c->p.gmres_max_it;
  RC(launch_gmres_init(G, c->st));
  for (;;) {
    IB_CUDA_CHECK(cudaMemcpyAsync(G.xin, x, 8 * (size_t)c->nf, cudaMemcpyDeviceToDevice, c->st));
    RC(op_schur(c, G.xin, G.Av, true));
    RC(launch_gmres_start(G, b, x, c->p.rtol, c->p.atol, max_it, c->st));
    RC(read_ist(c));
    if (c->h_ist[1] != 0) break;
    for (;;) {
      RC(op_schur(c, G.xin, G.Av, true));
      RC(launch_gmres_arnoldi(G, max_it, c->st));
      RC(read_ist(c));
      if (!c->h_ist[3]) break;
    }
    RC(launch_gmres_update(G, x, c->st));
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

// timestepper.F90:18-556
int op_advance(Ctx* c) {
  const GridDims& g = c->g;
  const int L = c->L;
  const IbParams& p = c->p;
  cudaStream_t st = c->st;
  c->itime += 1;
  const int it = c->itime;
  if (it == 1 && p.num_stat && c->nf > 0) RC(preprocess_chol(c));
  // boundary values of the previous step (timestepper.F90:103-117)
  for (int k = 0; k < L - 1; ++k) RC(launch_get_bc(g, c->omega[k + 1], 0.25, c->lastbc[k], st));
  IB_CUDA_CHECK(cudaMemsetAsync(c->lastbc[L - 1], 0, 8 * (size_t)g.nbc, st));
  // predictor, coarse to fine (timestepper.F90:121-236)
  for (int k = L - 1; k >= 0; --k) {
    const double* obc = c->zero_ring;
    if (k < L - 1) {
      RC(launch_get_bc(g, c->omega[k + 1], 0.25, c->omegabc, st));
      obc = c->omegabc;
    }
    RC(launch_nonlinear(g, c->omega[k], c->lastbc[k], c->qx[k], c->q0x[k], c->qy[k], c->q0y[k], c->nlx, c->nly, st));
    RC(launch_rhsbc(g, c->rhsbc, c->lastbc[k], obc, c->vfac[k], st));
    RC(launch_rot(g, c->nlx, c->nly, c->rhs, st));
    if (it == 1) IB_CUDA_CHECK(cudaMemcpyAsync(c->rhs_old[k], c->rhs, 8 * (size_t)g.ns, cudaMemcpyDeviceToDevice, st));
    RC(op_predictor(c, k, c->omega[k], c->rhs, c->rhs_old[k], c->rhsbc));
    IB_CUDA_CHECK(cudaMemcpyAsync(c->rhs_old[k], c->rhs, 8 * (size_t)g.ns, cudaMemcpyDeviceToDevice, st));
  }
  RC(op_vort2flux(c, c->omega.data(), c->s.data(), c->qx.data(), c->qy.data(), true));
  // forces (timestepper.F90:249-486)
  if (c->nf > 0) {
    if (!p.num_stat) {
      if (it == 1) RC(launch_tors_initial_acc(c->nt, c->tb, c->ts, p.dt, c->delta, c->f, st));
      RC(launch_tors_save(c->nt, c->ts, st));
      double err = 10.0;
      int fsi_count = 0;
      c->ksp_iter = 0;
      while (err >= p.fsi_tol && fsi_count <= p.fsi_max_it) {
        fsi_count += 1;
        IB_CUDA_CHECK(cudaMemsetAsync(c->rhsf, 0, 8 * (size_t)c->nf, st));
        RC(launch_tors_rhs(c->nt, c->tb, c->ts, p.dt, c->delta, c->rhsf, st));
        RC(launch_regT(g, c->nf, c->qx[0], c->q0x[0], c->qy[0], c->q0y[0], c->reg, c->rhsf, c->rhsf, st));
        int its = 0, reason = 0;
        RC(op_gmres(c, c->rhsf, c->f, &its, &reason));
        c->ksp_iter += its;
        RC(op_redistribute(c, c->f, c->f_rdst));
        RC(launch_tors_dx(c->nt, c->tb, c->ts, p.dt, c->delta, c->f, c->xb, c->yb, c->err_fsi, st));
        if (c->nt > 0) RC(op_reg_prep(c));
        IB_CUDA_CHECK(cudaMemcpyAsync(c->h_scal, c->err_fsi, sizeof(double), cudaMemcpyDeviceToHost, st));
        IB_CUDA_CHECK(cudaStreamSynchronize(st));
        err = c->h_scal[0];
        if (!std::isfinite(err)) return IB_ERR_NONFINITE;
      }
      c->fsi_iter = fsi_count;
    } else {
      RC(launch_regT(g, c->nf, c->qx[0], c->q0x[0], c->qy[0], c->q0y[0], c->reg, nullptr, c->rhsf, st));
      RC(launch_chol_solve(c->nf, c->cholM, c->rhsf, c->f, st));
      RC(op_redistribute(c, c->f, c->f_rdst));
    }
  }
  // correction on the finest grid (timestepper.F90:488-553)
  RC(launch_reg(g, c->nf, c->f, c->reg, c->hx, c->hy, st));
  RC(launch_rot(g, c->hx, c->hy, c->vort, st));
  RC(op_ainv(c, c->vort, c->vort));
  RC(launch_sub(g.ns, c->omega[0], c->vort, c->omega[0], st));
  RC(op_vort2flux(c, c->omega.data(), c->s.data(), c->qx.data(), c->qy.data(), true));
  return check_err(c);
}

}  // namespace ib
