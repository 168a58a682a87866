// extern "C" entry points of include/ib_gpu.h.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.cuh"

using ib::Ctx;

static thread_local std::string g_err;

static int fail(int rc, const char* what) {
  g_err = what;
  return rc;
}

namespace ib {
void set_last_error(const char* msg) { g_err = msg; }
}  // namespace ib

struct IbCtx {
  Ctx* c;
  bool borrowed = false;   // a batch's simulation (ib_batch_context): the batch owns it
};

namespace {

bool is_device(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Resolves an argument array to device memory: device pointers are used in
// place, host arrays are copied into (and, for outputs, back from) one of the
// context's staging buffers.
struct Staging {
  Ctx* c;
  int next = 0;
  struct Out { double* dev; double* host; size_t n; };
  Out outs[8];
  int nout = 0;
  int rc = IB_OK;
  explicit Staging(Ctx* cc) : c(cc) {}
  double* in(const double* p, size_t n) {
    if (!p) { rc = IB_ERR_ARG; return nullptr; }
    if (is_device(p)) return const_cast<double*>(p);
    if (next >= 8 || n > c->stage_n) { rc = IB_ERR_ARG; return nullptr; }
    double* d = c->stage[next++];
    if (cudaMemcpyAsync(d, p, 8 * n, cudaMemcpyHostToDevice, c->st) != cudaSuccess) rc = IB_ERR_CUDA;
    return d;
  }
  double* out(double* p, size_t n, bool copy_in) {
    if (!p) { rc = IB_ERR_ARG; return nullptr; }
    if (is_device(p)) return p;
    if (next >= 8 || n > c->stage_n) { rc = IB_ERR_ARG; return nullptr; }
    double* d = c->stage[next++];
    if (copy_in && cudaMemcpyAsync(d, p, 8 * n, cudaMemcpyHostToDevice, c->st) != cudaSuccess) rc = IB_ERR_CUDA;
    outs[nout++] = {d, p, n};
    return d;
  }
  int finish(int op_rc) {
    if (op_rc != IB_OK) { cudaStreamSynchronize(c->st); return op_rc; }
    for (int i = 0; i < nout; ++i)
      if (cudaMemcpyAsync(outs[i].host, outs[i].dev, 8 * outs[i].n, cudaMemcpyDeviceToHost, c->st) != cudaSuccess)
        return IB_ERR_CUDA;
    if (cudaStreamSynchronize(c->st) != cudaSuccess) return IB_ERR_CUDA;
    return IB_OK;
  }
};

// Every entry point but the step's output getters may change the state: the pinned copy of the
// last step's outputs stops being the state's.
#define CTX_OR_FAIL(h)                                             \
  if (!(h) || !(h)->c) return fail(IB_ERR_ARG, "null context");    \
  Ctx* c = (h)->c;                                                 \
  c->out_fresh = false;
#define CTX_OR_FAIL_KEEP(h)                                        \
  if (!(h) || !(h)->c) return fail(IB_ERR_ARG, "null context");    \
  Ctx* c = (h)->c;

#define STAGE_CHECK(S) \
  if ((S).rc != IB_OK) return fail((S).rc, "bad array argument");

int op_result(int rc, const char* what) {
  if (rc != IB_OK) {
    cudaError_t e = cudaGetLastError();
    std::string m = what;
    if (e != cudaSuccess) m += std::string(": ") + cudaGetErrorString(e);
    return fail(rc, m.c_str());
  }
  return IB_OK;
}

}  // namespace

extern "C" {

const char* ib_last_error(void) { return g_err.c_str(); }
int ib_version(void) { return 1; }

int ib_create(const IbParams* p, const IbBody* bodies, int nbody, IbCtx** out) {
  if (!p || !out) return fail(IB_ERR_ARG, "null argument");
  std::string msg;
  Ctx* c = nullptr;
  int rc = ib::ctx_create(p, bodies, nbody, &c, &msg);
  if (rc != IB_OK) return fail(rc, msg.c_str());
  *out = new IbCtx{c};
  return IB_OK;
}

int ib_destroy(IbCtx* h) {
  if (!h) return IB_OK;
  if (h->borrowed) return fail(IB_ERR_ARG, "the context belongs to a batch: ib_batch_destroy frees it");
  ib::ctx_destroy(h->c);
  delete h;
  return IB_OK;
}

int ib_synchronize(IbCtx* h) {
  CTX_OR_FAIL(h);
  if (cudaStreamSynchronize(c->st) != cudaSuccess) return fail(IB_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
  return IB_OK;
}

int ib_advance(IbCtx* h, int* itime) {
  CTX_OR_FAIL(h);
  int rc = ib::op_advance(c);
  // the step is complete (possibly with a solver that stopped short): its outputs are in place
  c->out_fresh = c->out_queued && (rc == IB_OK || rc == IB_ERR_GMRES || rc == IB_ERR_FSI);
  if (itime) *itime = c->itime;
  if (rc == IB_ERR_GMRES) {
    std::string m = "advance: the step is complete, but a Krylov solve stopped without converging (KSP reason " +
                    std::to_string(c->gmres_reason) + ")";
    return fail(rc, m.c_str());
  }
  if (rc == IB_ERR_FSI) {
    std::string m = "advance: the step is complete, but the FSI iterations stopped at fsi_max_it with error " +
                    std::to_string(c->fsi_err_capped);
    return fail(rc, m.c_str());
  }
  return op_result(rc, "advance failed");
}

int ib_set_frame(IbCtx* h, const double* uvw) {
  CTX_OR_FAIL(h);
  if (!uvw) return fail(IB_ERR_ARG, "bad argument");
  if (c->end_pending) return fail(IB_ERR_STATE, "a step is in progress");
  for (int i = 0; i < 3; ++i)
    if (!std::isfinite(uvw[i])) return fail(IB_ERR_ARG, "frame velocity not finite");
  ib::FrameLevels fl;
  for (int k = 0; k < c->L; ++k) {
    fl.q0x[k] = c->q0x[k];
    fl.q0y[k] = c->q0y[k];
  }
  const auto& p = c->p;
  if (!c->frame_lines && cudaMalloc(&c->frame_lines, 8 * (size_t)c->L * (c->g.n + c->g.m)) != cudaSuccess) {
    c->frame_lines = nullptr;
    cudaGetLastError();
    return fail(IB_ERR_NOMEM, "device allocation failed");
  }
  const int rc = ib::launch_frame_flux(c->g, fl, c->L, c->delta, p.offsetx, p.offsety, uvw[0], uvw[1], uvw[2],
                                       p.motion[3], p.motion[4], c->frame_lines, c->st);
  if (rc != IB_OK) return op_result(rc, "frame fluxes failed");
  for (int i = 0; i < 3; ++i) c->p.motion[i] = uvw[i];   // what the restart file records
  return IB_OK;
}

static int field_ptr(Ctx* c, int field, int level, double** p, size_t* n) {
  if (level < 0 || level >= c->L) return IB_ERR_ARG;
  switch (field) {
    case IB_FIELD_OMEGA: *p = c->omega[level]; *n = c->g.ns; break;
    case IB_FIELD_S: *p = c->s[level]; *n = c->g.ns; break;
    case IB_FIELD_QX: *p = c->qx[level]; *n = c->g.nu; break;
    case IB_FIELD_QY: *p = c->qy[level]; *n = c->g.nv; break;
    case IB_FIELD_RHS_OLD: *p = c->rhs_old[level]; *n = c->g.ns; break;
    case IB_FIELD_Q0X: *p = c->q0x[level]; *n = c->g.nu; break;
    case IB_FIELD_Q0Y: *p = c->q0y[level]; *n = c->g.nv; break;
    default: return IB_ERR_ARG;
  }
  return IB_OK;
}

int ib_get_field(IbCtx* h, int field, int level, double* out) {
  CTX_OR_FAIL(h);
  double* p; size_t n;
  if (!out || field_ptr(c, field, level, &p, &n)) return fail(IB_ERR_ARG, "bad field or level");
  if (cudaMemcpyAsync(out, p, 8 * n, cudaMemcpyDefault, c->st) != cudaSuccess ||
      cudaStreamSynchronize(c->st) != cudaSuccess)
    return fail(IB_ERR_CUDA, "copy failed");
  return IB_OK;
}

int ib_set_field(IbCtx* h, int field, int level, const double* in) {
  CTX_OR_FAIL(h);
  double* p; size_t n;
  if (!in || field_ptr(c, field, level, &p, &n)) return fail(IB_ERR_ARG, "bad field or level");
  if (cudaMemcpyAsync(p, in, 8 * n, cudaMemcpyDefault, c->st) != cudaSuccess ||
      cudaStreamSynchronize(c->st) != cudaSuccess)
    return fail(IB_ERR_CUDA, "copy failed");
  return IB_OK;
}

static double* vec_ptr(Ctx* c, int which) {
  switch (which) {
    case IB_VEC_F: return c->f;
    case IB_VEC_F_RDST: return c->f_rdst;
    case IB_VEC_XB: return c->xb;
    case IB_VEC_YB: return c->yb;
    case IB_VEC_UB: return c->ub;
    default: return nullptr;
  }
}

int ib_get_vector(IbCtx* h, int which, double* out) {
  CTX_OR_FAIL(h);
  double* p = vec_ptr(c, which);
  if (!p || !out) return fail(IB_ERR_ARG, "bad vector");
  if (c->nf == 0) return IB_OK;
  if (cudaMemcpyAsync(out, p, 8 * (size_t)c->nf, cudaMemcpyDefault, c->st) != cudaSuccess ||
      cudaStreamSynchronize(c->st) != cudaSuccess)
    return fail(IB_ERR_CUDA, "copy failed");
  return IB_OK;
}

int ib_set_vector(IbCtx* h, int which, const double* in) {
  CTX_OR_FAIL(h);
  double* p = vec_ptr(c, which);
  if (!p || !in) return fail(IB_ERR_ARG, "bad vector");
  if (c->nf == 0) return IB_OK;
  if (cudaMemcpyAsync(p, in, 8 * (size_t)c->nf, cudaMemcpyDefault, c->st) != cudaSuccess)
    return fail(IB_ERR_CUDA, "copy failed");
  int rc = IB_OK;
  if (which == IB_VEC_XB || which == IB_VEC_YB) rc = ib::op_reg_prep(c);
  if (which == IB_VEC_UB && !c->ub_on) {
    // from now on every Schur right-hand side carries -delta u_B: the captured phases that
    // form it are captured again
    c->ub_on = true;
    ib::drop_phase(&c->graph_fsi_rhs);
    ib::drop_phase(&c->graph_fsi_loop);
    ib::drop_phase(&c->graph_step);
  }
  if (rc == IB_OK) rc = ib::check_err(c);
  return op_result(rc, "set_vector failed");
}

int ib_get_forces(IbCtx* h, double* cx, double* cy) {
  CTX_OR_FAIL_KEEP(h);
  if (!cx || !cy) return fail(IB_ERR_ARG, "null output");
  c->want_out = true;   // later steps queue their outputs' copies
  if (c->nbody == 0) return IB_OK;
  if (c->out_fresh) {
    std::memcpy(cx, c->h_out, 8 * (size_t)c->nbody);
    std::memcpy(cy, c->h_out + c->nbody, 8 * (size_t)c->nbody);
    return IB_OK;
  }
  int rc = ib::launch_force_coeffs(c->nf, c->nbody, c->comp, c->bid, c->f, c->p.dt, c->delta, c->forces, c->st);
  if (rc) return op_result(rc, "force coefficients failed");
  if (cudaMemcpyAsync(cx, c->forces, 8 * (size_t)c->nbody, cudaMemcpyDefault, c->st) != cudaSuccess ||
      cudaMemcpyAsync(cy, c->forces + c->nbody, 8 * (size_t)c->nbody, cudaMemcpyDefault, c->st) != cudaSuccess ||
      cudaStreamSynchronize(c->st) != cudaSuccess)
    return fail(IB_ERR_CUDA, "copy failed");
  return IB_OK;
}

int ib_get_body_state(IbCtx* h, double* theta, double* thetad, double* thetadd) {
  CTX_OR_FAIL_KEEP(h);
  c->want_out = true;
  if (c->nt == 0) return IB_OK;
  if (c->out_fresh && !thetad && !thetadd) {
    if (theta) std::memcpy(theta, c->h_out + 2 * c->nbody, 8 * (size_t)c->nt);
    return IB_OK;
  }
  size_t n = 8 * (size_t)c->nt;
  if ((theta && cudaMemcpyAsync(theta, c->ts.theta, n, cudaMemcpyDefault, c->st) != cudaSuccess) ||
      (thetad && cudaMemcpyAsync(thetad, c->ts.thetad, n, cudaMemcpyDefault, c->st) != cudaSuccess) ||
      (thetadd && cudaMemcpyAsync(thetadd, c->ts.thetadd, n, cudaMemcpyDefault, c->st) != cudaSuccess) ||
      cudaStreamSynchronize(c->st) != cudaSuccess)
    return fail(IB_ERR_CUDA, "copy failed");
  return IB_OK;
}

int ib_write_variables(IbCtx* h, const char* path) {
  CTX_OR_FAIL(h);
  if (!path) return fail(IB_ERR_ARG, "null path");
  std::string msg;
  int rc = ib::op_write_variables(c, path, &msg);
  return rc == IB_OK ? IB_OK : fail(rc, ("write_variables: " + msg).c_str());
}

int ib_subdomain_setup(IbCtx* h, int full_rectangular, double sdxi, double sdxe, double sdyi, double sdye,
                       double delta_sd) {
  CTX_OR_FAIL(h);
  std::string msg;
  int rc = ib::sd_setup(c, full_rectangular, sdxi, sdxe, sdyi, sdye, delta_sd, &msg);
  return rc == IB_OK ? IB_OK : fail(rc, ("subdomain_setup: " + msg).c_str());
}

int ib_subdomain_precompute(IbCtx* h) {
  CTX_OR_FAIL(h);
  if (!c->sd.on) return fail(IB_ERR_STATE, "subdomain_precompute: no sub-domain set up");
  return op_result(ib::sd_precompute(c), "subdomain_precompute failed");
}

int ib_write_subdomain_matrix(IbCtx* h, const char* path) {
  CTX_OR_FAIL(h);
  if (!path) return fail(IB_ERR_ARG, "null path");
  std::string msg;
  int rc = ib::sd_write(c, path, &msg);
  return rc == IB_OK ? IB_OK : fail(rc, ("write_subdomain_matrix: " + msg).c_str());
}

int ib_read_subdomain_matrix(IbCtx* h, const char* path) {
  CTX_OR_FAIL(h);
  if (!path) return fail(IB_ERR_ARG, "null path");
  std::string msg;
  int rc = ib::sd_read(c, path, &msg);
  return rc == IB_OK ? IB_OK : fail(rc, ("read_subdomain_matrix: " + msg).c_str());
}

int ib_subdomain_operator(IbCtx* h, double* lumat) {
  CTX_OR_FAIL(h);
  if (!lumat) return fail(IB_ERR_ARG, "bad argument");
  if (!c->sd.on) return fail(IB_ERR_STATE, "subdomain_operator: no sub-domain set up");
  int rc = c->sd.ready ? IB_OK : ib::sd_precompute(c);
  if (rc == IB_OK) rc = ib::sd_assemble(c, true);
  if (rc == IB_OK) c->inf.active = true;
  const size_t nf = (size_t)c->nf;
  std::vector<double> St(nf * nf);
  if (rc == IB_OK && (cudaMemcpyAsync(St.data(), c->inf.St, 8 * nf * nf, cudaMemcpyDeviceToHost, c->st) != cudaSuccess ||
                      cudaStreamSynchronize(c->st) != cudaSuccess))
    rc = IB_ERR_CUDA;
  if (rc == IB_OK) rc = ib::check_err(c);
  if (rc != IB_OK) return op_result(rc, "subdomain_operator failed");
  for (size_t k = 0; k < nf; ++k)
    for (size_t l = 0; l < nf; ++l) lumat[k * nf + l] = St[l * nf + k];
  return IB_OK;
}

int ib_get_subdomain_stats(IbCtx* h, long long* counts, double* precompute_ms) {
  CTX_OR_FAIL(h);
  if (!counts || !precompute_ms) return fail(IB_ERR_ARG, "bad argument");
  counts[0] = c->sd.nf_sd;
  counts[1] = c->sd.candidates;
  counts[2] = c->sd.kept;
  counts[3] = c->sd.columns;
  *precompute_ms = c->sd.precompute_ms;
  return IB_OK;
}

int ib_adjoint_forward(IbCtx* h, int nsteps, int K, const double* frames, double* forces) {
  CTX_OR_FAIL(h);
  if (!frames || !forces) return fail(IB_ERR_ARG, "bad argument");
  std::string msg;
  int rc = ib::op_adjoint_forward(c, nsteps, K, frames, forces, &msg);
  if (rc != IB_OK && msg.empty()) return op_result(rc, "adjoint_forward failed");
  return rc == IB_OK ? IB_OK : fail(rc, ("adjoint_forward: " + msg).c_str());
}

int ib_adjoint_backward(IbCtx* h, const double* dforces, double* dframes) {
  CTX_OR_FAIL(h);
  if (!dforces || !dframes) return fail(IB_ERR_ARG, "bad argument");
  std::string msg;
  int rc = ib::op_adjoint_backward(c, dforces, dframes, &msg);
  if (rc != IB_OK && msg.empty()) return op_result(rc, "adjoint_backward failed");
  return rc == IB_OK ? IB_OK : fail(rc, ("adjoint_backward: " + msg).c_str());
}

int ib_read_variables(IbCtx* h, const char* path, int itime) {
  CTX_OR_FAIL(h);
  if (!path) return fail(IB_ERR_ARG, "null path");
  std::string msg;
  int rc = ib::op_read_variables(c, path, itime, &msg);
  return rc == IB_OK ? IB_OK : fail(rc, ("read_variables: " + msg).c_str());
}

// ---- batches of independent simulations
struct IbBatch {
  std::vector<IbCtx*> sims;
  std::vector<int> rc;
};

int ib_batch_create(const IbParams* params, const IbBody* bodies, const int* nbody, int nsim, IbBatch** out) {
  if (!params || !nbody || !out || nsim < 1) return fail(IB_ERR_ARG, "null argument or empty batch");
  IbBatch* b = new IbBatch();
  int off = 0;
  for (int i = 0; i < nsim; ++i) {
    if (nbody[i] < 0 || (nbody[i] > 0 && !bodies)) {
      ib_batch_destroy(b);
      return fail(IB_ERR_ARG, "bad body count");
    }
    std::string msg;
    Ctx* c = nullptr;
    int rc = ib::ctx_create(&params[i], nbody[i] ? bodies + off : nullptr, nbody[i], &c, &msg);
    if (rc != IB_OK) {
      ib_batch_destroy(b);
      return fail(rc, ("batch simulation " + std::to_string(i) + ": " + msg).c_str());
    }
    b->sims.push_back(new IbCtx{c, true});
    off += nbody[i];
  }
  b->rc.assign(nsim, IB_OK);
  *out = b;
  return IB_OK;
}

int ib_batch_destroy(IbBatch* b) {
  if (!b) return IB_OK;
  for (IbCtx* h : b->sims) {
    ib::ctx_destroy(h->c);
    delete h;
  }
  delete b;
  return IB_OK;
}

int ib_batch_size(IbBatch* b, int* nsim) {
  if (!b || !nsim) return fail(IB_ERR_ARG, "null argument");
  *nsim = (int)b->sims.size();
  return IB_OK;
}

int ib_batch_context(IbBatch* b, int i, IbCtx** ctx) {
  if (!b || !ctx || i < 0 || i >= (int)b->sims.size()) return fail(IB_ERR_ARG, "bad batch index");
  *ctx = b->sims[i];
  return IB_OK;
}

int ib_batch_advance(IbBatch* b, int* status) {
  if (!b) return fail(IB_ERR_ARG, "null batch");
  const int n = (int)b->sims.size();
  // every simulation's predictor, vort2flux and device FSI loop go on the GPU first, then each
  // simulation's counters are read and its correction launched, then each step is finished:
  // the host waits on a simulation only after the other simulations' work is queued
  for (int i = 0; i < n; ++i) b->rc[i] = ib::op_advance_begin(b->sims[i]->c);
  for (int i = 0; i < n; ++i)
    if (b->rc[i] == IB_OK) b->rc[i] = ib::op_advance_end(b->sims[i]->c);
  for (int i = 0; i < n; ++i) {
    ib::Ctx* c = b->sims[i]->c;
    c->out_fresh = false;
    if (b->rc[i] == IB_OK) {
      b->rc[i] = ib::op_advance_finish(c);
      c->out_fresh = c->out_queued && (b->rc[i] == IB_OK || b->rc[i] == IB_ERR_GMRES || b->rc[i] == IB_ERR_FSI);
    }
  }
  int first = IB_OK, where = -1;
  for (int i = 0; i < n; ++i) {
    if (status) status[i] = b->rc[i];
    if (b->rc[i] != IB_OK && first == IB_OK) { first = b->rc[i]; where = i; }
  }
  if (first != IB_OK) {
    cudaGetLastError();
    return fail(first, ("batch advance: simulation " + std::to_string(where) + " returned " +
                        std::to_string(first) + " (per-simulation codes in status)").c_str());
  }
  return IB_OK;
}

int ib_calculate_pressure(IbCtx* h, double* p) {
  CTX_OR_FAIL(h);
  if (!p) return fail(IB_ERR_ARG, "null output");
  int rc = ib::op_pressure(c);
  if (rc != IB_OK) return op_result(rc, "calculate_pressure failed");
  const size_t cells = (size_t)c->g.m * c->g.n;
  for (int k = 0; k < c->L; ++k)
    if (cudaMemcpyAsync(p + (size_t)k * cells, c->pres.p[k], 8 * cells, cudaMemcpyDefault, c->st) != cudaSuccess)
      return fail(IB_ERR_CUDA, "copy failed");
  if (cudaStreamSynchronize(c->st) != cudaSuccess) return fail(IB_ERR_CUDA, "copy failed");
  return IB_OK;
}

int ib_write_pressure(IbCtx* h, const char* path) {
  CTX_OR_FAIL(h);
  if (!path) return fail(IB_ERR_ARG, "null path");
  std::string msg;
  int rc = ib::op_write_pressure(c, path, &msg);
  return rc == IB_OK ? IB_OK : fail(rc, ("write_pressure: " + msg).c_str());
}

int ib_get_beam_state(IbCtx* h, double* q, double* qd, double* qdd) {
  CTX_OR_FAIL(h);
  size_t at = 0;
  for (const ib::BeamDev& b : c->beams_h) {
    const size_t n = 8 * (size_t)b.ndof;
    if ((q && cudaMemcpyAsync(q + at, b.q, n, cudaMemcpyDefault, c->st) != cudaSuccess) ||
        (qd && cudaMemcpyAsync(qd + at, b.qd, n, cudaMemcpyDefault, c->st) != cudaSuccess) ||
        (qdd && cudaMemcpyAsync(qdd + at, b.qdd, n, cudaMemcpyDefault, c->st) != cudaSuccess))
      return fail(IB_ERR_CUDA, "copy failed");
    at += b.ndof;
  }
  if (cudaStreamSynchronize(c->st) != cudaSuccess) return fail(IB_ERR_CUDA, "copy failed");
  return IB_OK;
}

int ib_get_counters(IbCtx* h, int* ksp_iter, int* fsi_iter) {
  CTX_OR_FAIL_KEEP(h);
  if (ksp_iter) *ksp_iter = c->ksp_iter;
  if (fsi_iter) *fsi_iter = c->fsi_iter;
  return IB_OK;
}

int ib_get_dims(IbCtx* h, int* nf, int* nbc, int* ns, int* nu, int* nv) {
  CTX_OR_FAIL(h);
  if (nf) *nf = c->nf;
  if (nbc) *nbc = c->g.nbc;
  if (ns) *ns = c->g.ns;
  if (nu) *nu = c->g.nu;
  if (nv) *nv = c->g.nv;
  return IB_OK;
}

// ------------------------------------------------------------ operators
int ib_nonlinear(IbCtx* h, const double* omega, const double* qx, const double* qy, const double* bc, double* nlx,
                 double* nly) {
  CTX_OR_FAIL(h);
  Staging S(c);
  const double* o = S.in(omega, c->g.ns);
  const double* x = S.in(qx, c->g.nu);
  const double* y = S.in(qy, c->g.nv);
  const double* r = S.in(bc, c->g.nbc);
  double* a = S.out(nlx, c->g.nu, false);
  double* b = S.out(nly, c->g.nv, false);
  STAGE_CHECK(S);
  int rc = ib::launch_nonlinear(c->g, o, r, x, nullptr, y, nullptr, a, b, c->st);
  return op_result(S.finish(rc), "nonlinear failed");
}

int ib_rot(IbCtx* h, const double* hx, const double* hy, double* vort) {
  CTX_OR_FAIL(h);
  Staging S(c);
  const double* x = S.in(hx, c->g.nu);
  const double* y = S.in(hy, c->g.nv);
  double* v = S.out(vort, c->g.ns, false);
  STAGE_CHECK(S);
  return op_result(S.finish(ib::launch_rot(c->g, x, y, v, c->st)), "rot failed");
}

int ib_curl(IbCtx* h, const double* s, const double* sbc, double* qx, double* qy) {
  CTX_OR_FAIL(h);
  Staging S(c);
  const double* sv = S.in(s, c->g.ns);
  const double* r = S.in(sbc, c->g.nbc);
  double* a = S.out(qx, c->g.nu, false);
  double* b = S.out(qy, c->g.nv, false);
  STAGE_CHECK(S);
  return op_result(S.finish(ib::launch_curl(c->g, sv, r, a, b, c->st)), "curl failed");
}

int ib_coarsify(IbCtx* h, const double* fine, double* coarse) {
  CTX_OR_FAIL(h);
  Staging S(c);
  const double* f = S.in(fine, c->g.ns);
  double* o = S.out(coarse, c->g.ns, true);
  STAGE_CHECK(S);
  return op_result(S.finish(ib::launch_coarsify(c->g, f, o, c->st)), "coarsify failed");
}

int ib_get_bc(IbCtx* h, const double* s, double fac, double* ring) {
  CTX_OR_FAIL(h);
  Staging S(c);
  const double* sv = S.in(s, c->g.ns);
  double* r = S.out(ring, c->g.nbc, false);
  STAGE_CHECK(S);
  return op_result(S.finish(ib::launch_get_bc(c->g, sv, fac, r, c->st)), "get_bc failed");
}

int ib_apply_bc(IbCtx* h, double* vort, const double* ring, double fac) {
  CTX_OR_FAIL(h);
  Staging S(c);
  const double* r = S.in(ring, c->g.nbc);
  double* v = S.out(vort, c->g.ns, true);
  STAGE_CHECK(S);
  return op_result(S.finish(ib::launch_apply_bc(c->g, v, r, fac, c->st)), "apply_bc failed");
}

int ib_dst(IbCtx* h, const double* in, double* out) {
  CTX_OR_FAIL(h);
  Staging S(c);
  const double* i = S.in(in, c->g.ns);
  double* o = S.out(out, c->g.ns, false);
  STAGE_CHECK(S);
  return op_result(S.finish(ib::op_dst(c, i, o)), "dst failed");
}

int ib_ctci(IbCtx* h, const double* vort, double* s) {
  CTX_OR_FAIL(h);
  Staging S(c);
  const double* i = S.in(vort, c->g.ns);
  double* o = S.out(s, c->g.ns, false);
  STAGE_CHECK(S);
  return op_result(S.finish(ib::op_ctci(c, i, o, nullptr)), "ctci failed");
}

int ib_ainv(IbCtx* h, double* vort) {
  CTX_OR_FAIL(h);
  Staging S(c);
  double* v = S.out(vort, c->g.ns, true);
  STAGE_CHECK(S);
  return op_result(S.finish(ib::op_ainv(c, v, v)), "ainv failed");
}

int ib_fluid_predictor(IbCtx* h, int level, double* omega, const double* rhs, const double* rhs_old,
                       const double* rhsbc) {
  CTX_OR_FAIL(h);
  if (level < 0 || level >= c->L) return fail(IB_ERR_ARG, "bad level");
  Staging S(c);
  const double* a = S.in(rhs, c->g.ns);
  const double* b = S.in(rhs_old, c->g.ns);
  const double* r = S.in(rhsbc, c->g.ns);
  double* o = S.out(omega, c->g.ns, true);
  STAGE_CHECK(S);
  return op_result(S.finish(ib::op_predictor(c, level, o, a, b, r)), "fluid_predictor failed");
}

int ib_vort2flux(IbCtx* h, double* omega, double* s, double* qx, double* qy) {
  CTX_OR_FAIL(h);
  const int L = c->L;
  Staging S(c);
  double* w = S.out(omega, (size_t)L * c->g.ns, true);
  double* sv = S.out(s, (size_t)L * c->g.ns, false);
  double* a = S.out(qx, (size_t)L * c->g.nu, false);
  double* b = S.out(qy, (size_t)L * c->g.nv, false);
  STAGE_CHECK(S);
  std::vector<double*> W(L), SS(L), QX(L), QY(L);
  for (int k = 0; k < L; ++k) {
    W[k] = w + (size_t)k * c->g.ns; SS[k] = sv + (size_t)k * c->g.ns;
    QX[k] = a + (size_t)k * c->g.nu; QY[k] = b + (size_t)k * c->g.nv;
  }
  return op_result(S.finish(ib::op_vort2flux(c, W.data(), SS.data(), QX.data(), QY.data(), true)),
                   "vort2flux failed");
}

int ib_reg_prep(IbCtx* h, const double* xb, const double* yb) {
  CTX_OR_FAIL(h);
  if (c->nf == 0) return IB_OK;
  if (cudaMemcpyAsync(c->xb, xb, 8 * (size_t)c->nf, cudaMemcpyDefault, c->st) != cudaSuccess ||
      cudaMemcpyAsync(c->yb, yb, 8 * (size_t)c->nf, cudaMemcpyDefault, c->st) != cudaSuccess)
    return fail(IB_ERR_CUDA, "copy failed");
  int rc = ib::op_reg_prep(c);
  if (rc == IB_OK) rc = ib::check_err(c);
  return op_result(rc, "reg_prep failed (stencil outside the grid?)");
}

int ib_reg(IbCtx* h, const double* h0, double* hx, double* hy) {
  CTX_OR_FAIL(h);
  Staging S(c);
  const double* f = S.in(h0, c->nf);
  double* a = S.out(hx, c->g.nu, false);
  double* b = S.out(hy, c->g.nv, false);
  STAGE_CHECK(S);
  return op_result(S.finish(ib::launch_reg(c->g, c->nf, f, c->reg, a, b, c->st)), "reg failed");
}

int ib_regT(IbCtx* h, const double* hx, const double* hy, double* h0) {
  CTX_OR_FAIL(h);
  Staging S(c);
  const double* a = S.in(hx, c->g.nu);
  const double* b = S.in(hy, c->g.nv);
  double* o = S.out(h0, c->nf, true);
  STAGE_CHECK(S);
  return op_result(S.finish(ib::launch_regT(c->g, c->nf, a, nullptr, b, nullptr, c->reg, o, o, c->st)),
                   "regT failed");
}

int ib_redistribute(IbCtx* h, const double* f, double* frdst) {
  CTX_OR_FAIL(h);
  Staging S(c);
  const double* a = S.in(f, c->nf);
  double* o = S.out(frdst, c->nf, false);
  STAGE_CHECK(S);
  return op_result(S.finish(ib::op_redistribute(c, a, o)), "redistribute failed");
}

int ib_schur_apply(IbCtx* h, const double* x, double* y) {
  CTX_OR_FAIL(h);
  Staging S(c);
  const double* a = S.in(x, c->nf);
  double* o = S.out(y, c->nf, false);
  STAGE_CHECK(S);
  return op_result(S.finish(ib::op_schur(c, a, o, true)), "schur_apply failed");
}

int ib_schur_apply_fluid(IbCtx* h, const double* x, double* y) {
  CTX_OR_FAIL(h);
  Staging S(c);
  const double* a = S.in(x, c->nf);
  double* o = S.out(y, c->nf, false);
  STAGE_CHECK(S);
  return op_result(S.finish(ib::op_schur(c, a, o, false)), "schur_apply_fluid failed");
}

int ib_struct_btimes(IbCtx* h, const double* x, double* y) {
  CTX_OR_FAIL(h);
  Staging S(c);
  const double* a = S.in(x, c->nf);
  double* o = S.out(y, c->nf, false);
  STAGE_CHECK(S);
  int rc = cudaMemsetAsync(o, 0, 8 * (size_t)c->nf, c->st) == cudaSuccess ? IB_OK : IB_ERR_CUDA;
  if (rc == IB_OK) rc = ib::launch_tors_btimes(c->nt, c->tb, c->ts, c->p.dt, c->delta, a, o, c->st);
  if (rc == IB_OK) rc = ib::launch_beam_btimes(c, a, o, c->st);
  return op_result(S.finish(rc), "struct_btimes failed");
}

int ib_struct_rhs(IbCtx* h, double* y) {
  CTX_OR_FAIL(h);
  Staging S(c);
  double* o = S.out(y, c->nf, false);
  STAGE_CHECK(S);
  int rc = cudaMemsetAsync(o, 0, 8 * (size_t)c->nf, c->st) == cudaSuccess ? IB_OK : IB_ERR_CUDA;
  if (rc == IB_OK) rc = ib::launch_tors_rhs(c->nt, c->tb, c->ts, c->p.dt, c->delta, o, c->st);
  if (rc == IB_OK) rc = ib::launch_beam_rhs(c, o, c->st);
  return op_result(S.finish(rc), "struct_rhs failed");
}

int ib_struct_dx(IbCtx* h, const double* f, double* err) {
  CTX_OR_FAIL(h);
  Staging S(c);
  const double* a = S.in(f, c->nf);
  STAGE_CHECK(S);
  int rc = ib::launch_tors_dx(c->nt, c->tb, c->ts, c->p.dt, c->delta, a, c->xb, c->yb, c->err_fsi, c->st);
  if (rc == IB_OK) rc = ib::launch_beam_dx(c, a, c->st);
  if (rc == IB_OK && (c->nt > 0 || c->nbeam > 0)) rc = ib::op_reg_prep(c);
  rc = S.finish(rc);
  if (rc == IB_OK && err) {
    if (cudaMemcpy(err, c->err_fsi, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) rc = IB_ERR_CUDA;
  }
  if (rc == IB_OK) rc = ib::check_err(c);
  return op_result(rc, "struct_dx failed");
}

int ib_schur_solve(IbCtx* h, const double* rhs, double* f, int* iterations) {
  CTX_OR_FAIL(h);
  Staging S(c);
  const double* b = S.in(rhs, c->nf);
  double* x = S.out(f, c->nf, true);
  STAGE_CHECK(S);
  int its = 0, reason = 0;
  int rc = ib::op_gmres(c, b, x, &its, &reason);
  if (iterations) *iterations = its;
  return op_result(S.finish(rc), "schur_solve failed");
}

int ib_get_stream(IbCtx* h, void** stream) {
  CTX_OR_FAIL(h);
  if (!stream) return fail(IB_ERR_ARG, "null output");
  *stream = (void*)c->st;
  return IB_OK;
}

int ib_get_work(IbCtx* h, long long* matvecs, long long* passes4) {
  CTX_OR_FAIL(h);
  if (matvecs) *matvecs = c->n_matvec;
  if (passes4)
    for (int i = 0; i < 4; ++i) passes4[i] = c->n_pass[i];
  return IB_OK;
}

long long ib_launch_count(void) { return ib::launch_count(); }

int ib_measure_fp64_peak(double* tflops) {
  if (!tflops) return fail(IB_ERR_ARG, "null output");
  int rc = ib::probe_fp64(tflops);
  return op_result(rc, "fp64 probe failed");
}

int ib_time_pass(IbCtx* h, int kind, int reps, double* avg_ms) {
  CTX_OR_FAIL(h);
  if (!avg_ms || reps <= 0 || kind < 0 || kind > 5) return fail(IB_ERR_ARG, "bad argument");
  if (kind == 2 || kind == 3)
    return op_result(ib::op_time_pressure_transform(c, kind == 2, reps, avg_ms), "time_pass failed");
  return op_result(ib::op_time_pass(c, kind, reps, avg_ms), "time_pass failed");
}

int ib_profile_schur(IbCtx* h, int reps, double* stage_ms) {
  CTX_OR_FAIL(h);
  if (!stage_ms || reps <= 0) return fail(IB_ERR_ARG, "bad argument");
  return op_result(ib::op_profile_schur(c, reps, stage_ms), "profile_schur failed");
}

int ib_step_profile(IbCtx* h, int mode, double* phase_ms, long long* nsteps) {
  CTX_OR_FAIL(h);
  if (mode < 0 || mode > 3) return fail(IB_ERR_ARG, "bad mode");
  return op_result(ib::op_step_profile(c, mode, phase_ms, nsteps), "step_profile failed");
}

int ib_get_launch_shapes(IbCtx* h, int* shapes) {
  CTX_OR_FAIL(h);
  if (!shapes) return fail(IB_ERR_ARG, "bad argument");
  int i = 0;
  for (const ib::DstLaunch* L : {&c->lx, &c->lx_small, &c->lx_batch, &c->ly_none}) {
    shapes[i++] = L->B;
    shapes[i++] = L->NT;
    shapes[i++] = L->narrow_scan;
  }
  shapes[i] = c->tl.Mb;
  return IB_OK;
}

int ib_schur_matrix(IbCtx* h, double* S, int* status) {
  CTX_OR_FAIL(h);
  if (!S || !status) return fail(IB_ERR_ARG, "bad argument");
  if (c->nf == 0) return fail(IB_ERR_STATE, "no body unknowns");
  if (c->p.schur_mode == 1) return fail(IB_ERR_STATE, "influence matrix disabled (schur_mode 1)");
  int rc = ib::inf_prepare(c);
  if (rc != IB_OK) return op_result(rc, "influence matrix failed");
  *status = c->inf.active ? 0 : (c->inf.flag_h ? c->inf.flag_h : 4);
  if (c->inf.active &&
      cudaMemcpyAsync(S, c->inf.S, sizeof(double) * (size_t)c->nf * c->nf, cudaMemcpyDefault, c->st) != cudaSuccess)
    return fail(IB_ERR_CUDA, "copy failed");
  if (cudaStreamSynchronize(c->st) != cudaSuccess) return fail(IB_ERR_CUDA, "sync failed");
  return IB_OK;
}

int ib_get_influence_stats(IbCtx* h, long long* counts, double* build_ms) {
  CTX_OR_FAIL(h);
  if (!counts || !build_ms) return fail(IB_ERR_ARG, "bad argument");
  const ib::Influence& I = c->inf;
  counts[0] = I.builds;
  counts[1] = I.columns;
  counts[2] = I.assemblies;
  counts[3] = I.fallbacks;
  counts[4] = I.nR;
  *build_ms = I.build_ms;
  return IB_OK;
}

int ib_get_coarse_stats(IbCtx* h, long long* counts, double* ms) {
  CTX_OR_FAIL(h);
  if (!counts || !ms) return fail(IB_ERR_ARG, "bad argument");
  const ib::CoarseResp& cr = c->inf.cr;
  long long held = 0;
  for (int k = 1; k < c->L; ++k) held += cr.n[k];
  counts[0] = cr.solves;
  counts[1] = held;
  counts[2] = (long long)cr.bytes;
  counts[3] = cr.enabled ? 1 : 0;
  *ms = cr.ms;
  return IB_OK;
}

int ib_get_ring_maps(IbCtx* h, long long* counts, double* ms) {
  CTX_OR_FAIL(h);
  if (!counts || !ms) return fail(IB_ERR_ARG, "bad argument");
  counts[0] = c->rmap.on ? 1 : 0;
  counts[1] = (long long)c->rmap.bytes;
  *ms = c->rmap.ms;
  return IB_OK;
}

int ib_get_step_graph_stats(IbCtx* h, long long* counts) {
  CTX_OR_FAIL(h);
  if (!counts) return fail(IB_ERR_ARG, "bad argument");
  counts[0] = c->n_step_graph;
  counts[1] = c->n_step_gate_closed;
  counts[2] = c->n_step_phased;
  return IB_OK;
}

int ib_profile(IbCtx* h, int enable) {
  CTX_OR_FAIL(h);
  if (cudaStreamSynchronize(c->st) != cudaSuccess) return fail(IB_ERR_CUDA, "sync failed");
  if (enable) c->prof_n = 0;
  c->prof_on = enable != 0;
  return IB_OK;
}

int ib_profile_read(IbCtx* h, int kind, int* count, double* total_ms, double* bytes) {
  CTX_OR_FAIL(h);
  if (cudaStreamSynchronize(c->st) != cudaSuccess) return fail(IB_ERR_CUDA, "sync failed");
  int n = 0;
  double t = 0.0, b = 0.0;
  for (int i = 0; i < c->prof_n; ++i) {
    if (c->prof_kind[i] != kind) continue;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->prof_ev[2 * i], c->prof_ev[2 * i + 1]) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    ++n;
    t += ms;
    b += c->prof_bytes[i];
  }
  if (count) *count = n;
  if (total_ms) *total_ms = t;
  if (bytes) *bytes = b;
  return IB_OK;
}

}  // extern "C"
