// The reference's restart file, output/dataRR_IIIIIII.var (write_variables and read_variables,
// variables.F90:709-913), written from and read into a context.
//
// The file is a Fortran unformatted sequential stream: every WRITE statement is one record,
// framed by its byte length as a 4-byte integer before and after the data.  Integers are
// 4 bytes (PetscInt without 64-bit indices), reals 8.  The reference's own reader,
// output/getdata.m, reads it with exactly this layout.  Records, for one rank:
//    m, n, mgridlev, nb
//    Re, dt, len, offsetx, offsety
//    xsi, xse, xsm, ysi, yse, ysm          vertex index range   (2, m, m-1, 2, n, n-1)
//    xui, xue, xum, yui, yue, yum          u-face index range   (1, m+1, m+1, 1, n, n)
//    xvi, xve, xvm, yvi, yve, yvm          v-face index range   (1, m, m, 1, n+1, n+1)
//    per level: omega, s, qx, q0px, q0rx, qy, q0py, q0ry       (eight records)
//    rhs_old of every level                                    (one record, level slowest)
//    rot_angle, rox, roy
//    xfm, xfi, xfe                          force vector range  (nf, 1, nf)
//    f;  xb;  yb
//    mt_body                                torsional bodies
//    theta(mt_body), thetad(mt_body), thetadd(mt_body)        (one record, only if mt_body > 0)
//    f_rdst
// The frame flux q0 is kept as one field here; the file's potential part q0p is the uniform
// -delta 2^(k-1) (u, v) of the frame velocity, and its rotational part q0r = q0 - q0p (zero
// unless the frame rotates).  Reading sums them back (q0 = q0p + q0r, variables.F90:908-911),
// which returns q0 exactly when the frame does not rotate and to the last bit otherwise.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "ctx.cuh"

namespace ib {

namespace {

struct RecordWriter {
  FILE* f = nullptr;
  bool ok = true;
  void rec(const void* data, size_t bytes) {
    if (!ok) return;
    if (bytes > 0x7fffffffu) { ok = false; return; }   // one 4-byte-framed record
    const int32_t n = (int32_t)bytes;
    ok = fwrite(&n, 4, 1, f) == 1 && (bytes == 0 || fwrite(data, 1, bytes, f) == bytes) && fwrite(&n, 4, 1, f) == 1;
  }
  template <typename T>
  void vals(std::initializer_list<T> v) {
    std::vector<T> a(v);
    rec(a.data(), sizeof(T) * a.size());
  }
};

struct RecordReader {
  FILE* f = nullptr;
  bool ok = true;
  std::string why;
  // reads one record, which must hold exactly `bytes` bytes
  void rec(void* data, size_t bytes, const char* what) {
    if (!ok) return;
    int32_t a = 0, b = 0;
    if (fread(&a, 4, 1, f) != 1 || (size_t)a != bytes || (bytes && fread(data, 1, bytes, f) != bytes) ||
        fread(&b, 4, 1, f) != 1 || b != a) {
      ok = false;
      why = std::string("record '") + what + "' missing or of the wrong length";
    }
  }
};

// the uniform potential part of the frame flux on level k (1-based), variables.F90:299-320
void frame_potential(const Ctx* c, int k, double* px, double* py) {
  const double fac = c->delta * std::pow(2.0, k - 1);
  *px = -fac * c->p.motion[0];
  *py = -fac * c->p.motion[1];
}

int copy_d2h(Ctx* c, std::vector<double>& h, const double* d, size_t n) {
  h.resize(n);
  if (n && cudaMemcpyAsync(h.data(), d, 8 * n, cudaMemcpyDeviceToHost, c->st) != cudaSuccess) return IB_ERR_CUDA;
  return cudaStreamSynchronize(c->st) == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}

int copy_h2d(Ctx* c, double* d, const std::vector<double>& h) {
  if (!h.empty() && cudaMemcpyAsync(d, h.data(), 8 * h.size(), cudaMemcpyHostToDevice, c->st) != cudaSuccess)
    return IB_ERR_CUDA;
  return cudaStreamSynchronize(c->st) == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}

}  // namespace

int op_write_variables(Ctx* c, const char* path, std::string* msg) {
  const GridDims& g = c->g;
  const int L = c->L, nf = c->nf;
  FILE* f = std::fopen(path, "wb");
  if (!f) { *msg = std::string("cannot open ") + path + " for writing"; return IB_ERR_ARG; }
  RecordWriter w;
  w.f = f;
  const IbParams& p = c->p;
  w.vals<int32_t>({g.m, g.n, L, c->nb});
  w.vals<double>({p.Re, p.dt, p.len, p.offsetx, p.offsety});
  w.vals<int32_t>({2, g.m, g.m - 1, 2, g.n, g.n - 1});
  w.vals<int32_t>({1, g.m + 1, g.m + 1, 1, g.n, g.n});
  w.vals<int32_t>({1, g.m, g.m, 1, g.n + 1, g.n + 1});
  std::vector<double> a, q0, part;
  int rc = IB_OK;
  auto field = [&](const double* d, size_t n) {
    if (rc == IB_OK) rc = copy_d2h(c, a, d, n);
    if (rc == IB_OK) w.rec(a.data(), 8 * n);
  };
  // q0 split into its uniform potential part and the rest
  auto split = [&](const double* d, size_t n, double pot) {
    if (rc == IB_OK) rc = copy_d2h(c, q0, d, n);
    if (rc != IB_OK) return;
    part.assign(n, pot);
    w.rec(part.data(), 8 * n);
    for (size_t i = 0; i < n; ++i) part[i] = q0[i] - pot;
    w.rec(part.data(), 8 * n);
  };
  for (int k = 0; k < L; ++k) {
    double px, py;
    frame_potential(c, k + 1, &px, &py);
    field(c->omega[k], g.ns);
    field(c->s[k], g.ns);
    field(c->qx[k], g.nu);
    split(c->q0x[k], g.nu, px);
    field(c->qy[k], g.nv);
    split(c->q0y[k], g.nv, py);
  }
  {
    std::vector<double> all((size_t)L * g.ns);
    for (int k = 0; k < L && rc == IB_OK; ++k) {
      rc = copy_d2h(c, a, c->rhs_old[k], g.ns);
      if (rc == IB_OK) std::copy(a.begin(), a.end(), all.begin() + (size_t)k * g.ns);
    }
    if (rc == IB_OK) w.rec(all.data(), 8 * all.size());
  }
  // the frame's rotation angle after itime steps at constant angular velocity, and its centre
  w.vals<double>({p.motion[2] * p.dt * c->itime, p.motion[3], p.motion[4]});
  w.vals<int32_t>({nf, 1, nf});
  field(c->f, nf);
  field(c->xb, nf);
  field(c->yb, nf);
  w.vals<int32_t>({c->nt});
  if (c->nt > 0 && rc == IB_OK) {
    std::vector<double> th;
    std::vector<double> t3;
    for (const double* d : {c->ts.theta, c->ts.thetad, c->ts.thetadd}) {
      if (rc == IB_OK) rc = copy_d2h(c, th, d, c->nt);
      t3.insert(t3.end(), th.begin(), th.end());
    }
    if (rc == IB_OK) w.rec(t3.data(), 8 * t3.size());
  }
  field(c->f_rdst, nf);
  const bool closed = std::fclose(f) == 0;
  if (rc != IB_OK) { *msg = "device copy failed"; return rc; }
  if (!w.ok || !closed) { *msg = std::string("write to ") + path + " failed"; return IB_ERR_ARG; }
  return IB_OK;
}

int op_read_variables(Ctx* c, const char* path, int itime, std::string* msg) {
  const GridDims& g = c->g;
  const int L = c->L, nf = c->nf;
  if (itime < 0) { *msg = "itime must be >= 0"; return IB_ERR_ARG; }
  FILE* f = std::fopen(path, "rb");
  if (!f) { *msg = std::string("cannot open ") + path; return IB_ERR_ARG; }
  RecordReader r;
  r.f = f;
  int32_t h4[4] = {}, h6[6] = {};
  double h5[5] = {};
  r.rec(h4, sizeof(h4), "m, n, mgridlev, nb");
  if (r.ok && (h4[0] != g.m || h4[1] != g.n || h4[2] != L || h4[3] != c->nb)) {
    std::fclose(f);
    *msg = "the file's m, n, mgridlev or nb differ from the context's";
    return IB_ERR_ARG;
  }
  r.rec(h5, sizeof(h5), "Re, dt, len, offsetx, offsety");   // dt is read into dt_old and not used
  const int32_t want[3][6] = {{2, g.m, g.m - 1, 2, g.n, g.n - 1},
                              {1, g.m + 1, g.m + 1, 1, g.n, g.n},
                              {1, g.m, g.m, 1, g.n + 1, g.n + 1}};
  for (int q = 0; q < 3; ++q) {
    r.rec(h6, sizeof(h6), "index ranges");
    for (int i = 0; i < 6 && r.ok; ++i)
      if (h6[i] != want[q][i]) { r.ok = false; r.why = "index ranges of another decomposition (one rank only)"; }
  }
  // every record is read before anything is copied to the device
  std::vector<std::vector<double>> om(L), s(L), qx(L), q0x(L), qy(L), q0y(L);
  std::vector<double> p1, p2;
  for (int k = 0; k < L && r.ok; ++k) {
    om[k].resize(g.ns); s[k].resize(g.ns); qx[k].resize(g.nu); qy[k].resize(g.nv);
    p1.resize(g.nu); p2.resize(g.nu);
    r.rec(om[k].data(), 8 * g.ns, "omega");
    r.rec(s[k].data(), 8 * g.ns, "s");
    r.rec(qx[k].data(), 8 * g.nu, "qx");
    r.rec(p1.data(), 8 * g.nu, "q0px");
    r.rec(p2.data(), 8 * g.nu, "q0rx");
    q0x[k].resize(g.nu);
    for (size_t i = 0; i < g.nu; ++i) q0x[k][i] = p1[i] + p2[i];
    r.rec(qy[k].data(), 8 * g.nv, "qy");
    p1.resize(g.nv); p2.resize(g.nv);
    r.rec(p1.data(), 8 * g.nv, "q0py");
    r.rec(p2.data(), 8 * g.nv, "q0ry");
    q0y[k].resize(g.nv);
    for (size_t i = 0; i < g.nv; ++i) q0y[k][i] = p1[i] + p2[i];
  }
  std::vector<double> rhs_old((size_t)L * g.ns);
  r.rec(rhs_old.data(), 8 * rhs_old.size(), "rhs_old");
  double rot[3];
  r.rec(rot, sizeof(rot), "rot_angle, rox, roy");
  int32_t fr[3] = {};
  r.rec(fr, sizeof(fr), "xfm, xfi, xfe");
  if (r.ok && (fr[0] != nf || fr[1] != 1 || fr[2] != nf)) { r.ok = false; r.why = "force vector range differs"; }
  std::vector<double> fv(nf), xb(nf), yb(nf);
  r.rec(fv.data(), 8 * (size_t)nf, "f");
  r.rec(xb.data(), 8 * (size_t)nf, "xb");
  r.rec(yb.data(), 8 * (size_t)nf, "yb");
  int32_t mt = 0;
  r.rec(&mt, 4, "mt_body");
  if (r.ok && mt != c->nt) { r.ok = false; r.why = "number of torsional bodies differs"; }
  std::vector<double> t3(3 * (size_t)c->nt);
  if (c->nt > 0) r.rec(t3.data(), 8 * t3.size(), "theta, thetad, thetadd");
  // f_rdst follows; the reference's reader stops before it (variables.F90:900-906)
  std::fclose(f);
  if (!r.ok) { *msg = std::string(path) + ": " + r.why; return IB_ERR_ARG; }
  int rc = IB_OK;
  for (int k = 0; k < L && rc == IB_OK; ++k) {
    rc = copy_h2d(c, c->omega[k], om[k]);
    if (rc == IB_OK) rc = copy_h2d(c, c->s[k], s[k]);
    if (rc == IB_OK) rc = copy_h2d(c, c->qx[k], qx[k]);
    if (rc == IB_OK) rc = copy_h2d(c, c->qy[k], qy[k]);
    if (rc == IB_OK) rc = copy_h2d(c, c->q0x[k], q0x[k]);
    if (rc == IB_OK) rc = copy_h2d(c, c->q0y[k], q0y[k]);
    if (rc == IB_OK)
      rc = copy_h2d(c, c->rhs_old[k], std::vector<double>(rhs_old.begin() + (size_t)k * g.ns,
                                                           rhs_old.begin() + (size_t)(k + 1) * g.ns));
  }
  if (rc == IB_OK && nf > 0) {
    rc = copy_h2d(c, c->f, fv);
    if (rc == IB_OK) rc = copy_h2d(c, c->xb, xb);
    if (rc == IB_OK) rc = copy_h2d(c, c->yb, yb);
  }
  if (rc == IB_OK && c->nt > 0) {
    const size_t nt = c->nt;
    rc = copy_h2d(c, c->ts.theta, std::vector<double>(t3.begin(), t3.begin() + nt));
    if (rc == IB_OK) rc = copy_h2d(c, c->ts.thetad, std::vector<double>(t3.begin() + nt, t3.begin() + 2 * nt));
    if (rc == IB_OK) rc = copy_h2d(c, c->ts.thetadd, std::vector<double>(t3.begin() + 2 * nt, t3.end()));
    if (rc == IB_OK) rc = launch_tors_trig(c->nt, c->tb, c->ts, c->st);   // sin, cos of the new angles
  }
  if (rc != IB_OK) { *msg = "device copy failed"; return rc; }
  // weights and stencils at the positions read (E is rebuilt from them, variables.F90:364-373)
  if (nf > 0) RC(op_reg_prep(c));
  RC(check_err(c));
  c->itime = itime;
  // the step after a restart needs every level's fields, which the file holds whole
  c->q0_partial = false;
  IB_CUDA_CHECK(cudaStreamSynchronize(c->st));
  return IB_OK;
}

// write_pressure (operators_pressure.F90:857-879): output/pressureRR_IIIIIII.var of one rank, the
// index range xpi, xpe, xpm, ypi, ype, ypm (1, m, m, 1, n, n) and then every level's m x n cells
int op_write_pressure(Ctx* c, const char* path, std::string* msg) {
  const GridDims& g = c->g;
  if (!c->pres.computed) { *msg = "no pressure computed (ib_calculate_pressure first)"; return IB_ERR_STATE; }
  FILE* f = std::fopen(path, "wb");
  if (!f) { *msg = std::string("cannot open ") + path + " for writing"; return IB_ERR_ARG; }
  RecordWriter w;
  w.f = f;
  w.vals<int32_t>({1, g.m, g.m, 1, g.n, g.n});
  std::vector<double> a;
  int rc = IB_OK;
  for (int k = 0; k < c->L && rc == IB_OK; ++k) {
    rc = copy_d2h(c, a, c->pres.p[k], (size_t)g.m * g.n);
    if (rc == IB_OK) w.rec(a.data(), 8 * a.size());
  }
  const bool closed = std::fclose(f) == 0;
  if (rc != IB_OK) { *msg = "device copy failed"; return rc; }
  if (!w.ok || !closed) { *msg = std::string("write to ") + path + " failed"; return IB_ERR_ARG; }
  return IB_OK;
}

}  // namespace ib
