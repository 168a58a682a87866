// The reference's input files: the namelist &read_parameters of input/ib.inp (parameters.F90:
// 51-78) and the body files input/body.NNN.inp (grid.F90:252-288), read on the host.
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ib_gpu.h"

namespace ib {

void set_last_error(const char* msg);  // capi.cu

namespace {

bool read_file(const char* path, std::string* out) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  char buf[65536];
  size_t n;
  out->clear();
  while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) out->append(buf, n);
  std::fclose(f);
  return true;
}

std::string lower(std::string s) {
  for (char& ch : s) ch = (char)std::tolower((unsigned char)ch);
  return s;
}

// A Fortran real constant (E or D exponent, optional sign); the whole token must be used.
bool parse_real(const std::string& t, double* v) {
  if (t.empty()) return false;
  std::string u = t;
  for (char& ch : u)
    if (ch == 'd' || ch == 'D') ch = 'e';
  char* end = nullptr;
  *v = std::strtod(u.c_str(), &end);
  return end && *end == '\0' && end != u.c_str();
}

bool parse_int(const std::string& t, int* v) {
  if (t.empty()) return false;
  char* end = nullptr;
  long x = std::strtol(t.c_str(), &end, 10);
  if (!end || *end != '\0' || end == t.c_str() || x < -2147483647L || x > 2147483647L) return false;
  *v = (int)x;
  return true;
}

// A Fortran logical value: T, F, .T., .F., .TRUE., .FALSE. (any case; as list-directed input
// accepts, the first letter after an optional period decides).
bool parse_logical(const std::string& t, int* v) {
  std::string u = lower(t);
  size_t i = u.empty() || u[0] != '.' ? 0 : 1;
  if (i >= u.size()) return false;
  if (u[i] == 't') { *v = 1; return true; }
  if (u[i] == 'f') { *v = 0; return true; }
  return false;
}

}  // namespace

int read_namelist(const char* path, IbParams* p, IbRunControl* rc, std::string* msg) {
  std::string text;
  if (!read_file(path, &text)) { *msg = std::string("cannot open ") + path; return IB_ERR_ARG; }
  // comments: '!' to the end of the line
  std::string body;
  for (size_t i = 0; i < text.size(); ++i) {
    if (text[i] == '!') {
      while (i < text.size() && text[i] != '\n') ++i;
      if (i < text.size()) body += '\n';
      continue;
    }
    body += text[i];
  }
  const std::string lb = lower(body);
  const size_t g = lb.find("&read_parameters");
  if (g == std::string::npos) { *msg = "no &read_parameters group"; return IB_ERR_ARG; }
  const size_t start = g + std::strlen("&read_parameters");
  const size_t stop = body.find('/', start);
  if (stop == std::string::npos) { *msg = "namelist group not terminated by '/'"; return IB_ERR_ARG; }
  // tokens: names, '=', values (commas and blanks separate)
  std::vector<std::string> tok;
  std::string cur;
  auto flush = [&]() { if (!cur.empty()) { tok.push_back(cur); cur.clear(); } };
  for (size_t i = start; i < stop; ++i) {
    const char ch = body[i];
    if (ch == '=') { flush(); tok.push_back("="); }
    else if (ch == ',' || std::isspace((unsigned char)ch)) flush();
    else cur += ch;
  }
  flush();
  for (size_t i = 0; i < tok.size(); i += 3) {
    if (i + 2 >= tok.size() || tok[i + 1] != "=") { *msg = "malformed item near '" + tok[i] + "'"; return IB_ERR_ARG; }
    const std::string key = lower(tok[i]), val = tok[i + 2];
    bool ok = true;
    int iv = 0;
    double dv = 0.0;
    auto I = [&](int* dst) { ok = parse_int(val, &iv); if (ok) *dst = iv; };
    auto R = [&](double* dst) { ok = parse_real(val, &dv); if (ok) *dst = dv; };
    auto B = [&](int* dst) { ok = parse_logical(val, &iv); if (ok) *dst = iv; };
    if (key == "istart") I(&rc->istart);
    else if (key == "istop") I(&rc->istop);
    else if (key == "isave") I(&rc->isave);
    else if (key == "irestart") I(&rc->irestart);
    else if (key == "m") I(&p->m);
    else if (key == "n") I(&p->n);
    else if (key == "dt") R(&p->dt);
    else if (key == "re") R(&p->Re);
    else if (key == "fsi_tol") R(&p->fsi_tol);
    else if (key == "atol") R(&p->atol);
    else if (key == "rtol") R(&p->rtol);
    else if (key == "len") R(&p->len);
    else if (key == "offsetx") R(&p->offsetx);
    else if (key == "offsety") R(&p->offsety);
    else if (key == "mgridlev") I(&p->mgridlev);
    else if (key == "compute_pressure") B(&rc->compute_pressure);
    else if (key == "dimen") I(&rc->dimen);
    else if (key == "num_stat") B(&p->num_stat);
    else if (key == "motion_prescribed") B(&rc->motion_prescribed);
    else if (key == "sub_domain") B(&rc->sub_domain);
    else if (key == "sub_domain_full_rectangular") B(&rc->sub_domain_full_rectangular);
    else if (key == "sub_domain_precomputed") B(&rc->sub_domain_precomputed);
    else if (key == "sdxi") R(&rc->sdxi);
    else if (key == "sdxe") R(&rc->sdxe);
    else if (key == "sdyi") R(&rc->sdyi);
    else if (key == "sdye") R(&rc->sdye);
    else if (key == "delta_sd") R(&rc->delta_sd);
    else { *msg = "unknown namelist item '" + tok[i] + "'"; return IB_ERR_ARG; }
    if (!ok) { *msg = "bad value '" + val + "' for " + tok[i]; return IB_ERR_ARG; }
  }
  return IB_OK;
}

// List-directed reads of a body file: each READ takes the values it needs from the current
// line on (continuing onto following lines if the line runs short) and then moves to the line
// after the last one it used.
namespace {
struct ListReader {
  std::vector<std::string> lines;
  size_t line = 0;
  bool values(size_t k, std::vector<std::string>* out) {
    out->clear();
    while (out->size() < k) {
      if (line >= lines.size()) return false;
      std::string cur;
      const std::string& L = lines[line++];
      for (size_t i = 0; i <= L.size() && out->size() < k; ++i) {
        const char ch = i < L.size() ? L[i] : ' ';
        if (ch == ',' || std::isspace((unsigned char)ch)) {
          if (!cur.empty()) { out->push_back(cur); cur.clear(); }
        } else {
          cur += ch;
        }
      }
    }
    return true;
  }
};
}  // namespace

int read_body(const char* path, IbBody* b, double* x, double* y, int cap, std::string* msg) {
  std::string text;
  if (!read_file(path, &text)) { *msg = std::string("cannot open ") + path; return IB_ERR_ARG; }
  ListReader r;
  size_t s = 0;
  for (size_t i = 0; i <= text.size(); ++i)
    if (i == text.size() || text[i] == '\n') {
      std::string L = text.substr(s, i - s);
      if (!L.empty() && L.back() == '\r') L.pop_back();
      r.lines.push_back(L);
      s = i + 1;
    }
  std::vector<std::string> v;
  int npts = 0, fam = 0;
  if (!r.values(1, &v) || !parse_int(v[0], &npts) || npts < 1) { *msg = "bad point count"; return IB_ERR_ARG; }
  if (!r.values(1, &v) || !parse_int(v[0], &fam)) { *msg = "bad body family '" + (v.empty() ? "" : v[0]) + "'"; return IB_ERR_ARG; }
  double g0 = 0.0, a0 = 0.0, it = 0.0, kt = 0.0, ct = 0.0;
  int nel = 0;
  if (fam == 2) {
    double* dst[5] = {&g0, &a0, &it, &kt, &ct};
    for (double* d : dst)
      if (!r.values(1, &v) || !parse_real(v[0], d)) { *msg = "bad torsion parameter"; return IB_ERR_ARG; }
  } else if (fam == 3) {
    // the beam family has no file layout in the reference: mass per unit length, bending
    // stiffness EI and the number of elements, one per line, as the torsion parameters are
    if (!r.values(1, &v) || !parse_real(v[0], &it) || !r.values(1, &v) || !parse_real(v[0], &kt) ||
        !r.values(1, &v) || !parse_int(v[0], &nel)) { *msg = "bad beam parameter"; return IB_ERR_ARG; }
  }
  b->npts = npts;
  b->fam = fam;
  b->gamma0_deg = g0; b->alpha0_deg = a0; b->itheta = it; b->ktheta = kt; b->ctheta = ct;
  b->nelem = nel;
  b->x = x; b->y = y;
  if (cap < npts || !x || !y) {
    *msg = "arrays hold " + std::to_string(cap) + " points, the body has " + std::to_string(npts);
    return IB_ERR_ARG;
  }
  for (int i = 0; i < npts; ++i) {
    double xv, yv;
    if (!r.values(2, &v) || !parse_real(v[0], &xv) || !parse_real(v[1], &yv)) {
      *msg = "bad coordinates of point " + std::to_string(i + 1);
      return IB_ERR_ARG;
    }
    x[i] = xv;
    y[i] = yv;
  }
  return IB_OK;
}

}  // namespace ib

extern "C" {

int ib_read_namelist(const char* path, IbParams* p, IbRunControl* rc) {
  if (!path || !p || !rc) { ib::set_last_error("ib_read_namelist: null argument"); return IB_ERR_ARG; }
  std::string msg;
  int r = ib::read_namelist(path, p, rc, &msg);
  if (r != IB_OK) ib::set_last_error(("ib_read_namelist: " + msg).c_str());
  return r;
}

int ib_read_body(const char* path, IbBody* body, double* x, double* y, int cap) {
  if (!path || !body) { ib::set_last_error("ib_read_body: null argument"); return IB_ERR_ARG; }
  std::string msg;
  int r = ib::read_body(path, body, x, y, cap, &msg);
  if (r != IB_OK) ib::set_last_error(("ib_read_body: " + std::string(path) + ": " + msg).c_str());
  return r;
}

int ib_count_bodies(const char* dir, int* nbody) {
  if (!dir || !nbody) { ib::set_last_error("ib_count_bodies: null argument"); return IB_ERR_ARG; }
  int k = 0;
  for (;;) {
    char name[32];
    std::snprintf(name, sizeof(name), "/body.%03d.inp", k + 1);
    FILE* f = std::fopen((std::string(dir) + name).c_str(), "rb");
    if (!f) break;
    std::fclose(f);
    if (++k >= 999) break;
  }
  *nbody = k;
  return IB_OK;
}

}  // extern "C"
