// Batched DST-I kernels (see dst.cuh for the algorithm).
#include "dst.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace ib {

// ---------------------------------------------------------------- tables
// exp(-2 pi i num/den) evaluated in long double and rounded to double.
static double2 twiddle(long long num, long long den) {
  const long double PI_L = 3.141592653589793238462643383279502884L;
  long long r = num % den;
  if (r < 0) r += den;
  long double a = 2.0L * PI_L * (long double)r / (long double)den;
  return make_double2((double)cosl(a), (double)(-sinl(a)));
}

static bool factor_radices(int P, int* rad, int* nrad);

// The Stockham stages' twiddles, stage by stage: the stage of span Ns (the product of the earlier
// radices) and radix R uses w^(r k P/(Ns R)), r = 1..R-1, k = 0..Ns-1, stored at
// Ns - 1 + (r-1) Ns + k, so that a warp's lanes (consecutive k) read consecutive entries.  The
// stages' blocks [Ns - 1, R Ns - 1) tile [0, P - 1).
static void stage_twiddles(int P, const int* rad, int nrad, std::vector<double2>& tw) {
  tw.assign(P, make_double2(1.0, 0.0));
  int Ns = 1;
  for (int s = 0; s < nrad; ++s) {
    const int R = rad[s], step = P / (Ns * R);
    for (int r = 1; r < R; ++r)
      for (int k = 0; k < Ns; ++k) tw[Ns - 1 + (r - 1) * Ns + k] = twiddle((long long)r * k * step, P);
    Ns *= R;
  }
}

static bool factor_radices(int P, int* rad, int* nrad) {
  // radix-5 and radix-3 stages first (no twiddles in the first stage), then 4, then 2.
  int n = 0, q = P;
  while (q % 5 == 0) { rad[n++] = 5; q /= 5; }
  while (q % 3 == 0) { rad[n++] = 3; q /= 3; }
  while (q % 4 == 0) { rad[n++] = 4; q /= 4; }
  while (q % 2 == 0) { rad[n++] = 2; q /= 2; }
  if (q != 1 || n > kMaxRadices) return false;
  *nrad = n;
  return true;
}

int dst_plan_create(DstPlan* p, int N) {
  int M = N + 1;
  if (N < 3 || M % 4 != 0) return IB_ERR_ARG;
  p->N = N; p->M = M; p->P = M / 2;
  if (!factor_radices(p->P, p->rad, &p->nrad)) return IB_ERR_ARG;
  std::vector<double2> tw, uw(p->P / 2);
  std::vector<double> sn(p->P + 1);
  stage_twiddles(p->P, p->rad, p->nrad, tw);
  for (int k = 0; k < p->P / 2; ++k) uw[k] = twiddle(k, M);
  const long double PI_L = 3.141592653589793238462643383279502884L;
  for (int j = 0; j <= p->P; ++j) sn[j] = (double)sinl(PI_L * (long double)j / (long double)M);
  if (cudaMalloc(&p->tw, sizeof(double2) * p->P) != cudaSuccess) return IB_ERR_NOMEM;
  if (cudaMalloc(&p->uw, sizeof(double2) * (p->P / 2)) != cudaSuccess) return IB_ERR_NOMEM;
  if (cudaMalloc(&p->sn, sizeof(double) * (p->P + 1)) != cudaSuccess) return IB_ERR_NOMEM;
  IB_CUDA_CHECK(cudaMemcpy(p->tw, tw.data(), sizeof(double2) * p->P, cudaMemcpyHostToDevice));
  IB_CUDA_CHECK(cudaMemcpy(p->uw, uw.data(), sizeof(double2) * (p->P / 2), cudaMemcpyHostToDevice));
  IB_CUDA_CHECK(cudaMemcpy(p->sn, sn.data(), sizeof(double) * (p->P + 1), cudaMemcpyHostToDevice));
  return IB_OK;
}

size_t dst_plan_table_doubles(int N) {
  int M = N + 1;
  if (N < 3 || M % 4 != 0) return 0;
  int rad[kMaxRadices], nrad = 0;
  if (!factor_radices(M / 2, rad, &nrad)) return 0;
  int P = M / 2;
  return 2 * (size_t)P + 2 * (size_t)(P / 2) + (size_t)P + 1 + 4;
}

int dst_plan_init_external(DstPlan* p, int N, double* dev, cudaStream_t st) {
  int M = N + 1;
  if (dst_plan_table_doubles(N) == 0) return IB_ERR_ARG;
  p->N = N; p->M = M; p->P = M / 2;
  if (!factor_radices(p->P, p->rad, &p->nrad)) return IB_ERR_ARG;
  std::vector<double2> tw, uw(p->P / 2);
  std::vector<double> sn(p->P + 1);
  stage_twiddles(p->P, p->rad, p->nrad, tw);
  for (int k = 0; k < p->P / 2; ++k) uw[k] = twiddle(k, M);
  const long double PI_L = 3.141592653589793238462643383279502884L;
  for (int j = 0; j <= p->P; ++j) sn[j] = (double)sinl(PI_L * (long double)j / (long double)M);
  p->tw = reinterpret_cast<double2*>(dev);
  p->uw = p->tw + p->P;
  p->sn = reinterpret_cast<double*>(p->uw + p->P / 2);
  IB_CUDA_CHECK(cudaMemcpyAsync(p->tw, tw.data(), sizeof(double2) * p->P, cudaMemcpyHostToDevice, st));
  IB_CUDA_CHECK(cudaMemcpyAsync(p->uw, uw.data(), sizeof(double2) * (p->P / 2), cudaMemcpyHostToDevice, st));
  IB_CUDA_CHECK(cudaMemcpyAsync(p->sn, sn.data(), sizeof(double) * (p->P + 1), cudaMemcpyHostToDevice, st));
  IB_CUDA_CHECK(cudaStreamSynchronize(st));
  return IB_OK;
}

void dst_plan_destroy(DstPlan* p) {
  if (p->tw) cudaFree(p->tw);
  if (p->uw) cudaFree(p->uw);
  if (p->sn) cudaFree(p->sn);
  p->tw = p->uw = nullptr; p->sn = nullptr;
}

struct DstDev {
  int N, M, P, nrad;
  int rad[kMaxRadices];
  FastDiv fd_nb[kMaxRadices];   // butterflies per line of each stage (P/R)
  FastDiv fd_ns[kMaxRadices];   // span of each stage (product of the earlier radices)
  FastDiv fd_N, fd_P, fd_H;     // line length, complex length, half of it
  const double2* tw;
  const double2* uw;
  const double* sn;
};

static DstDev to_dev(const DstPlan& p) {
  DstDev d;
  d.N = p.N; d.M = p.M; d.P = p.P; d.nrad = p.nrad;
  int Ns = 1;
  for (int i = 0; i < kMaxRadices; ++i) {
    d.rad[i] = p.rad[i];
    if (i < p.nrad) {
      d.fd_nb[i] = FastDiv(p.P / p.rad[i]);
      d.fd_ns[i] = FastDiv(Ns);
      Ns *= p.rad[i];
    }
  }
  d.fd_N = FastDiv(p.N); d.fd_P = FastDiv(p.P); d.fd_H = FastDiv(p.P / 2);
  d.tw = p.tw; d.uw = p.uw; d.sn = p.sn;
  return d;
}

// ------------------------------------------------------- device helpers
__device__ __forceinline__ double2 cmul(double2 a, double2 w) {
  return make_double2(fma(a.x, w.x, -a.y * w.y), fma(a.x, w.y, a.y * w.x));
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

template <int R> struct Dft;
template <> struct Dft<2> {
  __device__ static void run(double2* v) {
    double2 a = v[0], b = v[1];
    v[0] = cadd(a, b); v[1] = csub(a, b);
  }
};
template <> struct Dft<4> {
  __device__ static void run(double2* v) {
    double2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    double2 s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    // y1 = d02 - i d13, y3 = d02 + i d13
    v[1] = make_double2(d02.x + d13.y, d02.y - d13.x);
    v[3] = make_double2(d02.x - d13.y, d02.y + d13.x);
  }
};
template <> struct Dft<3> {
  __device__ static void run(double2* v) {
    const double h = 0.86602540378443864676;  // sin(2 pi/3)
    double2 t = cadd(v[1], v[2]);
    double2 d = csub(v[1], v[2]);
    double2 a = make_double2(fma(-0.5, t.x, v[0].x), fma(-0.5, t.y, v[0].y));
    v[0] = cadd(v[0], t);
    v[1] = make_double2(fma(h, d.y, a.x), fma(-h, d.x, a.y));
    v[2] = make_double2(fma(-h, d.y, a.x), fma(h, d.x, a.y));
  }
};
template <> struct Dft<5> {
  __device__ static void run(double2* v) {
    const double c1 = 0.30901699437494742410;   // cos(2 pi/5)
    const double c2 = -0.80901699437494742410;  // cos(4 pi/5)
    const double s1 = 0.95105651629515357212;   // sin(2 pi/5)
    const double s2 = 0.58778525229247312917;   // sin(4 pi/5)
    double2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
    double2 d1 = csub(v[1], v[4]), d2 = csub(v[2], v[3]);
    double2 x0 = v[0];
    double2 a1 = make_double2(fma(c2, t2.x, fma(c1, t1.x, x0.x)), fma(c2, t2.y, fma(c1, t1.y, x0.y)));
    double2 a2 = make_double2(fma(c1, t2.x, fma(c2, t1.x, x0.x)), fma(c1, t2.y, fma(c2, t1.y, x0.y)));
    double2 b1 = make_double2(fma(s2, d2.x, s1 * d1.x), fma(s2, d2.y, s1 * d1.y));
    double2 b2 = make_double2(fma(-s1, d2.x, s2 * d1.x), fma(-s1, d2.y, s2 * d1.y));
    v[0] = cadd(cadd(x0, t1), t2);
    v[1] = make_double2(a1.x + b1.y, a1.y - b1.x);
    v[4] = make_double2(a1.x - b1.y, a1.y + b1.x);
    v[2] = make_double2(a2.x + b2.y, a2.y - b2.x);
    v[3] = make_double2(a2.x - b2.y, a2.y + b2.x);
  }
};

// One Stockham stage over B lines (line b at in + b*P).
template <int R>
__device__ __forceinline__ void stockham_stage(const double2* __restrict__ in, double2* __restrict__ out,
                                               int P, const FastDiv& fnb, const FastDiv& fns,
                                               const double2* __restrict__ tw, int B, int tid, int NT) {
  const int nb = fnb.d, Ns = fns.d;
  const int total = B * nb;
  const double2* __restrict__ tws = tw + Ns - 1;   // this stage's twiddles (stage_twiddles)
  for (int it = tid; it < total; it += NT) {
    int b = fnb.div(it);
    int j = it - b * nb;
    const double2* src = in + b * P;
    double2* dst = out + b * P;
    int jq = fns.div(j);
    int k = j - jq * Ns;
    double2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[j + r * nb];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], __ldg(&tws[(r - 1) * Ns + k]));
    }
    Dft<R>::run(v);
    int idxD = jq * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[idxD + r * Ns] = v[r];
  }
}

// Transform B lines in place: line b holds x_1..x_N at xb[b*ldx + 0..N-1] and
// receives Y_1..Y_N there.  zA, zB: B*P complex workspace each.
__device__ void dst_lines(const DstDev& pl, int B, double* xb, int ldx, double2* zA, double2* zB, int narrow_scan) {
  const int tid = threadIdx.x, NT = blockDim.x;
  const int P = pl.P, M = pl.M;
  // --- pre-processing: y (length M, real) written into zA viewed as doubles
  for (int it = tid; it < B * P; it += NT) {
    int b = pl.fd_P.div(it);
    int t = it - b * P;
    const double* x = xb + b * ldx;
    double* y = reinterpret_cast<double*>(zA + b * P);
    if (t == 0) {
      double xp = x[P - 1];
      y[0] = 0.0;
      y[P] = xp + xp;
    } else {
      double xj = x[t - 1], xm = x[M - t - 1];
      double a = xj + xm;
      double h = 0.5 * (xj - xm);
      double s = __ldg(&pl.sn[t]);
      y[t] = fma(s, a, h);
      y[M - t] = fma(s, a, -h);
    }
  }
  __syncthreads();
  // --- complex FFT of length P (Stockham, ping-pong zA <-> zB)
  double2* cur = zA;
  double2* nxt = zB;
  for (int s = 0; s < pl.nrad; ++s) {
    int R = pl.rad[s];
    switch (R) {
      case 2: stockham_stage<2>(cur, nxt, P, pl.fd_nb[s], pl.fd_ns[s], pl.tw, B, tid, NT); break;
      case 3: stockham_stage<3>(cur, nxt, P, pl.fd_nb[s], pl.fd_ns[s], pl.tw, B, tid, NT); break;
      case 4: stockham_stage<4>(cur, nxt, P, pl.fd_nb[s], pl.fd_ns[s], pl.tw, B, tid, NT); break;
      default: stockham_stage<5>(cur, nxt, P, pl.fd_nb[s], pl.fd_ns[s], pl.tw, B, tid, NT); break;
    }
    __syncthreads();
    double2* t = cur; cur = nxt; nxt = t;
  }
  // --- unpack the real FFT: even outputs directly, odd increments in place
  const int H = P / 2;
  for (int it = tid; it < B * H; it += NT) {
    int b = pl.fd_H.div(it);
    int k = it - b * H;
    const double2* Z = cur + b * P;
    double* o = xb + b * ldx;
    if (k == 0) {
      double2 z0 = Z[0];
      double2 zh = Z[H];
      o[0] = z0.x + z0.y;     // D_1
      o[P - 1] = zh.y + zh.y; // D_P
      o[P] = zh.x + zh.x;     // Re(2Y_{P/2})
    } else {
      double2 zk = Z[k], zp = Z[P - k];
      double2 E = make_double2(zk.x + zp.x, zk.y - zp.y);
      double2 O = make_double2(zk.y + zp.y, zp.x - zk.x);
      double2 T = cmul(O, __ldg(&pl.uw[k]));
      o[2 * k - 1] = -E.y - T.y;
      o[2 * k] = E.x + T.x;
      o[2 * (P - k) - 1] = E.y - T.y;
      o[2 * (P - k)] = E.x - T.x;
    }
  }
  __syncthreads();
  // --- inclusive prefix sum over positions 0,2,...,2(P-1): odd outputs
  const int lane = tid & 31, warp = tid >> 5, nwarps = NT >> 5;
  if (narrow_scan) {
    // one warp per line: sequential runs of ceil(P/32) per lane and a warp shuffle scan, the
    // fewest FP64 instructions (for launches whose other CTAs keep the SM busy meanwhile)
    const int c = (P + 31) >> 5;
    for (int b = warp; b < B; b += nwarps) {
      double* o = xb + b * ldx;
      const int s0 = min(lane * c, P), s1 = min(s0 + c, P);
      double acc = 0.0;
      for (int i = s0; i < s1; ++i) acc += o[2 * i];
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        double v = __shfl_up_sync(0xffffffffu, acc, off);
        if (lane >= off) acc += v;
      }
      double run = __shfl_up_sync(0xffffffffu, acc, 1);
      if (lane == 0) run = 0.0;
      for (int i = s0; i < s1; ++i) {
        run += o[2 * i];
        o[2 * i] = run;
      }
    }
    __syncthreads();
    return;
  }
  // every warp of the CTA takes part: a group of wpl warps per line, short sequential runs per
  // thread, a warp shuffle scan, then the group's warp totals in shared memory (the shortest
  // dependent chain, for latency-bound launches)
  __shared__ double s_wt[32];
  const int wpl = nwarps >= B ? nwarps / B : 1;           // warps per line
  const int groups = nwarps >= B ? B : nwarps;            // lines in flight at once
  const int c = (P + 32 * wpl - 1) / (32 * wpl);
  for (int b0 = 0; b0 < B; b0 += groups) {
    const int grp = warp / wpl, gw = warp - grp * wpl;
    const int b = b0 + grp;
    const bool act = grp < groups && b < B;
    double* o = xb + (act ? b : 0) * ldx;
    const int gt = gw * 32 + lane;
    const int s0 = min(gt * c, P), s1 = min(s0 + c, P);
    double acc = 0.0;
    if (act)
      for (int i = s0; i < s1; ++i) acc += o[2 * i];
    double incl = acc;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      double v = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += v;
    }
    if (lane == 31 && grp < groups) s_wt[grp * wpl + gw] = incl;
    double excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = 0.0;
    __syncthreads();
    if (act) {
      double run = 0.0;
      for (int j = 0; j < gw; ++j) run += s_wt[grp * wpl + j];
      run += excl;
      for (int i = s0; i < s1; ++i) {
        run += o[2 * i];
        o[2 * i] = run;
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------- x pass
// The pre-op operands of one CTA's level (the top-level fields, or level blockIdx.y of a batch).
struct XPre {
  const double *in2, *in3, *in4, *ring;
  double* save;
  double ca, cb, alpha, beta, fac;
  int bi0, bj0, bi1, bj1;   // PRE_ROT: the face box [bi0, bi1) x [bj0, bj1), read once per CTA
};
__device__ __forceinline__ XPre x_pre(const DstXArgs& a, int l, bool batch) {
  XPre p;
  if (batch) {
    p.in2 = a.lin2[l]; p.in3 = nullptr; p.in4 = a.lin4[l]; p.ring = a.lring[l]; p.save = a.lsave[l];
    p.ca = a.lca[l]; p.cb = a.lcb[l]; p.alpha = a.lalpha[l]; p.beta = a.lbeta[l]; p.fac = a.lfac[l];
    p.bi0 = p.bj0 = p.bi1 = p.bj1 = 0;
  } else {
    p.in2 = a.in2; p.in3 = a.in3; p.in4 = a.in4; p.ring = a.ring; p.save = a.save;
    p.ca = a.ca; p.cb = a.cb; p.alpha = a.alpha; p.beta = a.beta; p.fac = a.fac;
    p.bi0 = p.bj0 = p.bi1 = p.bj1 = 0;
    if (a.box) {
      p.bi0 = a.box[0];
      p.bj0 = a.box[1];
      p.bi1 = p.bi0 + a.box[2];
      p.bj1 = p.bj0 + a.box[3];
    }
  }
  return p;
}

template <int PRE>
__device__ __forceinline__ double x_load(const XPre& a, const double* __restrict__ in, const GridDims& g, int row,
                                         int j, int nrows, int N, int ld) {
  size_t idx = (size_t)row * ld + j;
  double v = 0.0;
  if (PRE == PRE_COPY) {
    v = in[idx];
  } else if (PRE == PRE_COMBINE) {
    v = fma(a.cb, a.in2[idx], a.ca * in[idx]) + a.in3[idx];
  } else if (PRE == PRE_ROT) {
    const int I = j + 2, J = row + 2;
    auto inbox = [&](int i, int jj) { return i >= a.bi0 && i < a.bi1 && jj >= a.bj0 && jj < a.bj1; };
    const double* hx = in;
    const double* hy = a.in2;
    const double va = inbox(I, J) ? hy[(size_t)(J - 1) * g.nvx + (I - 1)] : 0.0;
    const double vb = inbox(I - 1, J) ? hy[(size_t)(J - 1) * g.nvx + (I - 2)] : 0.0;
    const double vc = inbox(I, J) ? hx[(size_t)(J - 1) * g.nux + (I - 1)] : 0.0;
    const double vd = inbox(I, J - 1) ? hx[(size_t)(J - 2) * g.nux + (I - 1)] : 0.0;
    v = va - vb - vc + vd;
  } else if (PRE == PRE_PRED) {
    // con1 rhs + con2 rhs_old + rhsbc + (w - c L w)/normalize, L the 5-point
    // Laplacian with zero boundary: alpha = (1-4c)/normalize, beta = c/normalize
    const double ro = a.in2[idx], r = in[idx];
    double base = fma(a.cb, ro, a.ca * r);
    if (a.save) a.save[idx] = r;
    if (a.in3) {
      base = base + a.in3[idx];
    } else {
      const int I = j + 2, J = row + 2;
      if (I == 2 || I == g.m || J == 2 || J == g.n) {
        // rhsbc = 0; apply_bc(rhsbc, lastbc, f)
        double x = 0.0;
        const double* ra = a.ring;
        if (I == 2) x = x + a.fac * ra[g.left + J - 1];
        if (I == g.m) x = x + a.fac * ra[g.right + J - 1];
        if (J == 2) x = x + a.fac * ra[g.bottom + I - 1];
        if (J == g.n) x = x + a.fac * ra[g.top + I - 1];
        base = base + x;
      }
    }
    const double* w = a.in4;
    double nb = 0.0;
    if (j > 0) nb += w[idx - 1];
    if (j < N - 1) nb += w[idx + 1];
    if (row > 0) nb += w[idx - ld];
    if (row < nrows - 1) nb += w[idx + ld];
    v = fma(a.beta, nb, fma(a.alpha, w[idx], base));
  } else {
    // apply_bc (operators_fluid.F90:539-549): left, right, bottom, top; a null input is zero
    v = in ? in[idx] : 0.0;
    int I = j + 2, J = row + 2;
    if (I == 2) v = v + a.fac * a.ring[g.left + J - 1];
    if (I == g.m) v = v + a.fac * a.ring[g.right + J - 1];
    if (J == 2) v = v + a.fac * a.ring[g.bottom + I - 1];
    if (J == g.n) v = v + a.fac * a.ring[g.top + I - 1];
  }
  return v;
}

template <int PRE>
__global__ void __launch_bounds__(512) k_dst_x(DstDev pl, int nrows, int ld, const __grid_constant__ DstXArgs a,
                                               GridDims g, int B, int narrow_scan) {
  IB_GRID_DEP_WAIT();
  const double* ain = a.nlev ? a.lin[blockIdx.y] : a.in;
  double* aout = a.nlev ? a.lout[blockIdx.y] : a.out;
  const XPre pre = x_pre(a, blockIdx.y, PRE == PRE_PRED && a.nlev > 0);
  extern __shared__ double2 smem2[];
  __shared__ int s_mode[64];
  __shared__ int s_any;
  const int ldx = pl.M;
  double* xb = reinterpret_cast<double*>(smem2);
  double2* zA = smem2 + (B * ldx) / 2;
  double2* zB = zA + B * pl.P;
  const int N = pl.N;
  const int line0 = blockIdx.x * B;
  const int nl = a.nlines ? a.nlines : nrows;
  __shared__ int s_row[64];
  if (threadIdx.x == 0) s_any = 0;
  __syncthreads();
  if (threadIdx.x < B) {
    int line = line0 + threadIdx.x;
    int row = a.nlines ? a.row0 + line * a.row_step : line;
    s_row[threadIdx.x] = row;
    int mode = ROW_FFT;
    if (line >= nl || row >= nrows) mode = ROW_SKIP;
    else if (a.rowrange) {
      const int lo = max(0, a.rowrange[0] - a.row_margin), hi = min(nrows, a.rowrange[1] + a.row_margin);
      mode = (row >= lo && row < hi) ? ROW_FFT : a.rowrange[2];
      if (a.fft_edge_rows && (row == 0 || row == nrows - 1)) mode = ROW_FFT;
      if (a.rows_used && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) {
        a.rows_used[0] = lo;
        a.rows_used[1] = hi;
      }
    }
    else if (a.rowmode && (int)blockIdx.y >= a.rowmode_level0) mode = a.rowmode[row];
    s_mode[threadIdx.x] = mode;
    if (mode == ROW_FFT) atomicOr(&s_any, 1);
  }
  __syncthreads();
  const bool any_fft = s_any != 0;
  if (any_fft) {
    // 4 independent loads in flight per thread before the shared-memory stores
    const int tot = B * N, nt = blockDim.x;
    for (int it0 = threadIdx.x; it0 < tot; it0 += 4 * nt) {
      double v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        int it = it0 + u * nt;
        v[u] = 0.0;
        if (it < tot) {
          int b = pl.fd_N.div(it), j = it - b * N;
          if (s_mode[b] == ROW_FFT) v[u] = x_load<PRE>(pre, ain, g, s_row[b], j, nrows, N, ld);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        int it = it0 + u * nt;
        if (it < tot) {
          int b = pl.fd_N.div(it), j = it - b * N;
          xb[b * ldx + j] = v[u];
        }
      }
    }
    __syncthreads();
    dst_lines(pl, B, xb, ldx, zA, zB, narrow_scan);
  }
  for (int it = threadIdx.x; it < B * N; it += blockDim.x) {
    int b = pl.fd_N.div(it), j = it - b * N;
    int row = s_row[b];
    int mode = s_mode[b];
    if (mode == ROW_SKIP) continue;
    size_t o = (size_t)row * ld + j;
    double v;
    if (mode == ROW_FFT) {
      v = xb[b * ldx + j];
    } else if (mode == ROW_EDGES) {
      double x1 = x_load<PRE>(pre, ain, g, row, 0, nrows, N, ld);
      double xn = x_load<PRE>(pre, ain, g, row, N - 1, nrows, N, ld);
      int k = j + 1;
      double sk = __ldg(&pl.sn[k <= pl.P ? k : pl.M - k]);
      v = 2.0 * sk * ((k & 1) ? x1 + xn : x1 - xn);
    } else if (mode == ROW_SCALE) {
      v = a.row_scale * (a.nlev ? a.lin2[blockIdx.y] : a.in2)[o];
    } else {
      v = 0.0;
    }
    if (a.post_add) v = fma(a.post_scale, a.post_add[o], v);
    aout[o] = v;
  }
}


// fac * get_bc (operators_fluid.F90:475-535) of the inverse x transform of a coarser level's
// modes, without the transform (dot products with W at the points get_bc reads), and with it
// what the finer level's solve adds to its right-hand side modes
// (the boundary terms of apply_bc, operators_fluid.F90:539-549, transformed along x):
//  - sd[r] = x_1 + x_N and sd[nsy + r] = x_1 - x_N of its row r, the ring's left and right
//    entries r+1 (closed form 2 sin(pi k/M)(x_1 + (-1)^(k+1) x_N) of every row's two end values);
//  - edge[k] and edge[N + k]: the x transform of the ring's bottom and top entries 1..m-1,
//    which is fac E s_J, E the edge matrix and s_J the coarse modes of the row get_bc reads.
// The points get_bc reads come in mirror pairs about the centre column (the left and right
// sides; a bottom or top vertex and its mirror), and each pair is one warp's dot product
// (warp_sum_mirror); E keeps only its entries of equal parity.  CTAs of kReWarps warps:
// [0, nlr) take kReSeg entries of both the left and the right side (kReWarps vertex pairs);
// [nlr, nlr + 2 nbt) kReSeg entries of the left half of the bottom or top side and their
// mirrors; then one warp per mode k for the two edge dot products (dst_ring_from_modes launches
// the first two groups alone, sd and edge null).
constexpr int kReWarps = 8;
constexpr int kReSeg = 2 * (kReWarps - 1);   // entries a CTA writes on a side (kReWarps vertices)
__global__ void __launch_bounds__(32 * kReWarps) k_ring_edge(int N, GridDims g, const double* __restrict__ spec,
                                                             int ld, const double* __restrict__ W,
                                                             const double* __restrict__ Ec, double fac,
                                                             double* __restrict__ ring, double* __restrict__ sd,
                                                             double* __restrict__ edge, int nlr, int nbt) {
  IB_GRID_DEP_WAIT();
  __shared__ double sp[kReWarps], spm[kReWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int b = blockIdx.x;
  if (b < nlr) {
    // vertex q of the left side (row J = n/4+1+q, column m/4+1) and of the right (its mirror)
    const int len = g.n + 1, qmax = (len - 1) / 2;
    const int q0 = b * (kReSeg / 2), q = q0 + warp;
    double2 v = make_double2(0.0, 0.0);
    if (q <= qmax)
      v = warp_sum_mirror(warp_dot_part(spec + (size_t)(g.n / 4 - 1 + q) * ld, W + (size_t)(g.m / 4 - 1) * N, N, lane));
    if (lane == 0) {
      sp[warp] = v.x;
      spm[warp] = v.y;
    }
    __syncthreads();
    if ((int)threadIdx.x < kReSeg) {
      const int p = b * kReSeg + (int)threadIdx.x;
      if (p < len) {
        const int qq = p / 2 - q0;
        const double vl = (p & 1) ? 0.5 * (sp[qq] + sp[qq + 1]) : sp[qq];
        const double vr = (p & 1) ? 0.5 * (spm[qq] + spm[qq + 1]) : spm[qq];
        const double xl = vl * fac, xr = vr * fac;
        ring[g.left + p] = xl;
        ring[g.right + p] = xr;
        const int r = p - 1;
        if (sd && r >= 0 && r < g.nsy) {
          sd[r] = xl + xr;
          sd[g.nsy + r] = xl - xr;
        }
      }
    }
    return;
  }
  b -= nlr;
  if (b < 2 * nbt) {
    // vertex q <= m/4 of the bottom or top side (column m/4+1+q) and its mirror m/2-q
    const int side = b / nbt, cc = b - side * nbt;
    const int J = side == 0 ? g.n / 4 + 1 : 3 * g.n / 4 + 1;
    const int qc = g.m / 4;   // the centre vertex, its own mirror
    const int q0 = cc * (kReSeg / 2), q = q0 + warp;
    double2 v = make_double2(0.0, 0.0);
    if (q <= qc)
      v = warp_sum_mirror(warp_dot_part(spec + (size_t)(J - 2) * ld, W + (size_t)(g.m / 4 - 1 + q) * N, N, lane));
    if (lane == 0) {
      sp[warp] = v.x;
      spm[warp] = q == qc ? v.x : v.y;
    }
    __syncthreads();
    if ((int)threadIdx.x < kReSeg) {
      const int p = cc * kReSeg + (int)threadIdx.x;   // an entry of the left half
      if (p <= g.m / 2) {
        const int qq = p / 2 - q0;
        double* rs = ring + (side == 0 ? g.bottom : g.top);
        rs[p] = ((p & 1) ? 0.5 * (sp[qq] + sp[qq + 1]) : sp[qq]) * fac;
        if (p < g.m / 2) rs[g.m - p] = ((p & 1) ? 0.5 * (spm[qq] + spm[qq + 1]) : spm[qq]) * fac;
      }
    }
    return;
  }
  b -= 2 * nbt;
  const int k = b * kReWarps + warp;
  if (k >= N) return;
  const double2 e = warp_edge_dot(Ec, N, k, spec + (size_t)(g.n / 4 - 1) * ld, spec + (size_t)(3 * g.n / 4 - 1) * ld,
                                  lane);   // rows J = n/4 + 1 and 3n/4 + 1
  if (lane == 0) {
    edge[k] = fac * e.x;
    edge[N + k] = fac * e.y;
  }
}

// The ring alone (sd and edge null): the side and bottom/top CTAs only.
int dst_ring_from_modes(const DstPlan& px, const GridDims& g, const double* spec, int ld, const double* W, double fac,
                        double* ring, cudaStream_t st) {
  const int nlr = cdiv(g.n + 1, kReSeg), nbt = cdiv(g.m / 2 + 1, kReSeg);
  count_launch();
  k_ring_edge<<<nlr + 2 * nbt, 32 * kReWarps, 0, st>>>(px.N, g, spec, ld, W, nullptr, fac, ring, nullptr, nullptr,
                                                       nlr, nbt);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

int dst_ring_edge_from_modes(const DstPlan& px, const GridDims& g, const double* spec, int ld, const double* W,
                             const double* E, double fac, double* ring, double* sd, double* edge, cudaStream_t st) {
  const int nlr = cdiv(g.n + 1, kReSeg), nbt = cdiv(g.m / 2 + 1, kReSeg);
  count_launch();
  k_ring_edge<<<nlr + 2 * nbt + cdiv(px.N, kReWarps), 32 * kReWarps, 0, st>>>(px.N, g, spec, ld, W, E, fac, ring, sd,
                                                                              edge, nlr, nbt);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

// E[k][k'] = sum_j W[k][j] P(j, k'), P(j, .) the row of W at the coarse vertex get_bc puts on
// entry p = j+1 of a side (I = m/4 + 1 + p/2 for even p, the mean of two for odd p), for k' of
// k's parity (stored at t = k'/2 of row k, pitch (N+1)/2).  One thread per entry; compensated
// dot product (Ogita, Rump and Oishi's Dot2: error-free product by fma and Knuth's two-sum),
// so E is close to the exact product of the tabulated W.
__global__ void k_edge_matrix(int N, int mq, const double* __restrict__ W, double* __restrict__ E) {
  const int Nh = (N + 1) / 2;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)N * Nh) return;
  const int k = (int)(idx / Nh), kp = 2 * (int)(idx - (long long)k * Nh) + (k & 1);
  if (kp >= N) {
    E[idx] = 0.0;
    return;
  }
  const double* wk = W + (size_t)k * N;
  double sum = 0.0, comp = 0.0;
  for (int j = 0; j < N; ++j) {
    const int p = j + 1, r0 = mq - 1 + p / 2;
    const double pw = (p & 1) ? 0.5 * (W[(size_t)r0 * N + kp] + W[(size_t)(r0 + 1) * N + kp]) : W[(size_t)r0 * N + kp];
    const double a = wk[j];
    const double h = a * pw, l = fma(a, pw, -h);
    const double t = sum + h, z = t - sum;
    comp += ((sum - (t - z)) + (h - z)) + l;
    sum = t;
  }
  E[idx] = sum + comp;
}

int dst_edge_matrix(const DstPlan& px, const GridDims& g, const double* W, double* E) {
  const long long n = (long long)px.N * ((px.N + 1) / 2);
  k_edge_matrix<<<(unsigned)cdiv(n, 256), 256>>>(px.N, g.m / 4, W, E);
  IB_CUDA_CHECK(cudaGetLastError());
  IB_CUDA_CHECK(cudaDeviceSynchronize());
  return IB_OK;
}


// out = post_scale*post_add + S_x(apply_bc(ring)) on every row (operators_fluid.F90:539-549 with
// factor 1 on a zero field).  The first nEdge CTAs take the two edge rows 0 and n-2, whose
// boundary field is a full row: both rows are built once per CTA in shared memory and one warp
// per mode k reads row k of the (symmetric) DST matrix once for both dot products.  The other
// CTAs take kRowsPerCta interior rows each, whose boundary field is zero except
// x_1 = ring(left) and x_N = ring(right): Y_k = 2 sin(pi k/M)(x_1 + (-1)^(k+1) x_N), one FMA per
// output from the row's two sums and the tabulated 2 sin(pi k/M).  With fft_edges the two edge
// rows are instead transformed by the FFT line transform, one CTA each (about 2 x 700 FP64
// instructions instead of 2 N^2 multiply-adds: for the band build's and the sub-domain
// precompute's concurrent columns, which share the FP64 pipes).  In place allowed.
constexpr int kRowsPerCta = 8;
__global__ void __launch_bounds__(256) k_dst_bc_modes(DstDev pl, GridDims g, const double* __restrict__ ring,
                                                      const double* __restrict__ W, const double* __restrict__ sk2,
                                                      const double* __restrict__ post_add, double post_scale,
                                                      double* __restrict__ out, int nEdge, int fft_edges) {
  IB_GRID_DEP_WAIT();
  const int N = pl.N;
  if (fft_edges && (int)blockIdx.x < nEdge) {
    extern __shared__ double line[];   // the row (N, padded to N+1), then two P-point complex buffers
    double2* zA = reinterpret_cast<double2*>(line + (N + 1));
    double2* zB = zA + pl.P;
    const int e = blockIdx.x;
    const int J = e == 0 ? 2 : g.n;
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
      const int I = j + 2;
      double v = 0.0;
      if (I == 2) v = v + ring[g.left + J - 1];
      if (I == g.m) v = v + ring[g.right + J - 1];
      if (J == 2) v = v + ring[g.bottom + I - 1];
      if (J == g.n) v = v + ring[g.top + I - 1];
      line[j] = v;
    }
    __syncthreads();
    dst_lines(pl, 1, line, N + 1, zA, zB, 1);
    const size_t row = e == 0 ? 0 : (size_t)(g.nsy - 1) * g.nsx;
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
      const size_t o = row + k;
      out[o] = post_add ? fma(post_scale, post_add[o], line[k]) : line[k];
    }
    return;
  }
  if ((int)blockIdx.x >= nEdge) {
    __shared__ double s_sum[kRowsPerCta][2];   // x_1 + x_N, x_1 - x_N per row
    const int r0 = 1 + ((int)blockIdx.x - nEdge) * kRowsPerCta;
    const int nr = min(kRowsPerCta, g.nsy - 1 - r0);
    if ((int)threadIdx.x < nr) {
      const int J = r0 + (int)threadIdx.x + 2;
      const double x1 = 0.0 + ring[g.left + J - 1];
      const double xn = 0.0 + ring[g.right + J - 1];
      s_sum[threadIdx.x][0] = x1 + xn;
      s_sum[threadIdx.x][1] = x1 - xn;
    }
    __syncthreads();
    // out may alias post_add: every load of a thread's outputs is issued before its stores
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
      const double a = __ldg(&sk2[k]);
      const int par = (k & 1);   // mode kk = k+1 odd <=> k even
      double pa[kRowsPerCta];
#pragma unroll
      for (int i = 0; i < kRowsPerCta; ++i)
        pa[i] = (post_add && i < nr) ? post_add[(size_t)(r0 + i) * g.nsx + k] : 0.0;
#pragma unroll
      for (int i = 0; i < kRowsPerCta; ++i) {
        if (i >= nr) break;
        const double sv = s_sum[i][par];
        out[(size_t)(r0 + i) * g.nsx + k] = post_add ? fma(a, sv, post_scale * pa[i]) : a * sv;
      }
    }
    return;
  }
  extern __shared__ double bc[];   // 2 x N: rows 0 and n-2 of the boundary field
  for (int q = threadIdx.x; q < 2 * N; q += blockDim.x) {
    const int e = q / N, j = q - e * N;
    const int I = j + 2, J = e == 0 ? 2 : g.n;
    double v = 0.0;
    if (I == 2) v = v + ring[g.left + J - 1];
    if (I == g.m) v = v + ring[g.right + J - 1];
    if (J == 2) v = v + ring[g.bottom + I - 1];
    if (J == g.n) v = v + ring[g.top + I - 1];
    bc[q] = v;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (k >= N) return;
  const double* wk = W + (size_t)k * N;
  double a0 = 0.0, a1 = 0.0;
#pragma unroll 5
  for (int j = lane; j < N; j += 32) {
    const double w = wk[j];
    a0 = fma(bc[j], w, a0);
    a1 = fma(bc[N + j], w, a1);
  }
  for (int o = 16; o > 0; o >>= 1) {
    a0 += __shfl_xor_sync(0xffffffffu, a0, o);
    a1 += __shfl_xor_sync(0xffffffffu, a1, o);
  }
  if (lane == 0) {
    const size_t o0 = (size_t)k, o1 = (size_t)(g.nsy - 1) * g.nsx + k;
    out[o0] = post_add ? fma(post_scale, post_add[o0], a0) : a0;
    out[o1] = post_add ? fma(post_scale, post_add[o1], a1) : a1;
  }
}

int dst_x_bc_modes(const DstPlan& px, const GridDims& g, const double* ring, const double* W, const double* sk2,
                   const double* post_add, double post_scale, double* out, cudaStream_t st, bool fft_edges) {
  const int N = px.N;
  const size_t smem = fft_edges ? sizeof(double) * 3 * ((size_t)N + 1) : 2 * sizeof(double) * (size_t)N;
  if (allow_dyn_smem(k_dst_bc_modes, sizeof(double) * 3 * ((size_t)N + 1)) != cudaSuccess) return IB_ERR_CUDA;
  const int nEdge = fft_edges ? 2 : cdiv(N, 8);
  const int nblk = nEdge + cdiv(std::max(0, g.nsy - 2), kRowsPerCta);
  DstDev d = to_dev(px);
  count_launch();
  k_dst_bc_modes<<<nblk, 256, smem, st>>>(d, g, ring, W, sk2, post_add, post_scale, out, nEdge, fft_edges ? 1 : 0);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

int dst_sin2_table(const DstPlan& px, double* dev_out) {
  const long double PI_L = 3.141592653589793238462643383279502884L;
  std::vector<double> v(px.N);
  for (int k = 1; k <= px.N; ++k) {
    const int kk = k <= px.P ? k : px.M - k;   // the plan's sin table entry the transform uses
    const double sk = (double)sinl(PI_L * (long double)kk / (long double)px.M);
    v[k - 1] = 2.0 * sk;
  }
  IB_CUDA_CHECK(cudaMemcpy(dev_out, v.data(), 8 * v.size(), cudaMemcpyHostToDevice));
  return IB_OK;
}

int dst_matrix_table(const DstPlan& px, double* dev_out) {
  const long double PI_L = 3.141592653589793238462643383279502884L;
  const int N = px.N, M = px.M;
  // entry (j, k) is 2 sin(pi r / M) with r = jk mod 2M: one table of the 2M values (long double is
  // software-emulated on some hosts, so it is not evaluated N^2 times)
  std::vector<double> tab(2 * (size_t)M);
  for (long long r = 0; r < 2LL * M; ++r) tab[r] = (double)(2.0L * sinl(PI_L * (long double)r / (long double)M));
  std::vector<double> w((size_t)N * N);
  for (int j = 1; j <= N; ++j)
    for (int k = 1; k <= N; ++k) w[(size_t)(j - 1) * N + (k - 1)] = tab[(long long)j * k % (2LL * M)];
  IB_CUDA_CHECK(cudaMemcpy(dev_out, w.data(), 8 * w.size(), cudaMemcpyHostToDevice));
  return IB_OK;
}



// ------------------------------------------------------------- y pass
__global__ void __launch_bounds__(512) k_dst_y(DstDev pl, int ncols, int ld, DstYArgs a, int B, int narrow_scan) {
  IB_GRID_DEP_WAIT();
  extern __shared__ double2 smem2[];
  const int ldx = pl.M;
  const int N = pl.N;
  double* xa = reinterpret_cast<double*>(smem2);
  double2* zA = reinterpret_cast<double2*>(xa + B * ldx);
  double2* zB = zA + B * pl.P;
  const int col0 = blockIdx.x * B;
  for (int it = threadIdx.x; it < B * N; it += blockDim.x) {
    int j = it / B, b = it - j * B;
    int col = col0 + b;
    xa[b * ldx + j] = col < ncols ? a.a[(size_t)j * ld + col] : 0.0;
  }
  __syncthreads();
  dst_lines(pl, B, xa, ldx, zA, zB, narrow_scan);
  for (int it = threadIdx.x; it < B * N; it += blockDim.x) {
    int j = it / B, b = it - j * B;
    int col = col0 + b;
    if (col < ncols) a.a[(size_t)j * ld + col] = xa[b * ldx + j];
  }
}

size_t dst_smem_x(const DstPlan& p, int B) { return (size_t)B * p.M * 8 * 3; }
size_t dst_smem_y(const DstPlan& p, int B, DstYMode) { return (size_t)B * p.M * 8 * 3; }

template <typename K>
static int launch_cfg(K kern, size_t smem) {
  static_assert(sizeof(K) > 0, "");
  // the largest shared-memory carveout: the transforms' occupancy is bound by shared memory
  if (cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared) !=
      cudaSuccess)
    return IB_ERR_CUDA;
  if (allow_dyn_smem(kern, smem) != cudaSuccess) return IB_ERR_CUDA;
  return IB_OK;
}

int dst_pass_x(const DstPlan& px, int nrows, int ld, DstPre pre, const DstXArgs& a, const GridDims& g,
               const DstLaunch& L, cudaStream_t st) {
  if (a.nlev < 0 || a.nlev > kMaxBatch || (a.nlev && pre != PRE_COPY && pre != PRE_PRED)) return IB_ERR_ARG;
  DstDev d = to_dev(px);
  size_t smem = dst_smem_x(px, L.B);
  dim3 grid(cdiv(a.nlines ? a.nlines : nrows, L.B), a.nlev ? a.nlev : 1);
  int rc = IB_OK;
  switch (pre) {
    case PRE_COPY:
      rc = launch_cfg(k_dst_x<PRE_COPY>, smem);
      if (rc) return rc;
      count_launch();
      k_dst_x<PRE_COPY><<<grid, L.NT, smem, st>>>(d, nrows, ld, a, g, L.B, L.narrow_scan);
      break;
    case PRE_COMBINE:
      rc = launch_cfg(k_dst_x<PRE_COMBINE>, smem);
      if (rc) return rc;
      count_launch();
      k_dst_x<PRE_COMBINE><<<grid, L.NT, smem, st>>>(d, nrows, ld, a, g, L.B, L.narrow_scan);
      break;
    case PRE_PRED:
      rc = launch_cfg(k_dst_x<PRE_PRED>, smem);
      if (rc) return rc;
      count_launch();
      k_dst_x<PRE_PRED><<<grid, L.NT, smem, st>>>(d, nrows, ld, a, g, L.B, L.narrow_scan);
      break;
    case PRE_ROT:
      if (!a.box || !a.in2) return IB_ERR_ARG;
      rc = launch_cfg(k_dst_x<PRE_ROT>, smem);
      if (rc) return rc;
      count_launch();
      k_dst_x<PRE_ROT><<<grid, L.NT, smem, st>>>(d, nrows, ld, a, g, L.B, L.narrow_scan);
      break;
    default:
      rc = launch_cfg(k_dst_x<PRE_APPLYBC>, smem);
      if (rc) return rc;
      count_launch();
      k_dst_x<PRE_APPLYBC><<<grid, L.NT, smem, st>>>(d, nrows, ld, a, g, L.B, L.narrow_scan);
      break;
  }
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

int dst_pass_y(const DstPlan& py, int ncols, int ld, DstYMode, const DstYArgs& a, const DstLaunch& L,
               cudaStream_t st) {
  DstDev d = to_dev(py);
  size_t smem = dst_smem_y(py, L.B, YMODE_NONE);
  dim3 grid(cdiv(ncols, L.B));
  int rc = launch_cfg(k_dst_y, smem);
  if (rc) return rc;
  count_launch();
  k_dst_y<<<grid, L.NT, smem, st>>>(d, ncols, ld, a, L.B, L.narrow_scan);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

}  // namespace ib
