// Torsional-body (family 2) structure operators of operators_struct.F90: a rigid
// plate hinged at its first point on a torsional spring/damper, integrated with
// the trapezoidal Newmark scheme.  Each body is handled by one CTA; the only
// reduction is the BR . x dot product.  The scalar recurrences (sin, cos, divisions)
// are FP64-latency-bound and every thread evaluates them, so rhs, dx and initial_acc
// run one warp per body; b_times keeps 256 threads, whose reduction order the fused
// Krylov kernel reproduces.  Gravity and pseudo-forces are zero in the
// reference user hooks (user.F90:178-206) and are omitted.
#include "fsi_dev.cuh"

namespace ib {


__device__ double block_sum(double v) {
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
    red[0] = s;
  }
  __syncthreads();
  s = red[0];
  __syncthreads();
  return s;
}


// b_times2 (operators_struct.F90:14-127): y += BR (BR . x)/K_eff * (delta^2/ds/dt)(2 ds/dt)
__global__ void k_tors_btimes(const TorsBody* __restrict__ tb, TorsState s, double dt, double delta,
                              const double* __restrict__ x, double* __restrict__ y) {
  IB_GRID_DEP_WAIT();
  TorsBody b = tb[blockIdx.x];
  double sn = s.sinv[blockIdx.x], cs = s.cosv[blockIdx.x];
  double part = 0.0;
  for (int j = threadIdx.x; j < 2 * b.npts; j += blockDim.x) part += br_val(b, sn, cs, j) * x[b.off + j];
  double dot = block_sum(part);
  double c = dot / keff(b, dt) * btimes_scale(b, dt, delta);
  for (int j = threadIdx.x; j < 2 * b.npts; j += blockDim.x) y[b.off + j] = y[b.off + j] + br_val(b, sn, cs, j) * c;
}

// compute_rhs (operators_struct.F90:342-398): y = BR * delta*(r_theta - J r_phi - thetad)
__global__ void k_tors_rhs(const TorsBody* __restrict__ tb, TorsState s, double dt, double delta,
                           double* __restrict__ y) {
  IB_GRID_DEP_WAIT();
  int t = blockIdx.x;
  TorsBody b = tb[t];
  double th = s.theta[t], th0 = s.theta0[t], thd = s.thetad[t], thd0 = s.thetad0[t], thdd0 = s.thetadd0[t];
  double I = b.itheta, C = b.ctheta, K = b.ktheta;
  double rth = thd0 + thd + 2.0 / dt * (th0 - th);
  double jr = 2.0 / dt / (4.0 / (dt * dt) * I + 2.0 / dt * C + K) *
              (I * (4.0 / (dt * dt) * th0 + 4.0 / dt * thd0 + thdd0) + C * (thd0 + 2.0 / dt * th0) -
               (4.0 / (dt * dt) * I + 2.0 / dt * C + K) * th);
  double c = delta * (rth - jr - thd);
  double sn = s.sinv[t], cs = s.cosv[t];
  for (int j = threadIdx.x; j < 2 * b.npts; j += blockDim.x) y[b.off + j] = br_val(b, sn, cs, j) * c;
}

// compute_dx + update_xb (operators_struct.F90:402-505, 600-620); err = max |dtheta|.  One
// warp per body (tors_dx_warp).
__global__ void k_tors_dx(const TorsBody* __restrict__ tb, TorsState s, double dt, double delta,
                          const double* __restrict__ f, double* __restrict__ xb, double* __restrict__ yb,
                          double* __restrict__ err_per_body, double* __restrict__ err_max) {
  IB_GRID_DEP_WAIT();
  const int t = blockIdx.x;
  const TorsBody b = tb[t];
  const TorsDx u = tors_dx_warp(b, s, t, f);
  const double cg = cos(u.g), sg = sin(u.g);
  const double th0 = s.theta0[t], thd0 = s.thetad0[t], thdd0 = s.thetadd0[t];
  __syncwarp();   // every lane has read the old theta, sinv, cosv
  if (threadIdx.x == 0) {
    s.theta[t] = u.thn;
    tors_rates(b, u.thn, th0, thd0, thdd0, &s.thetad[t], &s.thetadd[t]);
    err_per_body[t] = fabs(u.dth);
    if (err_max) *err_max = fabs(u.dth);   // one body: its error is the maximum
    s.sinv[t] = sg;
    s.cosv[t] = cg;
  }
  for (int j = threadIdx.x; j < 2 * b.npts; j += blockDim.x) {
    const double2 pp = tors_point(b, j, sg, cg);
    xb[b.off + j] = pp.x;
    yb[b.off + j] = pp.y;
  }
}

__global__ void k_tors_consts(int nt, TorsBody* tb, double dt, double delta) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  TorsBody& b = tb[t];
  const double I = b.itheta, C = b.ctheta, K = b.ktheta;
  b.a44 = 4.0 / (dt * dt);
  b.a4 = 4.0 / dt;
  b.a2 = 2.0 / dt;
  b.keff = b.a44 * I + b.a2 * C + K;
  b.keff_inv = 1.0 / b.keff;
  b.bq = b.deltas / (b.a44 * I + K);
  b.bs = delta / b.deltas / dt;
}

int launch_tors_consts(int nt, TorsBody* tb, double dt, double delta, cudaStream_t st) {
  if (nt == 0) return IB_OK;
  k_tors_consts<<<cdiv(nt, 128), 128, 0, st>>>(nt, tb, dt, delta);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

__global__ void k_max_reduce(int n, const double* __restrict__ v, double* out) {
  IB_GRID_DEP_WAIT();
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, v[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (threadIdx.x == 0) out[0] = m;
}

// initial_acc (operators_struct.F90:233-294)
__global__ void k_tors_initial_acc(const TorsBody* __restrict__ tb, TorsState s, double dt, double delta,
                                   const double* __restrict__ f) {
  IB_GRID_DEP_WAIT();
  int t = blockIdx.x;
  TorsBody b = tb[t];
  double th = s.theta[t];
  double sn = s.sinv[t], cs = s.cosv[t];
  double part = 0.0;
  for (int j = threadIdx.x; j < 2 * b.npts; j += blockDim.x) part += br_val(b, sn, cs, j) * f[b.off + j];
  double brf = block_sum(part);
  brf = brf * delta / b.deltas / dt;
  if (threadIdx.x == 0) {
    double ftint = b.ktheta * th;
    s.thetadd[t] = 1.0 / b.itheta * (-b.ctheta * s.thetad[t] - ftint + brf * b.deltas);
  }
}

__global__ void k_tors_trig(int nt, const TorsBody* __restrict__ tb, TorsState s) {
  IB_GRID_DEP_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  double g = tb[t].gamma0 - s.theta[t];
  s.sinv[t] = sin(g);
  s.cosv[t] = cos(g);
}

__global__ void k_tors_save(int nt, TorsState s) {
  IB_GRID_DEP_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  s.theta0[t] = s.theta[t];
  s.thetad0[t] = s.thetad[t];
  s.thetadd0[t] = s.thetadd[t];
}

int launch_tors_btimes(int nt, const TorsBody* tb, const TorsState& s, double dt, double delta, const double* x,
                       double* y, cudaStream_t st) {
  if (nt == 0) return IB_OK;
  count_launch();
  k_tors_btimes<<<nt, 256, 0, st>>>(tb, s, dt, delta, x, y);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}
int launch_tors_rhs(int nt, const TorsBody* tb, const TorsState& s, double dt, double delta, double* y,
                    cudaStream_t st) {
  if (nt == 0) return IB_OK;
  count_launch();
  k_tors_rhs<<<nt, 32, 0, st>>>(tb, s, dt, delta, y);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}
int launch_tors_dx(int nt, const TorsBody* tb, const TorsState& s, double dt, double delta, const double* f,
                   double* xb, double* yb, double* err, cudaStream_t st) {
  if (nt == 0) {
    IB_CUDA_CHECK(cudaMemsetAsync(err, 0, sizeof(double), st));
    return IB_OK;
  }
  // err[1..nt] holds per-body |dtheta|, err[0] their maximum
  count_launch();
  k_tors_dx<<<nt, 32, 0, st>>>(tb, s, dt, delta, f, xb, yb, err + 1, nt == 1 ? err : nullptr);
  if (nt > 1) {
    count_launch();
    k_max_reduce<<<1, 32, 0, st>>>(nt, err + 1, err);
  }
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}
int launch_tors_initial_acc(int nt, const TorsBody* tb, const TorsState& s, double dt, double delta,
                            const double* f, cudaStream_t st) {
  if (nt == 0) return IB_OK;
  count_launch();
  k_tors_initial_acc<<<nt, 32, 0, st>>>(tb, s, dt, delta, f);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}
int launch_tors_trig(int nt, const TorsBody* tb, const TorsState& s, cudaStream_t st) {
  if (nt == 0) return IB_OK;
  count_launch();
  k_tors_trig<<<cdiv(nt, 64), 64, 0, st>>>(nt, tb, s);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

int launch_tors_save(int nt, const TorsState& s, cudaStream_t st) {
  if (nt == 0) return IB_OK;
  count_launch();
  k_tors_save<<<cdiv(nt, 64), 64, 0, st>>>(nt, s);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

}  // namespace ib
