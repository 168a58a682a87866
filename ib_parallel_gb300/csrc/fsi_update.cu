// The end of one device FSI iteration in one kernel: structure update, weights and influence
// patches at the new positions (k_tors_dx, k_reg_weights and k_inf_patch of the host loop, on
// the same device bodies), and the loop condition.
#include "fsi_dev.cuh"

namespace ib {

// One CTA of 4 warps per 8 unknowns:
//  1. warps 0 and 1 evaluate the structure update of every torsional body with unknowns in
//     the CTA's range (each such CTA evaluates it alike), then sin and cos of the new angle side
//     by side; the CTA holding a body's first unknown writes its state, theta, sin and cos to
//     th_next/sin_next/cos_next (the other CTAs still read the current ones);
//  2. the positions of the CTA's unknowns (moved or read), their origins and weights;
//  3. their patches;
//  4. the CTA that finishes last (a ticket taken after a fence: no CTA waits for another)
//     commits theta, sin and cos, forms the maximum error and the loop condition of
//     timestepper.F90:249, keeps the most negative reason of the iterations' Krylov solves,
//     clears the band flag for the next patches and resets the ticket.
__global__ void __launch_bounds__(128) k_fsi_update(FsiUpdateArgs a) {
  IB_GRID_DEP_WAIT();
  __shared__ double fac[16][7];
  __shared__ double pos[8][2];
  __shared__ double wsm[8][49];
  __shared__ int org[8][2];
  __shared__ int moved[8];
  __shared__ int is_last;
  __shared__ double sc[8][2];    // sin, cos of the torsional bodies met (at most 4 in 8 unknowns)
  __shared__ int bt[8];
  __shared__ double bth[8][2];   // theta_new, dtheta
  const int k0 = blockIdx.x * 8, kend = min(a.nf, k0 + 8);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid < 8) moved[tid] = 0;
  // the torsional bodies with unknowns in [k0, kend): each evaluated alike by warps 0 and 1,
  // which then take sin and cos of the new angle side by side
  int nb = 0;
  if (warp < 2) {
    for (int t = 0; t < a.nt && nb < 8; ++t) {
      const TorsBody b = a.tb[t];
      if (b.off >= kend || b.off + 2 * b.npts <= k0) continue;
      const TorsDx u = tors_dx_warp(b, a.ts, t, a.f);
      const double v = warp == 0 ? sin(u.g) : cos(u.g);
      if (lane == 0) {
        sc[nb][warp] = v;
        if (warp == 0) {
          bt[nb] = t;
          bth[nb][0] = u.thn;
          bth[nb][1] = u.dth;
        }
      }
      ++nb;
    }
  }
  __syncthreads();
  if (warp == 0) {
    for (int i = 0; i < nb; ++i) {
      const int t = bt[i];
      const TorsBody b = a.tb[t];
      const double sg = sc[i][0], cg = sc[i][1], thn = bth[i][0];
      if (lane == 0 && b.off >= k0) {   // the body's first unknown is in this CTA
        const double th0 = a.ts.theta0[t], thd0 = a.ts.thetad0[t], thdd0 = a.ts.thetadd0[t];
        tors_rates(b, thn, th0, thd0, thdd0, &a.ts.thetad[t], &a.ts.thetadd[t]);
        a.err[1 + t] = fabs(bth[i][1]);
        a.th_next[t] = thn;
        a.sin_next[t] = sg;
        a.cos_next[t] = cg;
      }
      const int k = k0 + lane;
      if (lane < 8 && k < kend && k >= b.off && k < b.off + 2 * b.npts) {
        const double2 pp = tors_point(b, k - b.off, sg, cg);
        a.xb[k] = pp.x;
        a.yb[k] = pp.y;
        pos[lane][0] = pp.x;
        pos[lane][1] = pp.y;
        moved[lane] = 1;
      }
    }
  }
  __syncthreads();
  if (tid < 8 && k0 + tid < kend && !moved[tid]) {
    pos[tid][0] = a.xb[k0 + tid];
    pos[tid][1] = a.yb[k0 + tid];
  }
  __syncthreads();
  reg_weights_cta(a.g, a.nf, k0, pos, a.delta, a.ox, a.oy, a.comp, a.ix, a.iy, a.w, a.stale, a.d_err, fac, wsm,
                  org);
  if (a.rows && tid < 8 && k0 + tid < kend) {
    // E(curl s) at this stencil reads the streamfunction on vertex rows cy-5 .. cy+2
    const int cy = org[tid][1];
    const int r0 = max(0, cy - 5), r1 = min(a.g.nsy - 1, cy + 2);
    if (r0 < a.rows[0] || r1 >= a.rows[1]) atomicOr(a.flag, 4);
  }
  for (int t = tid; a.pval && t < 8 * 64; t += blockDim.x) {   // no patches without a band
    const int u = t >> 6, q = t & 63;
    if (k0 + u >= kend) break;
    patch_entry(a.g, k0 + u, q, a.comp[k0 + u] == 1, org[u][0], org[u][1], wsm[u], a.tile_of, a.ntx, a.tile,
                a.pval, a.pidx, a.used, a.flag);
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) is_last = atomicAdd(a.done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!is_last || tid != 0) return;
  __threadfence();
  for (int t = 0; t < a.nt; ++t) {
    a.ts.theta[t] = a.th_next[t];
    a.ts.sinv[t] = a.sin_next[t];
    a.ts.cosv[t] = a.cos_next[t];
  }
  double e = 0.0;
  if (a.nt == 1) {
    e = a.err[1];
  } else if (a.nt > 1) {
    for (int t = 0; t < a.nt; ++t) e = fmax(e, a.err[1 + t]);
  }
  a.err[0] = e;
  const int n = a.cnt[0] + 1;
  const int bf = *a.flag;
  *a.flag = 0;   // the next iteration's patches start from zero
  a.cnt[0] = n;
  a.cnt[1] += a.ist[0];
  a.cnt[2] += a.ist[0] + a.ist[4];
  a.cnt[3] = bf;
  a.cnt[4] = min(a.cnt[4], a.ist[1]);   // a failed Krylov solve (negative KSP reason) sticks
  const bool go = isfinite(e) && e >= a.tol && n <= a.max_it && bf == 0;
  cudaGraphSetConditional(a.h, go ? 1u : 0u);
  *a.done = 0u;
}

int launch_fsi_update(const FsiUpdateArgs& a, cudaStream_t st) {
  if (a.nf <= 0) return IB_ERR_ARG;
  count_launch();
  k_fsi_update<<<cdiv(a.nf, 8), 128, 0, st>>>(a);
  IB_CUDA_CHECK(cudaGetLastError());
  return IB_OK;
}

}  // namespace ib
