// Per-level grid stencils of operators_fluid.F90 (one rank, natural ordering).
#include "kernels.cuh"

namespace ib {

// ------------------------------------------------------------ nonlinear
// operators_fluid.F90:553-587.  omega ghosts come from the ring (bc); fluxes
// outside the physical face grids are zero.  qx, qy are the total fluxes q+q0,
// passed as q and q0 and summed on the fly.
__device__ __forceinline__ void nonlinear_at(const GridDims& g, int t, const double* __restrict__ om,
                                             const double* __restrict__ bc, const double* __restrict__ qx,
                                             const double* __restrict__ q0x, const double* __restrict__ qy,
                                             const double* __restrict__ q0y, double* __restrict__ nlx,
                                             double* __restrict__ nly) {
  auto QX = [&](int i, int j) -> double {  // i=1..m+1, j=0..n+1
    if (j < 1 || j > g.n) return 0.0;
    int idx = (j - 1) * g.nux + (i - 1);
    return qx[idx] + (q0x ? q0x[idx] : 0.0);
  };
  auto QY = [&](int i, int j) -> double {  // i=0..m+1, j=1..n+1
    if (i < 1 || i > g.m) return 0.0;
    int idx = (j - 1) * g.nvx + (i - 1);
    return qy[idx] + (q0y ? q0y[idx] : 0.0);
  };
  if (t < g.nu) {
    int i = t % g.nux + 1, j = t / g.nux + 1;  // u-face (i,j), i=1..m+1, j=1..n
    double v1 = 0.5 * (QY(i, j + 1) + QY(i - 1, j + 1));
    double v0 = 0.5 * (QY(i, j) + QY(i - 1, j));
    double w1 = ghost_vertex(om, bc, g, i, j + 1);
    double w0 = ghost_vertex(om, bc, g, i, j);
    nlx[t] = 0.5 * (v1 * w1 + v0 * w0);
  } else if (t < g.nu + g.nv) {
    int s = t - g.nu;
    int i = s % g.nvx + 1, j = s / g.nvx + 1;  // v-face (i,j), i=1..m, j=1..n+1
    double u1 = 0.5 * (QX(i + 1, j) + QX(i + 1, j - 1));
    double u0 = 0.5 * (QX(i, j) + QX(i, j - 1));
    double w1 = ghost_vertex(om, bc, g, i + 1, j);
    double w0 = ghost_vertex(om, bc, g, i, j);
    nly[s] = -0.5 * (u1 * w1 + u0 * w0);
  }
}

__global__ void k_nonlinear(GridDims g, const double* __restrict__ om, const double* __restrict__ bc,
                            const double* __restrict__ qx, const double* __restrict__ q0x,
                            const double* __restrict__ qy, const double* __restrict__ q0y,
                            double* __restrict__ nlx, double* __restrict__ nly) {
  IB_GRID_DEP_WAIT();
  nonlinear_at(g, blockIdx.x * blockDim.x + threadIdx.x, om, bc, qx, q0x, qy, q0y, nlx, nly);
}

// ------------------------------------------------------------------ rot
// rot_int + rot_bc (operators_fluid.F90:203-233): the transpose of curl.
__device__ __forceinline__ void rot_at(const GridDims& g, int t, const double* __restrict__ hx,
                                       const double* __restrict__ hy, double* __restrict__ vort) {
  if (t >= g.ns) return;
  int I = t % g.nsx + 2, J = t / g.nsx + 2;
  double a = hy[(J - 1) * g.nvx + (I - 1)];
  double b = hy[(J - 1) * g.nvx + (I - 2)];
  double c = hx[(J - 1) * g.nux + (I - 1)];
  double d = hx[(J - 2) * g.nux + (I - 1)];
  vort[t] = a - b - c + d;
}
__global__ void k_rot(GridDims g, const double* __restrict__ hx, const double* __restrict__ hy,
                      double* __restrict__ vort) {
  IB_GRID_DEP_WAIT();
  rot_at(g, blockIdx.x * blockDim.x + threadIdx.x, hx, hy, vort);
}
// nonlinear then rot of every level at once (blockIdx.y = level), on tiles of kNlTx x kNlTy
// vertices: the tile's total face fluxes (q + q0), their averages at the vertices and the
// ghosted vorticity are formed once in shared memory and serve every term that reads them,
// so the FP64 work per vertex falls from 25 to 15 operations; the face fields of the nonlinear
// terms stay in shared memory.  Same averages and products as nonlinear_at and rot_at.
constexpr int kNlTx = 32, kNlTy = 8;
__global__ void __launch_bounds__(kNlTx * kNlTy) k_nonlinear_rot_levels(GridDims g, NlBatch b, int tiles_x) {
  IB_GRID_DEP_WAIT();
  __shared__ double sQy[kNlTy + 2][kNlTx + 1];   // QY(i, j), i = I0-1+c, j = J0-1+r
  __shared__ double sQx[kNlTy + 1][kNlTx + 2];   // QX(i, j), i = I0-1+c, j = J0-1+r
  __shared__ double sW[kNlTy + 2][kNlTx + 2];    // omega with ghosts, i = I0-1+c, j = J0-1+r
  __shared__ double sV[kNlTy + 2][kNlTx];        // v averaged at vertex (i, j), i = I0+c, j = J0-1+r
  __shared__ double sU[kNlTy][kNlTx + 2];        // u averaged at vertex (i, j), i = I0-1+c, j = J0+r
  __shared__ double sNx[kNlTy + 1][kNlTx];       // nlx at u-face (i, j), i = I0+c, j = J0-1+r
  __shared__ double sNy[kNlTy][kNlTx + 1];       // nly at v-face (i, j), i = I0-1+c, j = J0+r
  const int l = blockIdx.y;
  const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
  const int I0 = 2 + tx * kNlTx, J0 = 2 + ty * kNlTy;
  const double* __restrict__ om = b.om[l];
  const double* __restrict__ bc = b.bc[l];
  const double* __restrict__ qx = b.qx[l];
  const double* __restrict__ q0x = b.q0x[l];
  const double* __restrict__ qy = b.qy[l];
  const double* __restrict__ q0y = b.q0y[l];
  const int tid = threadIdx.x, nt = blockDim.x;
  // fluxes outside the physical face grids are zero; entries beyond the vertex grid serve only
  // vertices outside the interior, which write nothing
  for (int q = tid; q < (kNlTy + 2) * (kNlTx + 1); q += nt) {
    const int r = q / (kNlTx + 1), c = q - r * (kNlTx + 1);
    const int i = I0 - 1 + c, j = J0 - 1 + r;
    double v = 0.0;
    if (i >= 1 && i <= g.m && j >= 1 && j <= g.n + 1) {
      const int idx = (j - 1) * g.nvx + (i - 1);
      v = qy[idx] + (q0y ? q0y[idx] : 0.0);
    }
    sQy[r][c] = v;
  }
  for (int q = tid; q < (kNlTy + 1) * (kNlTx + 2); q += nt) {
    const int r = q / (kNlTx + 2), c = q - r * (kNlTx + 2);
    const int i = I0 - 1 + c, j = J0 - 1 + r;
    double v = 0.0;
    if (i >= 1 && i <= g.m + 1 && j >= 1 && j <= g.n) {
      const int idx = (j - 1) * g.nux + (i - 1);
      v = qx[idx] + (q0x ? q0x[idx] : 0.0);
    }
    sQx[r][c] = v;
  }
  for (int q = tid; q < (kNlTy + 2) * (kNlTx + 2); q += nt) {
    const int r = q / (kNlTx + 2), c = q - r * (kNlTx + 2);
    const int i = I0 - 1 + c, j = J0 - 1 + r;
    sW[r][c] = (i >= 1 && i <= g.m + 1 && j >= 1 && j <= g.n + 1) ? ghost_vertex(om, bc, g, i, j) : 0.0;
  }
  __syncthreads();
  for (int q = tid; q < (kNlTy + 2) * kNlTx; q += nt) {
    const int r = q / kNlTx, c = q - r * kNlTx;
    sV[r][c] = 0.5 * (sQy[r][c + 1] + sQy[r][c]);   // 0.5 (QY(i, j) + QY(i-1, j))
  }
  for (int q = tid; q < kNlTy * (kNlTx + 2); q += nt) {
    const int r = q / (kNlTx + 2), c = q - r * (kNlTx + 2);
    sU[r][c] = 0.5 * (sQx[r + 1][c] + sQx[r][c]);   // 0.5 (QX(i, j) + QX(i, j-1))
  }
  __syncthreads();
  for (int q = tid; q < (kNlTy + 1) * kNlTx; q += nt) {
    const int r = q / kNlTx, c = q - r * kNlTx;
    const double v1 = sV[r + 1][c], v0 = sV[r][c], w1 = sW[r + 1][c + 1], w0 = sW[r][c + 1];
    sNx[r][c] = 0.5 * (v1 * w1 + v0 * w0);
  }
  for (int q = tid; q < kNlTy * (kNlTx + 1); q += nt) {
    const int r = q / (kNlTx + 1), c = q - r * (kNlTx + 1);
    const double u1 = sU[r][c + 1], u0 = sU[r][c], w1 = sW[r + 1][c + 1], w0 = sW[r + 1][c];
    sNy[r][c] = -0.5 * (u1 * w1 + u0 * w0);
  }
  __syncthreads();
  const int cx = tid % kNlTx, cy = tid / kNlTx;
  const int I = I0 + cx, J = J0 + cy;
  if (cy < kNlTy && I <= g.m && J <= g.n) {
    const double a = sNy[cy][cx + 1], bb = sNy[cy][cx], c = sNx[cy + 1][cx], d = sNx[cy][cx];
    b.out[l][(size_t)(J - 2) * g.nsx + (I - 2)] = a - bb - c + d;
  }
}

// The same kernel with the interior tiles' rows brought into shared memory by bulk copies
// (cp.async.bulk, completing on an mbarrier), the measured alternative to the plain loads
// above (op_time_pass kinds 4 and 5).  The fields keep the reference's layout, whose row pitches
// (799, 800 and 801 doubles) are not all multiples of 16 bytes, so no tiled tensor map can
// describe them.  Each row is copied from the even element at or before its first one, a
// 16-byte boundary of the 256-byte-aligned fields, over an even number of elements, and read
// from its offset in shared memory.  Tiles on the domain's edges, and any row whose rounded copy
// would pass the end of its field, take the plain loads.  The wait on the mbarrier is bounded:
// past the limit the CTA records IB_ERR_CUDA in err, waits (bounded again) for its copies, and
// writes nothing.
constexpr int kNlPitch = 40;   // doubles a staged row holds (a tile row plus the alignment slack)
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__global__ void __launch_bounds__(kNlTx * kNlTy) k_nonlinear_rot_levels_bulk(GridDims g, NlBatch b, int tiles_x,
                                                                            int* err) {
  IB_GRID_DEP_WAIT();
  __shared__ double sQy[kNlTy + 2][kNlTx + 1];
  __shared__ double sQx[kNlTy + 1][kNlTx + 2];
  __shared__ double sW[kNlTy + 2][kNlTx + 2];
  __shared__ double sV[kNlTy + 2][kNlTx];
  __shared__ double sU[kNlTy][kNlTx + 2];
  __shared__ double sNx[kNlTy + 1][kNlTx];
  __shared__ double sNy[kNlTy][kNlTx + 1];
  // staged rows: qy, q0y (kNlTy + 2 rows), qx, q0x (kNlTy + 1), omega (kNlTy + 2)
  constexpr int kRows = 2 * (kNlTy + 2) + 2 * (kNlTy + 1) + (kNlTy + 2);
  __shared__ __align__(16) double raw[kRows][kNlPitch];
  __shared__ int s_off[kRows];
  __shared__ __align__(8) unsigned long long mbar;
  const int l = blockIdx.y;
  const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
  const int I0 = 2 + tx * kNlTx, J0 = 2 + ty * kNlTy;
  const double* __restrict__ om = b.om[l];
  const double* __restrict__ bc = b.bc[l];
  const double* __restrict__ qx = b.qx[l];
  const double* __restrict__ q0x = b.q0x[l];
  const double* __restrict__ qy = b.qy[l];
  const double* __restrict__ q0y = b.q0y[l];
  const int tid = threadIdx.x, nt = blockDim.x;
  // staged row k: its field, first element, length and the field's size
  auto row_of = [&](int k, const double** src, long long* e0, int* len, long long* total) {
    if (k < 2 * (kNlTy + 2)) {            // qy / q0y rows j = J0-1+r, faces i = I0-1 .. I0+kNlTx-1
      const int r = k % (kNlTy + 2);
      *src = k < kNlTy + 2 ? qy : q0y;
      *e0 = (long long)(J0 - 1 + r - 1) * g.nvx + (I0 - 1 - 1);
      *len = kNlTx + 1;
      *total = g.nv;
      return;
    }
    k -= 2 * (kNlTy + 2);
    if (k < 2 * (kNlTy + 1)) {            // qx / q0x rows j = J0-1+r, faces i = I0-1 .. I0+kNlTx
      const int r = k % (kNlTy + 1);
      *src = k < kNlTy + 1 ? qx : q0x;
      *e0 = (long long)(J0 - 1 + r - 1) * g.nux + (I0 - 1 - 1);
      *len = kNlTx + 2;
      *total = g.nu;
      return;
    }
    k -= 2 * (kNlTy + 1);                  // omega rows J = J0-1+r, vertices I = I0-1 .. I0+kNlTx
    *src = om;
    *e0 = (long long)(J0 - 1 + k - 2) * g.nsx + (I0 - 1 - 2);
    *len = kNlTx + 2;
    *total = g.ns;
  };
  // an interior tile: every face and vertex it reads lies inside its field, omega's away from
  // the ring; and every rounded row copy ends inside its field
  bool bulk = q0x && q0y && tx >= 1 && ty >= 1 && I0 + kNlTx <= g.m && J0 + kNlTy <= g.n;
  if (bulk)
    for (int k = 0; k < kRows; ++k) {
      const double* src;
      long long e0, total;
      int len;
      row_of(k, &src, &e0, &len, &total);
      const long long a = e0 & ~1LL;
      const long long n = ((e0 + len - a) + 1) & ~1LL;
      if (e0 < 0 || a + n > total || n > kNlPitch || ((unsigned long long)src & 15ull) != 0) bulk = false;
    }
  if (bulk) {
    if (tid == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar)), "r"(1) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid < 32) {
      if (tid == 0) {
        unsigned total_bytes = 0;
        for (int k = 0; k < kRows; ++k) {
          const double* src;
          long long e0, total;
          int len;
          row_of(k, &src, &e0, &len, &total);
          const long long a = e0 & ~1LL;
          total_bytes += (unsigned)(8 * (((e0 + len - a) + 1) & ~1LL));
        }
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&mbar)),
                     "r"(total_bytes) : "memory");
      }
      __syncwarp();
      for (int k = tid; k < kRows; k += 32) {
        const double* src;
        long long e0, total;
        int len;
        row_of(k, &src, &e0, &len, &total);
        const long long a = e0 & ~1LL;
        const unsigned bytes = (unsigned)(8 * (((e0 + len - a) + 1) & ~1LL));
        s_off[k] = (int)(e0 - a);
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(&raw[k][0])),
                     "l"(src + a), "r"(bytes), "r"(smem_u32(&mbar))
                     : "memory");
      }
    }
    auto wait_bounded = [&]() -> unsigned {
      unsigned done = 0;
      for (int it = 0; it < (1 << 22) && !done; ++it)
        asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                     : "=r"(done)
                     : "r"(smem_u32(&mbar)), "r"(0)
                     : "memory");
      return done;
    };
    const unsigned done = wait_bounded();
    // every thread takes the same branch: the copies landed, or the CTA records the failure,
    // waits once more for them and stops (the barrier also orders s_off)
    if (__syncthreads_or(!done)) {
      if (tid == 0) atomicExch(err, IB_ERR_CUDA);
      if (!done) wait_bounded();
      return;
    }
    for (int q = tid; q < (kNlTy + 2) * (kNlTx + 1); q += nt) {
      const int r = q / (kNlTx + 1), c = q - r * (kNlTx + 1);
      sQy[r][c] = raw[r][c + s_off[r]] + raw[kNlTy + 2 + r][c + s_off[kNlTy + 2 + r]];
    }
    const int bx = 2 * (kNlTy + 2), bw = bx + 2 * (kNlTy + 1);
    for (int q = tid; q < (kNlTy + 1) * (kNlTx + 2); q += nt) {
      const int r = q / (kNlTx + 2), c = q - r * (kNlTx + 2);
      sQx[r][c] = raw[bx + r][c + s_off[bx + r]] + raw[bx + kNlTy + 1 + r][c + s_off[bx + kNlTy + 1 + r]];
    }
    for (int q = tid; q < (kNlTy + 2) * (kNlTx + 2); q += nt) {
      const int r = q / (kNlTx + 2), c = q - r * (kNlTx + 2);
      sW[r][c] = raw[bw + r][c + s_off[bw + r]];
    }
  } else {
    for (int q = tid; q < (kNlTy + 2) * (kNlTx + 1); q += nt) {
      const int r = q / (kNlTx + 1), c = q - r * (kNlTx + 1);
      const int i = I0 - 1 + c, j = J0 - 1 + r;
      double v = 0.0;
      if (i >= 1 && i <= g.m && j >= 1 && j <= g.n + 1) {
        const int idx = (j - 1) * g.nvx + (i - 1);
        v = qy[idx] + (q0y ? q0y[idx] : 0.0);
      }
      sQy[r][c] = v;
    }
    for (int q = tid; q < (kNlTy + 1) * (kNlTx + 2); q += nt) {
      const int r = q / (kNlTx + 2), c = q - r * (kNlTx + 2);
      const int i = I0 - 1 + c, j = J0 - 1 + r;
      double v = 0.0;
      if (i >= 1 && i <= g.m + 1 && j >= 1 && j <= g.n) {
        const int idx = (j - 1) * g.nux + (i - 1);
        v = qx[idx] + (q0x ? q0x[idx] : 0.0);
      }
      sQx[r][c] = v;
    }
    for (int q = tid; q < (kNlTy + 2) * (kNlTx + 2); q += nt) {
      const int r = q / (kNlTx + 2), c = q - r * (kNlTx + 2);
      const int i = I0 - 1 + c, j = J0 - 1 + r;
      sW[r][c] = (i >= 1 && i <= g.m + 1 && j >= 1 && j <= g.n + 1) ? ghost_vertex(om, bc, g, i, j) : 0.0;
    }
  }
  __syncthreads();
  for (int q = tid; q < (kNlTy + 2) * kNlTx; q += nt) {
    const int r = q / kNlTx, c = q - r * kNlTx;
    sV[r][c] = 0.5 * (sQy[r][c + 1] + sQy[r][c]);
  }
  for (int q = tid; q < kNlTy * (kNlTx + 2); q += nt) {
    const int r = q / (kNlTx + 2), c = q - r * (kNlTx + 2);
    sU[r][c] = 0.5 * (sQx[r + 1][c] + sQx[r][c]);
  }
  __syncthreads();
  for (int q = tid; q < (kNlTy + 1) * kNlTx; q += nt) {
    const int r = q / kNlTx, c = q - r * kNlTx;
    const double v1 = sV[r + 1][c], v0 = sV[r][c], w1 = sW[r + 1][c + 1], w0 = sW[r][c + 1];
    sNx[r][c] = 0.5 * (v1 * w1 + v0 * w0);
  }
  for (int q = tid; q < kNlTy * (kNlTx + 1); q += nt) {
    const int r = q / (kNlTx + 1), c = q - r * (kNlTx + 1);
    const double u1 = sU[r][c + 1], u0 = sU[r][c], w1 = sW[r + 1][c + 1], w0 = sW[r + 1][c];
    sNy[r][c] = -0.5 * (u1 * w1 + u0 * w0);
  }
  __syncthreads();
  const int cx = tid % kNlTx, cy = tid / kNlTx;
  const int I = I0 + cx, J = J0 + cy;
  if (cy < kNlTy && I <= g.m && J <= g.n) {
    const double a = sNy[cy][cx + 1], bb = sNy[cy][cx], c = sNx[cy + 1][cx], d = sNx[cy][cx];
    b.out[l][(size_t)(J - 2) * g.nsx + (I - 2)] = a - bb - c + d;
  }
}

// ----------------------------------------------------------------- curl
// curl_int + curl_bc (operators_fluid.F90:423-471), s ghosts from the ring.
__global__ void k_curl(GridDims g, const double* __restrict__ s, const double* __restrict__ sbc,
                       double* __restrict__ qx, double* __restrict__ qy) {
  IB_GRID_DEP_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < g.nu) {
    int i = t % g.nux + 1, j = t / g.nux + 1;
    qx[t] = ghost_vertex(s, sbc, g, i, j + 1) - ghost_vertex(s, sbc, g, i, j);
  } else if (t < g.nu + g.nv) {
    int u = t - g.nu;
    int i = u % g.nvx + 1, j = u / g.nvx + 1;
    qy[u] = ghost_vertex(s, sbc, g, i, j) - ghost_vertex(s, sbc, g, i + 1, j);
  }
}

// The same for every level at once (blockIdx.y = level).
__global__ void k_curl_levels(GridDims g, CurlBatch cb) {
  IB_GRID_DEP_WAIT();
  const int l = blockIdx.y;
  const double* __restrict__ s = cb.s[l];
  const double* __restrict__ sbc = cb.sbc[l];
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < g.nu) {
    int i = t % g.nux + 1, j = t / g.nux + 1;
    cb.qx[l][t] = ghost_vertex(s, sbc, g, i, j + 1) - ghost_vertex(s, sbc, g, i, j);
  } else if (t < g.nu + g.nv) {
    int u = t - g.nu;
    int i = u % g.nvx + 1, j = u / g.nvx + 1;
    cb.qy[l][u] = ghost_vertex(s, sbc, g, i, j) - ghost_vertex(s, sbc, g, i + 1, j);
  }
}

// ------------------------------------------------------------- coarsify
// operators_fluid.F90:381-419 with grid.F90:1061-1087: the full-weighting sum
// at odd fine points I=3..m-1, J=3..n-1 overwrites coarse point
// ((I-1)/2+m/4+1, (J-1)/2+n/4+1).
__global__ void k_coarsify(GridDims g, const double* __restrict__ fine, double* __restrict__ coarse) {
  IB_GRID_DEP_WAIT();
  int cx = g.m / 2 - 1, cy = g.n / 2 - 1;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cx * cy) return;
  int a = t % cx, b = t / cx;
  int I = 2 * a + 3, J = 2 * b + 3;
  auto F = [&](int ii, int jj) { return fine[(jj - 2) * g.nsx + (ii - 2)]; };
  double v = F(I, J) + 0.5 * (F(I + 1, J) + F(I, J + 1) + F(I - 1, J) + F(I, J - 1)) +
             0.25 * (F(I + 1, J + 1) + F(I + 1, J - 1) + F(I - 1, J - 1) + F(I - 1, J + 1));
  int Ic = (I - 1) / 2 + g.m / 4 + 1, Jc = (J - 1) / 2 + g.n / 4 + 1;
  coarse[(Jc - 2) * g.nsx + (Ic - 2)] = v;
}

// --------------------------------------------------------------- frame fluxes
// q0 = q0p + q0r of every level for a frame moving at (u, v) and turning at w about (cx, cy)
// (motion_potential + motion_rotation, variables.F90:299-360): on level k (1-based, spacing
// delta 2^(k-1)) the u-face (i, j) takes -fac u + fac (0 + w (y_j - cy)) and the v-face
// -fac v + fac (0 - w (x_i - cx)), fac = delta 2^(k-1), x_i and y_j the face centres less the
// offsets.  A u-face's value depends on its row only and a v-face's on its column only, so
// k_frame_lines forms the n + m values of each level and k_frame_fill writes the fields.  Every
// operation is rounded on its own in the order written, as the context's creation forms the
// same fluxes on the host (built without contraction), so a frame equal to the configured
// motion gives the same fluxes bit for bit.
__global__ void k_frame_lines(GridDims g, int nlev, double delta, double offx, double offy, double u, double v,
                              double w, double cx, double cy, double* __restrict__ lines) {
  IB_GRID_DEP_WAIT();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int per = g.n + g.m;
  if (t >= nlev * per) return;
  const int k = t / per, r = t - k * per;
  const double pw = ldexp(1.0, k);   // 2^(level - 1), exact
  const double fac = __dmul_rn(delta, pw);
  if (r < g.n) {   // u-face row j = r + 1
    double yy = __dsub_rn(__dsub_rn((double)(r + 1), 0.5), (double)(g.n / 2));
    yy = __dmul_rn(__dmul_rn(yy, delta), pw);
    yy = __dsub_rn(__dadd_rn(yy, __dmul_rn((double)(g.n / 2), delta)), offy);
    const double e = __dadd_rn(0.0, __dmul_rn(w, __dsub_rn(yy, cy)));
    lines[t] = __dadd_rn(__dmul_rn(-fac, u), __dmul_rn(fac, e));
  } else {         // v-face column i = r - n + 1
    double xx = __dsub_rn(__dsub_rn((double)(r - g.n + 1), 0.5), (double)(g.m / 2));
    xx = __dmul_rn(__dmul_rn(xx, delta), pw);
    xx = __dsub_rn(__dadd_rn(xx, __dmul_rn((double)(g.m / 2), delta)), offx);
    const double e = __dsub_rn(0.0, __dmul_rn(w, __dsub_rn(xx, cx)));
    lines[t] = __dadd_rn(__dmul_rn(-fac, v), __dmul_rn(fac, e));
  }
}

// blockIdx.y = level, blockIdx.z = u-faces (0) or v-faces (1)
__global__ void k_frame_fill(GridDims g, FrameLevels fl, const double* __restrict__ lines) {
  IB_GRID_DEP_WAIT();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  const double* ln = lines + (size_t)k * (g.n + g.m);
  if (blockIdx.z == 0) {
    if (t < g.nu) fl.q0x[k][t] = ln[t / g.nux];
  } else {
    if (t < g.nv) fl.q0y[k][t] = ln[g.n + t % g.nvx];
  }
}

// --------------------------------------------------------------- get_bc
// operators_fluid.F90:475-535 with grid.F90:1091-1140: coarse values on the
// fine boundary; coincident points copied, midpoints averaged; times fac.
__global__ void k_get_bc(GridDims g, const double* __restrict__ s, double fac, double* __restrict__ ring) {
  IB_GRID_DEP_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.nbc) return;
  ring[t] = ring_value(s, g, t) * fac;
}

// The same for every level at once (blockIdx.y = level): ring l from field src[l], or zero
// where src[l] is null.
__global__ void k_get_bc_levels(GridDims g, RingBatch rb, double fac) {
  IB_GRID_DEP_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int l = blockIdx.y;
  if (t >= g.nbc) return;
  const double* s = rb.src[l];
  rb.dst[l][t] = s ? ring_value(s, g, t) * fac : 0.0;
}

// ------------------------------------------------------------- apply_bc
// operators_fluid.F90:539-549 in place: left, right, bottom, top.
__global__ void k_apply_bc(GridDims g, double* __restrict__ v, const double* __restrict__ ring, double fac) {
  IB_GRID_DEP_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.ns) return;
  int I = t % g.nsx + 2, J = t / g.nsx + 2;
  if (I != 2 && I != g.m && J != 2 && J != g.n) return;
  double x = v[t];
  if (I == 2) x = x + fac * ring[g.left + J - 1];
  if (I == g.m) x = x + fac * ring[g.right + J - 1];
  if (J == 2) x = x + fac * ring[g.bottom + I - 1];
  if (J == g.n) x = x + fac * ring[g.top + I - 1];
  v[t] = x;
}

// rhsbc = 0; apply_bc(rhsbc, a, f); apply_bc(rhsbc, b, f)   (timestepper.F90:184-189)
__global__ void k_rhsbc(GridDims g, double* __restrict__ v, const double* __restrict__ ra,
                        const double* __restrict__ rb, double fac) {
  IB_GRID_DEP_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.ns) return;
  int I = t % g.nsx + 2, J = t / g.nsx + 2;
  double x = 0.0;
  if (I == 2 || I == g.m || J == 2 || J == g.n) {
    const double* rr[2] = {ra, rb};
    for (int q = 0; q < 2; ++q) {
      const double* r = rr[q];
      if (!r) continue;
      if (I == 2) x = x + fac * r[g.left + J - 1];
      if (I == g.m) x = x + fac * r[g.right + J - 1];
      if (J == 2) x = x + fac * r[g.bottom + I - 1];
      if (J == g.n) x = x + fac * r[g.top + I - 1];
    }
  }
  v[t] = x;
}

// -------------------------------------------------------- vector helpers
__global__ void k_axpby(int n, double a, const double* __restrict__ x, double b, const double* __restrict__ y,
                        double* __restrict__ z) {
  IB_GRID_DEP_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) z[t] = a * x[t] + b * y[t];
}
__global__ void k_sub(int n, const double* __restrict__ x, const double* __restrict__ y, double* __restrict__ z) {
  IB_GRID_DEP_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) z[t] = x[t] - y[t];
}
// z = z - d x, the product rounded before the difference (compute_rhs_prescribed's
// rhsf(i) - delta*u_B, user.F90:137-174)
__global__ void k_sub_scaled(int n, double d, const double* __restrict__ x, double* __restrict__ z) {
  IB_GRID_DEP_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) z[t] = __dsub_rn(z[t], __dmul_rn(d, x[t]));
}
__global__ void k_fill(int n, double v, double* __restrict__ z) {
  IB_GRID_DEP_WAIT();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) z[t] = v;
}

// ------------------------------------------------------------ launchers
static inline int blocks(long long n, int nt = 256) { return (int)((n + nt - 1) / nt); }

int launch_nonlinear(const GridDims& g, const double* om, const double* bc, const double* qx, const double* q0x,
                     const double* qy, const double* q0y, double* nlx, double* nly, cudaStream_t st) {
  count_launch();
  k_nonlinear<<<blocks(g.nu + g.nv), 256, 0, st>>>(g, om, bc, qx, q0x, qy, q0y, nlx, nly);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}
int launch_nonlinear_rot_levels(const GridDims& g, const NlBatch& b, int nlev, cudaStream_t st) {
  if (nlev < 1 || nlev > kMaxLevels) return IB_ERR_ARG;
  const int tiles_x = cdiv(g.nsx, kNlTx), tiles_y = cdiv(g.nsy, kNlTy);
  count_launch();
  k_nonlinear_rot_levels<<<dim3(tiles_x * tiles_y, nlev), kNlTx * kNlTy, 0, st>>>(g, b, tiles_x);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}
int launch_nonlinear_rot_levels_bulk(const GridDims& g, const NlBatch& b, int nlev, int* err, cudaStream_t st) {
  if (nlev < 1 || nlev > kMaxLevels) return IB_ERR_ARG;
  const int tiles_x = cdiv(g.nsx, kNlTx), tiles_y = cdiv(g.nsy, kNlTy);
  count_launch();
  k_nonlinear_rot_levels_bulk<<<dim3(tiles_x * tiles_y, nlev), kNlTx * kNlTy, 0, st>>>(g, b, tiles_x, err);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}
int launch_rot(const GridDims& g, const double* hx, const double* hy, double* vort, cudaStream_t st) {
  count_launch();
  k_rot<<<blocks(g.ns), 256, 0, st>>>(g, hx, hy, vort);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}
int launch_curl(const GridDims& g, const double* s, const double* sbc, double* qx, double* qy, cudaStream_t st) {
  count_launch();
  k_curl<<<blocks(g.nu + g.nv), 256, 0, st>>>(g, s, sbc, qx, qy);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}
int launch_curl_levels(const GridDims& g, const CurlBatch& cb, int nlev, cudaStream_t st) {
  if (nlev < 1 || nlev > kMaxLevels) return IB_ERR_ARG;
  count_launch();
  k_curl_levels<<<dim3(blocks(g.nu + g.nv), nlev), 256, 0, st>>>(g, cb);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}
int launch_coarsify(const GridDims& g, const double* fine, double* coarse, cudaStream_t st) {
  int n = (g.m / 2 - 1) * (g.n / 2 - 1);
  count_launch();
  k_coarsify<<<blocks(n), 256, 0, st>>>(g, fine, coarse);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}
int launch_frame_flux(const GridDims& g, const FrameLevels& fl, int nlev, double delta, double offx, double offy,
                      double u, double v, double w, double cx, double cy, double* lines, cudaStream_t st) {
  if (nlev < 1 || nlev > kMaxLevels) return IB_ERR_ARG;
  count_launches(2);
  k_frame_lines<<<blocks(nlev * (g.n + g.m)), 256, 0, st>>>(g, nlev, delta, offx, offy, u, v, w, cx, cy, lines);
  k_frame_fill<<<dim3(blocks(g.nu > g.nv ? g.nu : g.nv), nlev, 2), 256, 0, st>>>(g, fl, lines);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}
int launch_get_bc(const GridDims& g, const double* s, double fac, double* ring, cudaStream_t st) {
  count_launch();
  k_get_bc<<<blocks(g.nbc), 256, 0, st>>>(g, s, fac, ring);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}
int launch_get_bc_levels(const GridDims& g, const RingBatch& rb, int nlev, double fac, cudaStream_t st) {
  if (nlev < 1 || nlev > kMaxLevels) return IB_ERR_ARG;
  count_launch();
  k_get_bc_levels<<<dim3(blocks(g.nbc), nlev), 256, 0, st>>>(g, rb, fac);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}
int launch_apply_bc(const GridDims& g, double* v, const double* ring, double fac, cudaStream_t st) {
  count_launch();
  k_apply_bc<<<blocks(g.ns), 256, 0, st>>>(g, v, ring, fac);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}
int launch_rhsbc(const GridDims& g, double* v, const double* ra, const double* rb, double fac, cudaStream_t st) {
  count_launch();
  k_rhsbc<<<blocks(g.ns), 256, 0, st>>>(g, v, ra, rb, fac);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}
int launch_axpby(int n, double a, const double* x, double b, const double* y, double* z, cudaStream_t st) {
  count_launch();
  k_axpby<<<blocks(n), 256, 0, st>>>(n, a, x, b, y, z);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}
int launch_sub(int n, const double* x, const double* y, double* z, cudaStream_t st) {
  count_launch();
  k_sub<<<blocks(n), 256, 0, st>>>(n, x, y, z);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}
int launch_sub_scaled(int n, double d, const double* x, double* z, cudaStream_t st) {
  if (n <= 0) return IB_OK;
  count_launch();
  k_sub_scaled<<<blocks(n), 256, 0, st>>>(n, d, x, z);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}
int launch_fill(int n, double v, double* z, cudaStream_t st) {
  if (n <= 0) return IB_OK;
  count_launch();
  k_fill<<<blocks(n), 256, 0, st>>>(n, v, z);
  return cudaGetLastError() == cudaSuccess ? IB_OK : IB_ERR_CUDA;
}

}  // namespace ib
