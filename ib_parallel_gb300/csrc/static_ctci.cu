// A Poisson solve (ctci, myfft.F90:177-188) that allocates no device memory.
//
// Some callers cannot allocate device memory at the moment they need the solve: a host
// program that reserves its whole device-memory budget once at start-up (for instance
// because another solver shares the GPU and owns the rest of HBM), a time loop that must
// not pay cudaFree's implicit device-wide synchronisation, or a caller that holds no
// IbCtx (a context allocates every field of the nested grid; this solve needs only its
// two arrays).  ib_ctci_static serves them: its scratch field and its tables live in one
// file-scope device array of kStaticDoubles doubles (16 MiB) that every GPU loading this
// library holds until the process exits, and the caller passes the input and output.
//
// Set-up: the first call on a device, and the first call after the grid size changes,
// looks up the array's device address, fills the tables with host-to-device copies and waits
// for the device to finish them (cudaDeviceSynchronize); make that call before any stream
// capture.  Later calls with the same grid only
// launch three kernels on the caller's stream and return without waiting for them.
//
// Every call on a device shares the one array, which keeps what the last call left there.
// Each call overwrites the scratch field before reading it, so nothing has to start at
// zero; but calls whose kernels overlap on the GPU (two streams, or two host threads
// without ordering) race on the scratch field and give wrong results.
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ib_gpu.h"
#include "dst.cuh"
#include "tri.cuh"

namespace ib {

static constexpr size_t kStaticDoubles = size_t(1) << 21;  // 16 MiB

static __device__ __align__(256) double g_ctci_scratch[kStaticDoubles];

namespace {

struct StaticSolve {
  double* base = nullptr;  // device address of g_ctci_scratch on this device
  int m = 0, n = 0;        // grid the tables were filled for
  DstPlan px;
  TriOp tri;
};

std::mutex g_mu;
StaticSolve g_dev[64];

size_t align4(size_t n) { return (n + 3) & ~size_t(3); }

}  // namespace

void set_last_error(const char* msg);  // capi.cu: the message ib_last_error() returns

// Doubles of g_ctci_scratch the solve needs for an m x n grid (0 if the grid is unsupported).
static size_t needed(int m, int n) {
  size_t plan = dst_plan_table_doubles(m - 1);
  if (plan == 0) return 0;
  int s = 0, C = 0;
  tri_chunking(n, m - 1, &s, &C);
  return align4((size_t)(m - 1) * (n - 1)) + align4(plan) + align4(tri_table_doubles(m - 1, s, C));
}

int static_ctci(int m, int n, const double* vort, double* s, cudaStream_t st) {
  if (m < 8 || n < 8 || m % 4 || n % 4 || !vort || !s) {
    set_last_error("ib_ctci_static: m, n must be >= 8 and divisible by 4, arrays non-null");
    return IB_ERR_ARG;
  }
  size_t need = needed(m, n);
  if (need == 0) {
    set_last_error("ib_ctci_static: m must be 2^a 3^b 5^c");
    return IB_ERR_ARG;
  }
  if (need > kStaticDoubles) {
    set_last_error("ib_ctci_static: grid too large for the 16 MiB static scratch ((m-1)(n-1) plus tables must "
                   "fit in 2^21 doubles)");
    return IB_ERR_ARG;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    set_last_error("ib_ctci_static: no current CUDA device");
    return IB_ERR_CUDA;
  }
  for (const void* ptr : {static_cast<const void*>(vort), static_cast<const void*>(s)}) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess ||
        (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)) {
      cudaGetLastError();
      set_last_error("ib_ctci_static: vort and s must be device (or managed) memory");
      return IB_ERR_ARG;
    }
    // the kernels run on the current device: memory of another GPU would be a peer access
    if (at.type == cudaMemoryTypeDevice && at.device != dev) {
      set_last_error("ib_ctci_static: vort and s must be memory of the current device");
      return IB_ERR_ARG;
    }
  }
  GridDims g;
  g.init(m, n);
  StaticSolve* S = &g_dev[dev];
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!S->base) {
      // the symbol's device address on the current device (the host-side name is not one)
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_ctci_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        set_last_error("ib_ctci_static: cudaGetSymbolAddress failed");
        return IB_ERR_CUDA;
      }
      S->base = static_cast<double*>(p);
    }
    if (S->m != m || S->n != n) {
      // tables after the scratch field: DST plan of the x transform, then the tridiagonal
      // factors of (lam_x(k) + T_y)^-1 / (2m) (the same operator the context path uses).
      // The recorded grid is cleared first: if an upload below fails, no later call may take
      // the half-rewritten tables for the old grid's.
      S->m = 0; S->n = 0;
      double* plan_mem = S->base + align4((size_t)g.ns);
      int rc = dst_plan_init_external(&S->px, g.nsx, plan_mem, st);
      if (rc != IB_OK) { set_last_error("ib_ctci_static: table upload failed"); return rc; }
      double* tri_mem = plan_mem + align4(dst_plan_table_doubles(g.nsx));
      std::vector<double> lamx(g.nsx);
      const double pi = 4.0 * std::atan(1.0);
      for (int k = 1; k <= g.nsx; ++k) {
        double sn = std::sin(pi * (double)k / (2.0 * m));
        lamx[k - 1] = 4.0 * sn * sn;
      }
      rc = tri_build(&S->tri, g.nsx, g.nsy, lamx.data(), 1.0 / (2.0 * m), tri_mem);
      if (rc != IB_OK) { set_last_error("ib_ctci_static: table upload failed"); return rc; }
      // tri_build copies from pageable host memory, and such a copy may return before its DMA
      // has reached the device; the solve kernels run on the caller's stream, which nothing
      // orders after that copy.  Wait for it here (set-up runs outside any stream capture).
      if (cudaDeviceSynchronize() != cudaSuccess) {
        set_last_error("ib_ctci_static: table upload failed");
        return IB_ERR_CUDA;
      }
      S->m = m; S->n = n;
    }
  }
  // x transform into the static scratch, per-mode tridiagonal solve, inverse transform.
  // The scratch is fully overwritten by the first pass, so nothing needs clearing.
  double* spec = S->base;
  DstLaunch L;
  L.B = 2; L.NT = 160;
  DstXArgs a;
  a.in = vort; a.out = spec;
  int rc = dst_pass_x(S->px, g.nsy, g.nsx, PRE_COPY, a, g, L, st);
  TriLaunch T;
  T.Mb = 8;
  if (rc == IB_OK) rc = tri_solve(S->tri, spec, spec, g.nsx, T, st);
  DstXArgs b;
  b.in = spec; b.out = s;
  if (rc == IB_OK) rc = dst_pass_x(S->px, g.nsy, g.nsx, PRE_COPY, b, g, L, st);
  if (rc != IB_OK) set_last_error("ib_ctci_static: kernel launch failed");
  return rc;
}

}  // namespace ib

extern "C" int ib_ctci_static(int m, int n, const double* vort, double* s, void* stream) {
  return ib::static_ctci(m, n, vort, s, static_cast<cudaStream_t>(stream));
}

