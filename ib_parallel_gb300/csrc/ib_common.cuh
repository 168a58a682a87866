// Common definitions for the GB300 immersed-boundary time step.
//
// Layouts follow the reference (nirmaljp6/IB_Parallel, one rank, natural
// PETSc ordering, x fastest):
//   vertex field (omega, s, rhs):  (n-1) rows x (m-1) cols, element (I,J) of the
//       Fortran grid (I=2..m, J=2..n) at [(J-2)*(m-1) + (I-2)]   (grid.F90:186-203)
//   u-face flux qx:  n rows x (m+1) cols, face (i,j) at [(j-1)*(m+1) + (i-1)]
//   v-face flux qy:  (n+1) rows x m cols, face (i,j) at [(j-1)*m + (i-1)]
//   boundary ring (nbc = 2(m+1)+2(n+1)): left[0..n], right[0..n], bottom[0..m],
//       top[0..m]                                               (grid.F90:224-228)
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <map>
#include <mutex>
#include <utility>

#define IB_OK 0
#define IB_ERR_ARG 1
#define IB_ERR_CUDA 2
#define IB_ERR_NOMEM 3
#define IB_ERR_GMRES 4
#define IB_ERR_FSI 5
#define IB_ERR_NONFINITE 6
#define IB_ERR_DOMAIN 7
#define IB_ERR_STATE 8

namespace ib {

struct GridDims {
  int m, n;          // cells in x and y of one level
  int nsx, nsy;      // vertex interior: m-1, n-1
  int ns;            // (m-1)(n-1)
  int nux, nuy;      // u-faces: m+1, n
  int nu;
  int nvx, nvy;      // v-faces: m, n+1
  int nv;
  int nbc;           // ring length
  int left, right, bottom, top;
  __host__ __device__ void init(int m_, int n_) {
    m = m_; n = n_;
    nsx = m - 1; nsy = n - 1; ns = nsx * nsy;
    nux = m + 1; nuy = n; nu = nux * nuy;
    nvx = m; nvy = n + 1; nv = nvx * nvy;
    nbc = 2 * (m + 1) + 2 * (n + 1);
    left = 0; right = n + 1; bottom = 2 * (n + 1); top = 2 * (n + 1) + m + 1;
  }
};

// Ghosted vertex value at grid point (I,J), I=1..m+1, J=1..n+1: interior from the
// field, edges from the ring with the precedence left, right, bottom, top
// (later writes win at corners), as operators_fluid.F90:448-451 and 563-566 do.
__device__ __forceinline__ double ghost_vertex(const double* __restrict__ f,
                                               const double* __restrict__ ring,
                                               const GridDims& g, int I, int J) {
  if (J == 1) return ring[g.bottom + I - 1];
  if (J == g.n + 1) return ring[g.top + I - 1];
  if (I == 1) return ring[g.left + J - 1];
  if (I == g.m + 1) return ring[g.right + J - 1];
  return f[(J - 2) * g.nsx + (I - 2)];
}

// get_bc (operators_fluid.F90:475-535 with grid.F90:1091-1140) at ring index t: the value of
// the next coarser level's field s on this level's boundary; coincident points copied,
// midpoints averaged.
__device__ __forceinline__ double ring_value(const double* __restrict__ s, const GridDims& g, int t) {
  auto S = [&](int I, int J) { return s[(J - 2) * g.nsx + (I - 2)]; };
  if (t >= g.bottom) {  // bottom / top edges: p = 0..m
    bool top = t >= g.top;
    int p = t - (top ? g.top : g.bottom);
    int J = top ? 3 * g.n / 4 + 1 : g.n / 4 + 1;
    int I = g.m / 4 + 1 + p / 2;
    return (p & 1) ? 0.5 * (S(I, J) + S(I + 1, J)) : S(I, J);
  }
  bool right = t >= g.right;   // left / right edges: p = 0..n
  int p = t - (right ? g.right : g.left);
  int I = right ? 3 * g.m / 4 + 1 : g.m / 4 + 1;
  int J = g.n / 4 + 1 + p / 2;
  return (p & 1) ? 0.5 * (S(I, J) + S(I, J + 1)) : S(I, J);
}

inline int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

// Division of a non-negative int by a runtime divisor d >= 1 with a multiply-high and a
// shift (Granlund-Montgomery): q = (umulhi(n, mul) + n) >> shr, exact for n < 2^31.
struct FastDiv {
  unsigned mul = 0, shr = 0;
  int d = 1;
  __host__ __device__ FastDiv() {}
  __host__ FastDiv(int dd) : d(dd) {
    unsigned l = 0;
    while ((1u << l) < (unsigned)dd) ++l;
    unsigned long long m = (((1ull << 32) * ((1ull << l) - (unsigned long long)dd)) / (unsigned long long)dd) + 1ull;
    mul = (unsigned)m;
    shr = l;
  }
  __device__ __forceinline__ int div(int n) const { return (int)((__umulhi((unsigned)n, mul) + (unsigned)n) >> shr); }
  __device__ __forceinline__ int mod(int n) const { return n - div(n) * d; }
};

// Programmatic dependent launch: in the captured step graphs the edges between kernels are
// programmatic (make_edges_programmatic), so a kernel's CTAs may be scheduled while its
// predecessor finishes.  Every kernel of this library therefore waits here, first thing, for
// its predecessor's completion and memory; launched without such an edge it returns at once.
#define IB_GRID_DEP_WAIT() asm volatile("griddepcontrol.wait;" ::: "memory")

// Number of kernels this library has launched (all contexts), for the benchmark's
// launch count.  Defined in solver.cu.
void count_launch();
void count_launches(long long n);
long long launch_count();

}  // namespace ib

#define IB_CUDA_CHECK(expr)                                                     \
  do {                                                                          \
    cudaError_t _e = (expr);                                                    \
    if (_e != cudaSuccess) {                                                    \
      fprintf(stderr, "ib_gpu CUDA error %s at %s:%d\n", cudaGetErrorString(_e), \
              __FILE__, __LINE__);                                              \
      return IB_ERR_CUDA;                                                       \
    }                                                                           \
  } while (0)

namespace ib {

// Lets kernel `kern` take `bytes` of dynamic shared memory.  The limit is an attribute of the
// function, shared by every context in the process, and captured graphs launch with the sizes
// they were captured with: so it is only ever raised, once, to the most the device allows (the
// opt-in maximum less the kernel's static shared memory), never set to one context's size.
template <typename K>
inline cudaError_t allow_dyn_smem(K kern, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, int> raised;   // (device, kernel) -> limit set
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const auto key = std::make_pair(dev, reinterpret_cast<const void*>(kern));
  std::lock_guard<std::mutex> lock(mu);
  auto it = raised.find(key);
  if (it != raised.end()) return (size_t)it->second >= bytes ? cudaSuccess : cudaErrorInvalidValue;
  int optin = 0;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, kern);
  if (e != cudaSuccess) return e;
  const int lim = optin - (int)fa.sharedSizeBytes;
  if (lim < 0 || (size_t)lim < bytes) return cudaErrorInvalidValue;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  if (e == cudaSuccess) raised[key] = lim;
  return e;
}

}  // namespace ib
