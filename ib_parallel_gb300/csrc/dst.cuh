// Batched DST-I (FFTW RODFT00 semantics) for the spectral Poisson and
// Crank-Nicolson solves of myfft.F90:161-216.
//
// Y_k = 2 sum_{j=1}^{N} x_j sin(pi j k / M),  k = 1..N,  M = N+1 (unnormalised).
//
// One line of length N is transformed through a complex FFT of length P = M/2:
//   y_j = sin(j pi/M)(x_j + x_{M-j}) + (x_j - x_{M-j})/2,     y_0 = 0
//   Z   = FFT_P(y_0 + i y_1, y_2 + i y_3, ...)
//   2Y  = unpacked real FFT of y (length M)
//   D_{2k}   = -Im(2Y_k),      D_1 = Re(Y_0),   D_{2k+1} = D_{2k-1} + Re(2Y_k)
// (the classic odd-extension sine transform; the odd outputs are a prefix sum).
// The complex FFT is a Stockham auto-sort with radices 2, 3, 4 and 5 run in
// shared memory over all (line, butterfly) items of a CTA.
#pragma once
#include "ib_common.cuh"

namespace ib {

constexpr int kMaxRadices = 16;

struct DstPlan {
  int N = 0, M = 0, P = 0;
  int nrad = 0;
  int rad[kMaxRadices] = {0};
  double2* tw = nullptr;   // P entries: exp(-2 pi i t / P)
  double2* uw = nullptr;   // P/2 entries: exp(-2 pi i k / M)
  double* sn = nullptr;    // P+1 entries: sin(j pi / M)
};

// Launch geometry of one pass (chosen by the tuner in dst.cu).
struct DstLaunch {
  int B = 1;       // lines per CTA
  int NT = 128;    // threads per CTA
};

int dst_plan_create(DstPlan* p, int N);   // N = M-1, M divisible by 4, M = 2^a 3^b 5^c
void dst_plan_destroy(DstPlan* p);

enum DstPre { PRE_COPY = 0, PRE_COMBINE = 1, PRE_APPLYBC = 2 };
enum DstYMode { YMODE_NONE = 0, YMODE_DIAG = 1, YMODE_PRED = 2 };

struct DstXArgs {
  const double* in = nullptr;    // nlines rows, row pitch ld
  const double* in2 = nullptr;   // PRE_COMBINE second operand
  const double* in3 = nullptr;   // PRE_COMBINE third operand
  double ca = 1.0, cb = 0.0;     // PRE_COMBINE: ca*in + cb*in2 + in3
  const double* ring = nullptr;  // PRE_APPLYBC boundary ring
  double fac = 1.0;              // PRE_APPLYBC factor
  double* out = nullptr;         // nlines rows, pitch ld
};

struct DstYArgs {
  double* a = nullptr;           // spectral buffer (in/out), rows of pitch ld
  const double* b = nullptr;     // YMODE_PRED second input
  const double* t1 = nullptr;    // DIAG table, or PRED lam1i
  const double* t2 = nullptr;    // PRED lam1
};

// x direction: lines are the (n-1) rows of an (n-1)x(m-1) field, N = m-1.
int dst_pass_x(const DstPlan& px, int nrows, int ld, DstPre pre, const DstXArgs& a,
               const GridDims& g, const DstLaunch& L, cudaStream_t st);
// y direction: lines are the (m-1) columns, N = n-1, optional spectral combine.
int dst_pass_y(const DstPlan& py, int ncols, int ld, DstYMode mode, const DstYArgs& a,
               const DstLaunch& L, cudaStream_t st);

size_t dst_smem_x(const DstPlan& p, int B);
size_t dst_smem_y(const DstPlan& p, int B, DstYMode mode);

}  // namespace ib
