// Per-mode tridiagonal solves that replace the y-direction DST pairs of the
// spectral solves in myfft.F90 (ctci, ainv) and operators_fluid.F90
// (fluid_predictor).
//
// With S_y the DST-I along y (S_y S_y = 2n I) and T_y = tridiag(-1, 2, -1) the
// 1-D Dirichlet Laplacian, S_y diag(f(lam_y)) S_y = 2n f(T_y).  So each 2-D
// spectral solve
//     S_x S_y [ g(lam_x + lam_y) (.) S_y S_x v ]
// is an x transform, one tridiagonal solve per x mode k, and an x transform:
//     ctci:  (1/2m) (lam_x(k) + T_y)^-1
//     ainv:  (1/(2m c1)) (1/c1 + lam_x(k) + T_y)^-1
//     predictor (level k): (2n/c) (1/c + lam_x(k) + T_y)^-1 applied to
//            S_x[ con1 rhs + con2 rhs_old + rhsbc + (omega - c L omega)/normalize ]
// where c = dt/(2 Delta_k^2 Re) and L the 5-point Laplacian with zero boundary.
//
// Every system is tridiag(-1, a_k, -1) of size n-1.  For parallelism it is cut
// into C chunks of s = n/C - 1 rows separated by C-1 interface rows: each chunk is
// solved with zero ends (Thomas with tabulated pivots), the interface values then
// satisfy a constant-coefficient tridiagonal system of size C-1 (solved with its
// tabulated inverse), and each chunk adds the interface responses (tabulated).
// 5 FP64 operations per point.
#pragma once
#include "ib_common.cuh"

namespace ib {

struct TriOp {
  int nx = 0, ny = 0;     // modes (m-1), rows (n-1)
  int s = 0, C = 0;       // chunk rows, chunks: (s+1)*C = ny+1
  double sigma = 1.0;     // right-hand-side scale
  double* inv = nullptr;  // s x nx: 1/pivot
  double* sinv = nullptr; // s x nx: sigma/pivot
  double* gL = nullptr;   // s x nx: chunk response to a unit left end value
  double* rinv = nullptr; // (C-1)^2 x nx: inverse of the interface system, row-major per mode
};

struct TriLaunch {
  int Mb = 8;             // modes per CTA
};

// Chunking for ny = n-1 rows (n divisible by 4) and nx modes: C*(s+1) = n.
void tri_chunking(int n, int nx, int* s, int* C);
// Tables for shifts a_k = 2 + shift_k (k = 0..nx-1), uploaded into caller-provided
// device memory of tri_table_doubles() doubles.
size_t tri_table_doubles(int nx, int s, int C);
int tri_build(TriOp* op, int nx, int ny, const double* shift, double sigma, double* dev_mem);
// Boundary terms a solve adds to its right-hand side as it loads it (a finer level of the
// coarse-to-fine recursions, dst_ring_edge_from_modes): row r of mode k is
//     post_scale (F[r][k] + add2[r][k]) + sk2[k] sd[(k & 1) ny + r]
//     (+ edge[k] on row 0, + edge[nx + k] on row ny-1).
// sd == nullptr: post_scale (F + add2) only; add2 == nullptr: F alone (add2 has F's pitch).
struct TriBc {
  const double* sk2 = nullptr;
  const double* sd = nullptr;
  const double* edge = nullptr;
  const double* add2 = nullptr;
  double post_scale = 1.0;
};

// In place (F may equal U): U = sigma * A^-1 (F with the boundary terms bc) for every mode column.
int tri_solve(const TriOp& op, const double* F, double* U, int ld, const TriLaunch& L, cudaStream_t st,
              const TriBc& bc = TriBc());
size_t tri_smem(const TriOp& op, int Mb);

// Up to kTriBatch independent solves in one launch (levels of a recursion with their own
// tables, or columns of a precomputed response), each with the arithmetic of tri_solve's
// register-resident kernel.  The items must share nx, ny and the chunking.
constexpr int kTriBatch = 16;
struct TriBatch {
  int n = 0;
  TriOp op[kTriBatch];
  const double* F[kTriBatch] = {};
  double* U[kTriBatch] = {};
  TriBc bc[kTriBatch];
};
bool tri_batch_supported(const TriOp& op);
int tri_solve_batch(const TriBatch& b, int ld, const TriLaunch& L, cudaStream_t st);

}  // namespace ib
