// Descriptors and launch declarations of the matrix-vector kernels in refine.cu.
#pragma once

#include "bemgpu_internal.h"

namespace bemgpu {

constexpr int kChunks = 8;   // column chunks of the row-wise sweeps
constexpr int kGemvR = 4;    // right-hand sides per gemv pass
constexpr int kStats = 9;    // residual statistics per right-hand side

struct VecInst {
  const void* A;     // complex128 matrix, column-major
  int64_t n;         // order
  int64_t lda;
  double* rows;      // row scales (n), or null for unit scales
  double* cols;      // column scales (n), or null
  double* rowsum;    // row sums of |A| (n)
  double* cols_inv;  // 1 / cols (n), filled by the scaled-copy launch
  float* rows_inv;   // 1 / rows (n), filled by the row-statistics launch
  double* part;      // scratch: kChunks * nrhs * n * 3 doubles (>= kChunks * n * 2)
  void* out;         // scaled copy / correction work buffer (ld n)
  int32_t out_single;
  int32_t nrhs;
  int32_t* flag;     // nonfinite conversion flag
  const double* x;   // complex128 vectors (n x nrhs, ld ldx)
  int64_t ldx;
  const double* b;   // complex128 right-hand sides
  int64_t ldb;
  double* y;         // complex128 output / input vectors
  int64_t ldy;
  double* den;       // componentwise denominators (n x nrhs, ld ldy)
  double* stats;     // kStats doubles per right-hand side
  int32_t* active;   // per rhs: still refining (null = all)
  int32_t* changed;  // per rhs: last correction changed x
  // Compact system storage (mixed precision with FP32 regular pairs): A is complex64,
  // exact for every regular pair, and the near pairs carry an FP64 correction
  // dnear = a64 - (complex128)(complex64)a64, so A64 = A + the sparse corrections.
  int32_t a32;
  int32_t nbc;               // block columns of the near pattern: 1 (n x n) or 2 (2n x 2n)
  int64_t n_mesh, n_near;
  const int32_t* near_ptr;   // CSR row pointers over the mesh's near pairs (n_mesh + 1)
  const int32_t* near_i;
  const int32_t* near_j;
  const double* dnear;       // corrections, complex128 [block][n_near], block = nbc br + bc
  float4* xs;                // x split as FP32 (hi.re, hi.im, lo.re, lo.im), n x nrhs
  float* xa;                 // |x| in FP32, n x nrhs
  float* cols_inv32;         // 1 / cols in FP32 (n)
  double norm_floor;         // equilibration: lower bound of the row and column scales
};

#ifdef __CUDACC__
void launch_equilibrate(const Launch& L, const VecInst* d, int ninst, int64_t nmax);
void launch_scale_copy(const Launch& L, const VecInst* d, int ninst, int64_t nmax);
// mode 0: y = A x; mode 1: y = b - A x and den = |b| + |A||x|.  rows: rows per thread of
// the compact-storage product (1 or 2; results identical)
void launch_gemv(const Launch& L, const VecInst* d, int ninst, int64_t nmax, int32_t max_rhs,
                 int mode, int rows = 2);
// compact instances: out (complex128, ld n) += the near corrections, each scaled by
// 1 / (rows_i cols_j) (unit_scales = 0) or unscaled (unit_scales = 1)
void launch_near_add(const Launch& L, const VecInst* d, int ninst, int64_t max_near,
                     int unit_scales);
// compact instances: out (complex128, ld n) = complex128(A)
void launch_expand_a32(const Launch& L, const VecInst* d, int ninst, int64_t nmax);
void launch_resid_stats(const Launch& L, const VecInst* d, int ninst, int32_t max_rhs);
void launch_corr_prep(const Launch& L, const VecInst* d, int ninst, int64_t nmax,
                      int32_t max_rhs);
void launch_corr_apply(const Launch& L, const VecInst* d, int ninst, int64_t nmax,
                       int32_t max_rhs, int mode);
#endif

}  // namespace bemgpu
