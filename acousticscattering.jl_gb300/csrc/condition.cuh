// Singular values of small dense complex128 matrices (condition-number diagnostics).
#pragma once

#include "bemgpu_internal.h"

namespace bemgpu {

struct SvdInst {
  double2* a;          // n x n column-major working copy (overwritten by the rotations)
  int64_t n, lda;
  const double* rows;  // k_svd_scale: row and column scales (null: no scaling)
  const double* cols;
  int32_t* rotated;    // set when a round rotated a pair (cleared by the host per sweep)
  double* sigma;       // n singular values (unordered)
};

#ifdef __CUDACC__
void launch_svd_scale(const Launch& L, const SvdInst* d, int ninst, int64_t nmax);
void launch_jacobi_round(const Launch& L, const SvdInst* d, int ninst, int64_t nmax, int64_t r,
                         double tol);
void launch_column_norms(const Launch& L, const SvdInst* d, int ninst, int64_t nmax);
#endif

}  // namespace bemgpu
