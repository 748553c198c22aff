// Shared constants and launch declarations of the dense linear-algebra kernels.
#pragma once

#include "bemgpu_internal.h"
#include "quad_math.cuh"

namespace bemgpu {

constexpr int kPanelNB = 32;  // LU panel width (columns factored per getf2 launch)
constexpr int kTrsvNB = 64;   // triangular-solve block (rows per diagonal block)

void launch_getf2(const Launch& L, const MatInst* d, int ninst, int64_t k0, int nb, int prec);
void launch_laswp(const Launch& L, const MatInst* d, int ninst, int64_t k0, int nb, int64_t nmax,
                  int prec);
void launch_trsm_panel(const Launch& L, const MatInst* d, int ninst, int64_t k0, int nb,
                       int64_t nmax, int prec);
void launch_gemm_update(const Launch& L, const MatInst* d, int ninst, int64_t k0, int nb,
                        int64_t nmax, int prec);
void launch_rhs_swap(const Launch& L, const MatInst* d, int ninst, int32_t max_rhs, int reverse,
                     int prec);
void launch_getrs(const Launch& L, const MatInst* d, int ninst, int64_t nmax, int32_t max_rhs,
                  int trans, int prec, int swaps);
void launch_getrf_simt(const Launch& L, const MatInst* d, int ninst, int64_t nmax, int prec);

}  // namespace bemgpu
