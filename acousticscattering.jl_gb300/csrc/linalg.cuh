// Shared constants and launch declarations of the dense linear-algebra kernels.
#pragma once

#include "bemgpu_internal.h"
#include "quad_math.cuh"

namespace bemgpu {

constexpr int kPanelNB = 32;  // LU panel width (columns factored per getf2 launch)
constexpr int kTrsvNB = 64;   // triangular-solve block (rows per diagonal block)

void launch_getf2(const Launch& L, const MatInst* d, int ninst, int64_t k0, int nb, int prec);
// row interchanges k0 .. k0 + nb - 1 on columns [c_lo, c_hi) \ [s_lo, s_hi)
void launch_laswp(const Launch& L, const MatInst* d, int ninst, int64_t k0, int nb, int64_t c_lo,
                  int64_t c_hi, int64_t s_lo, int64_t s_hi, int prec);
// U12 = L11^{-1} A12 on columns [c_lo, c_hi); nb <= 32 or <= 128
void launch_trsm_panel(const Launch& L, const MatInst* d, int ninst, int64_t k0, int nb,
                       int64_t c_lo, int64_t c_hi, int prec);
// rows [k0 + nb, n) x columns [c_lo, c_hi) -= L21 U12 (SIMT)
void launch_gemm_update(const Launch& L, const MatInst* d, int ninst, int64_t k0, int nb,
                        int64_t nmax, int64_t c_lo, int64_t c_hi, int prec);
void launch_rhs_swap(const Launch& L, const MatInst* d, int ninst, int32_t max_rhs, int reverse,
                     int prec);
void launch_getrs(const Launch& L, const MatInst* d, int ninst, int64_t nmax, int32_t max_rhs,
                  int trans, int prec, int swaps);
void launch_getrf_simt(const Launch& L, const MatInst* d, int ninst, int64_t nmax, int prec);

}  // namespace bemgpu
