// Shared constants and launch declarations of the dense linear-algebra kernels.
#pragma once

#include "bemgpu_internal.h"
#include "quad_math.cuh"

namespace bemgpu {

constexpr int kPanelNB = 32;  // LU panel width (columns factored per getf2 launch)
constexpr int kTrsvNB = 64;   // triangular-solve block (rows per diagonal block)

// cs: CTAs per instance of the complex64 panel kernel (2, 4 or 8; 0 = the batch-size
// rule); the factor is identical for every choice
void launch_getf2(const Launch& L, const MatInst* d, int ninst, int64_t k0, int nb, int prec,
                  int cs = 0);
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
// Solve with the LU factor in place on MatInst.x (trans 1: A^H x = b; swaps 0 leaves
// out the row interchanges).  With work != null the flag-synchronised block solve is
// two-level blocked solve is used (needs MatInst.y and, for swaps, MatInst.perm).
void launch_getrs(const Launch& L, const MatInst* d, int ninst, int64_t nmax, int32_t max_rhs,
                  int trans, int prec, int swaps, const TrsvWork* work = nullptr);
// out[i] (kLinvB x kLinvB complex64, column-major) = -(L11^{-1} - I) of the unit lower
// block at (k0, k0) of instance i (complex64 factors).
void launch_linv_neg(const Launch& L, const MatInst* d, int ninst, int64_t k0, float2* const* outs);
// Row permutation of each factor from its pivots (one CTA per instance).
void launch_make_perm(const Launch& L, const MatInst* d, int ninst, int64_t nmax);

void launch_getrf_simt(const Launch& L, const MatInst* d, int ninst, int64_t nmax, int prec);

}  // namespace bemgpu
