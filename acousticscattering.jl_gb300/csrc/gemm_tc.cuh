// Descriptors and launch declarations of the tensor-core complex update (gemm_tc.cu).
#pragma once

#include "bemgpu_internal.h"

namespace bemgpu {

constexpr int kTcMaxInst = 256;  // instances per batched launch

// One operand panel to pack into swizzled bf16 hi/lo blocks.
struct TcPackInst {
  const void* a;   // complex64 column-major matrix
  int64_t lda;
  int64_t r0;      // first operand row (trans = 0: matrix row; 1: matrix column)
  int64_t k0;      // first K index (trans = 0: matrix column; 1: matrix row)
  int64_t rows;    // operand rows (M or N extent)
  int32_t kk;      // K extent
  int32_t trans;   // 0: element (r, k) at r + k lda (L21); 1: at k + r lda (U12)
  void* out;       // packed blocks, tc_pack_bytes(rows, kk)
  int32_t active;
  int32_t pad;
};

// One C -= A B update: C block rows [c_r0, c_r0 + m), columns [c_c0, c_c0 + n).
struct TcGemmInst {
  const void* apack;  // packed A (m rows)
  const void* bpack;  // packed B (n rows)
  void* c;            // complex64 column-major
  int64_t ldc;
  int64_t c_r0, c_c0;
  int64_t m, n;
  int32_t kk;
  int32_t active;
};

size_t tc_pack_bytes(int64_t rows, int kk);

#ifdef __CUDACC__
void launch_tc_pack(const Launch& L, const TcPackInst* d, int ninst, int64_t max_rows, int max_kk);
void launch_tc_cgemm(const Launch& L, const TcGemmInst* d, int ninst, int64_t total_tiles);
#endif

}  // namespace bemgpu
