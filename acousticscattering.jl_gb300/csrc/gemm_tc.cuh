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
  // Tensor map (device address, 64-byte aligned) of C viewed as FP32 pairs, used by
  // the reduction epilogue (launch_tc_cgemm with red = true; c_r0 must be even): -A B
  // is added into C by asynchronous bulk tensor reductions instead of reading C.
  const void* cmap;
};

constexpr size_t kTcMapBytes = 128;  // sizeof(CUtensorMap)

size_t tc_pack_bytes(int64_t rows, int kk);
// Encodes into map (kTcMapBytes, host memory) the tensor map of a column-major complex64
// matrix c with `rows` x `cols` addressable entries and leading dimension ldc, as used
// by the reduction epilogue.  False when the layout does not allow it (odd ldc,
// misaligned base) or the driver entry point is unavailable.
bool tc_encode_cmap(void* map, const void* c, int64_t ldc, int64_t rows, int64_t cols);

#ifdef __CUDACC__
void launch_tc_pack(const Launch& L, const TcPackInst* d, int ninst, int64_t max_rows, int max_kk);
// red: every instance carries cmap (reduction epilogue); otherwise C is read and written
void launch_tc_cgemm(const Launch& L, const TcGemmInst* d, int ninst, int64_t total_tiles,
                     bool red = false);
#endif

}  // namespace bemgpu
