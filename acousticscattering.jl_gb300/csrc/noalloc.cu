// Allocation-free entry point: the tensor-core complex64 update C -= A B with its
// scratch (the packed bf16 operand images, the launch descriptors and the timeout word)
// in one file-scope device array instead of memory from cudaMalloc.
//
// Some callers of this library cannot allocate device memory at the point where they
// need the update: hosts whose free HBM is already owned by their own pool allocator
// (a Julia or Python array pool that forbids further cudaMalloc), and real-time or
// safety-constrained codes that may not allocate after start-up.  They pass device
// inputs and outputs; everything else lives in g_noalloc_scratch.
//
// Limits: m, n <= kNoAllocMaxMN, k <= kNoAllocMaxK.  The array (4 MiB + 2 KiB) is part of
// the library image: every GPU that loads the library holds it until the process exits.
// All calls share it and it keeps the last call's contents; the timeout word is cleared
// at the start of every call, the operand images are rewritten in full.  Calls whose
// work overlaps on the GPU (concurrent streams, other host threads) race on the array.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

#include "bemgpu_internal.h"
#include "gemm_tc.cuh"

namespace bemgpu {
namespace {

constexpr int64_t kNoAllocMaxMN = 2048;
constexpr int kNoAllocMaxK = 128;
constexpr size_t kHeaderBytes = 2048;  // timeout word + descriptors
// packed images of one operand at the maximum size: 16 tiles x 4 chunks x 32 KB
constexpr size_t kPackMax = (size_t)(kNoAllocMaxMN / 128) * (kNoAllocMaxK / 32) * 2 * 16384;
constexpr size_t kScratchBytes = kHeaderBytes + 2 * kPackMax;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct Layout {
  int* err;
  TcPackInst* pack;   // 2 entries
  TcGemmInst* gemm;   // 1 entry
  unsigned char* apack;
  unsigned char* bpack;
};

Layout layout(void* base) {
  unsigned char* b = static_cast<unsigned char*>(base);
  Layout L;
  L.err = reinterpret_cast<int*>(b);
  L.pack = reinterpret_cast<TcPackInst*>(b + 256);
  L.gemm = reinterpret_cast<TcGemmInst*>(b + 256 + 2 * sizeof(TcPackInst) + 64);
  L.apack = b + kHeaderBytes;
  L.bpack = b + kHeaderBytes + kPackMax;
  return L;
}

// Writes the launch descriptors into the scratch header and clears the timeout word.
__global__ void k_noalloc_setup(int* err, TcPackInst* pack, TcGemmInst* gemm, const void* A,
                                int64_t lda, const void* B, int64_t ldb, void* C, int64_t ldc,
                                int64_t m, int64_t n, int32_t k, void* apack, void* bpack) {
  *err = 0;
  TcPackInst pa;
  memset(&pa, 0, sizeof pa);
  pa.a = A;
  pa.lda = lda;
  pa.rows = m;
  pa.kk = k;
  pa.trans = 0;
  pa.out = apack;
  pa.active = 1;
  TcPackInst pb = pa;
  pb.a = B;
  pb.lda = ldb;
  pb.rows = n;
  pb.trans = 1;
  pb.out = bpack;
  pack[0] = pa;
  pack[1] = pb;
  TcGemmInst g;
  memset(&g, 0, sizeof g);
  g.apack = apack;
  g.bpack = bpack;
  g.c = C;
  g.ldc = ldc;
  g.m = m;
  g.n = n;
  g.kk = k;
  g.active = 1;
  gemm[0] = g;
}

int set_error(int code, const std::string& msg) {
  bemgpu_set_process_error(msg.c_str());
  return code;
}

}  // namespace
}  // namespace bemgpu

using namespace bemgpu;

extern "C" int bemgpu_cgemm_update_noalloc(void* stream, int64_t m, int64_t n, int32_t k,
                                           const void* A, int64_t lda, const void* B,
                                           int64_t ldb, void* C, int64_t ldc) {
  if (m < 1 || n < 1 || k < 1)
    return set_error(BEMGPU_EINVAL, "m, n and k must be positive");
  if (m > kNoAllocMaxMN || n > kNoAllocMaxMN || k > kNoAllocMaxK) {
    char buf[160];
    std::snprintf(buf, sizeof buf,
                  "size beyond the allocation-free maximum (m, n <= %lld, k <= %d)",
                  (long long)kNoAllocMaxMN, kNoAllocMaxK);
    return set_error(BEMGPU_EINVAL, buf);
  }
  if (!A || !B || !C) return set_error(BEMGPU_EINVAL, "null device pointer");
  if (lda < m || ldb < k || ldc < m)
    return set_error(BEMGPU_EINVAL, "leading dimension smaller than the matrix");
  if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B) |
       reinterpret_cast<uintptr_t>(C)) & 7u)
    return set_error(BEMGPU_EINVAL, "complex64 operands must be 8-byte aligned");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(BEMGPU_ENODEV, "no current CUDA device");
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (s) {
    // the stream must belong to the current device: the array's address below is the
    // current device's
    int sdev = -1;
    e = cudaStreamGetDevice(s, &sdev);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_error(BEMGPU_EINVAL, std::string("cudaStreamGetDevice: ") +
                                          cudaGetErrorString(e));
    }
    if (sdev != dev)
      return set_error(BEMGPU_EINVAL, "stream belongs to another device than the current one");
  }
  // The device address of the array on the current device, looked up on every call (a
  // cheap query) so that it stays right after a cudaDeviceReset.  The first call on a
  // device may load the module there, so make it before any stream capture.
  void* base = nullptr;
  e = cudaGetSymbolAddress(&base, g_noalloc_scratch);
  if (e != cudaSuccess || !base) {
    cudaGetLastError();
    return set_error(BEMGPU_ECUDA, std::string("cudaGetSymbolAddress: ") +
                                       cudaGetErrorString(e));
  }
  const Layout Lo = layout(base);
  k_noalloc_setup<<<1, 1, 0, s>>>(Lo.err, Lo.pack, Lo.gemm, A, lda, B, ldb, C, ldc, m, n, k,
                                  Lo.apack, Lo.bpack);
  count_launch(1);
  const Launch L{s, Lo.err};
  launch_tc_pack(L, Lo.pack, 2, m > n ? m : n, k);
  launch_tc_cgemm(L, Lo.gemm, 1, ((m + 127) / 128) * ((n + 127) / 128));
  e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(BEMGPU_ECUDA, cudaGetErrorString(e));
  // the timeout word, read on the caller's stream (no device-wide synchronisation)
  int h = 0;
  e = cudaMemcpyAsync(&h, Lo.err, sizeof h, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return set_error(BEMGPU_ECUDA, cudaGetErrorString(e));
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(BEMGPU_ECUDA, cudaGetErrorString(e));
  if (h != 0) return set_error(BEMGPU_ETIMEOUT, "a bounded device wait gave up");
  return BEMGPU_OK;
}
