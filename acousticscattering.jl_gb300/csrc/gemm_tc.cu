// Tensor-core complex trailing update of the complex64 LU: C -= A B on sm_103a.
//
// Precision: every complex64 operand x is split into two bfloat16 numbers,
// hi = bf16(x) and lo = bf16(x - hi), and each real product is formed from three
// bfloat16 products (hi*hi + lo*hi + hi*lo) accumulated in FP32 in tensor memory.  The
// complex product uses the four real products (4M):
//   Cr += Ar Br - Ai Bi,   Ci += Ar Bi + Ai Br
// so one K-chunk issues 12 products x 2 K-steps = 24 tcgen05.mma instructions, the
// negative terms through the negate-A bit of the instruction descriptor.
//
// Layout: a pack kernel writes the operand panels as ready-to-copy shared-memory
// images: for every 128-row tile and 32-wide K-chunk, one 16 KB block per real /
// imaginary part whose 128-byte rows hold the 32 hi values then the 32 lo values of
// one M (or N) index, in the 128-byte swizzled order the UMMA shared-memory
// descriptors read.  The GEMM kernel then moves each block with a single bulk
// asynchronous copy (TMA engine) - no tensor map, no coordinate arithmetic.
//
// Kernel: persistent, one CTA per SM, 10 warps, warp-specialised:
//   warp 0      producer: 4 bulk copies (64 KB) per stage, 3-stage ring;
//   warp 1      TMEM allocation (512 columns) and the single-thread MMA issuer;
//   warps 2..9  epilogue: tcgen05.ld of the FP32 accumulators (thread = tile row).
//               With a tensor map of C, -acc is staged in shared memory 16 columns at
//               a time (two 16 KB buffers) and added into C by bulk tensor reductions
//               (cp.reduce.async.bulk.tensor .add.f32, performed at L2), so the SMs
//               never wait on C; without one, C is read, updated and written back.
// Two accumulator buffers (Cr | Ci, 128 + 128 columns each) let the epilogue of one
// tile overlap the MMAs of the next.  Every mbarrier wait is bounded: a timeout
// records BEMGPU_ETIMEOUT, stops all roles, drains the copies in flight and frees TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <cstdio>

#include "bemgpu_internal.h"
#include "gemm_tc.cuh"
#include "tma.cuh"

namespace bemgpu {

constexpr int kTcM = 128;          // tile rows (M)
constexpr int kTcN = 128;          // tile columns (N), complex
constexpr int kTcKC = 32;          // complex K per chunk / stage
constexpr int kTcStages = 3;
constexpr int kTcBlock = 16384;    // bytes of one packed 128 x (32 hi + 32 lo) bf16 block
constexpr int kTcStageBytes = 4 * kTcBlock;  // Ar, Ai, Br, Bi
constexpr int kTcThreads = 320;   // producer, MMA, 8 epilogue warps
constexpr int kTcEpiThreads = 256;
constexpr uint32_t kTmemCols = 512;
constexpr int kTcRedCols = 16;                      // columns per reduction chunk
constexpr int kTcRedBytes = kTcRedCols * kTcM * 8;  // 16 KB staging buffer
constexpr int kTcNamedBar = 1;                      // epilogue-only barrier id

// ------------------------------------------------------------------ descriptors
// UMMA shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row
// groups 1024 bytes apart (SBO), descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);          // start address
  d |= (uint64_t)1 << 16;                          // LBO (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;                // SBO
  d |= (uint64_t)1 << 46;                          // version
  d |= (uint64_t)2 << 61;                          // SWIZZLE_128B
  return d;
}

// Instruction descriptor, kind::f16: FP32 accumulate, BF16 A and B, both K-major,
// N = 128, M = 128; negate_a flips the sign of the A operand.
__host__ __device__ constexpr uint32_t idesc_bf16(bool negate_a) {
  return (1u << 4)              // D format F32
         | (1u << 7)            // A format BF16
         | (1u << 10)           // B format BF16
         | ((negate_a ? 1u : 0u) << 13)
         | ((uint32_t)(kTcN >> 3) << 17)
         | ((uint32_t)(kTcM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// 32 lanes x 16 consecutive 32-bit TMEM columns
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ------------------------------------------------------------------ packing
// Byte offset of (row, element e in 0..63) inside a swizzled 128 x 64 bf16 block.
__device__ __forceinline__ uint32_t swz_offset(int row, int e) {
  const int r8 = row & 7, atom = row >> 3, chunk = e >> 3, within = e & 7;
  return (uint32_t)(atom * 1024 + r8 * 128 + ((chunk ^ r8) << 4) + within * 2);
}

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16* hi, __nv_bfloat16* lo) {
  *hi = __float2bfloat16_rn(x);
  *lo = __float2bfloat16_rn(x - __bfloat162float(*hi));
}

__device__ __forceinline__ uint32_t pack2(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&v);
}

// Packs rows [r0, r0 + rows) x K-columns [k0, k0 + kk) of a column-major complex64
// matrix (element (r, k) at r + k * lda) as "row-operand" blocks: block
// (tile, chunk, part) holds 128 rows of 32 complex K values.  trans = 1 reads
// element (r, k) at k + r * lda instead (the B operand, whose rows are columns of U12).
// One work item = one row and 8 consecutive K values: it writes the four swizzled
// 16-byte chunks (re hi, re lo, im hi, im lo) with vector stores.
__global__ void __launch_bounds__(256) k_tc_pack(const TcPackInst* __restrict__ insts) {
  const TcPackInst& P = insts[blockIdx.z];
  const int64_t tiles = (P.rows + kTcM - 1) / kTcM;
  const int chunks = (P.kk + kTcKC - 1) / kTcKC;
  const int64_t tile = blockIdx.x;
  const int ch = blockIdx.y;
  if (!P.active || tile >= tiles || ch >= chunks) return;
  const float2* A = reinterpret_cast<const float2*>(P.a);
  uint8_t* out = reinterpret_cast<uint8_t*>(P.out) + ((size_t)tile * chunks + ch) * 2 * kTcBlock;
  for (int item = threadIdx.x; item < kTcM * 4; item += blockDim.x) {
    int r, q;
    if (P.trans) {  // 4 consecutive threads cover one row's 32 contiguous values
      q = item & 3;
      r = item >> 2;
    } else {        // consecutive threads on consecutive rows (contiguous per column)
      r = item % kTcM;
      q = item / kTcM;
    }
    const int64_t gr = (int64_t)tile * kTcM + r;
    float re[8], im[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int gk = ch * kTcKC + q * 8 + e;
      float2 v = make_float2(0.f, 0.f);
      if (gr < P.rows && gk < P.kk) {
        const int64_t off = P.trans ? (P.k0 + gk) + (P.r0 + gr) * P.lda
                                    : (P.r0 + gr) + (P.k0 + gk) * P.lda;
        v = A[off];
      }
      re[e] = v.x;
      im[e] = v.y;
    }
    uint32_t rh[4], rl[4], ih[4], il[4];
#pragma unroll
    for (int e = 0; e < 8; e += 2) {
      __nv_bfloat16 h0, l0, h1, l1;
      split_bf16(re[e], &h0, &l0);
      split_bf16(re[e + 1], &h1, &l1);
      rh[e / 2] = pack2(__bfloat162float(h0), __bfloat162float(h1));
      rl[e / 2] = pack2(__bfloat162float(l0), __bfloat162float(l1));
      split_bf16(im[e], &h0, &l0);
      split_bf16(im[e + 1], &h1, &l1);
      ih[e / 2] = pack2(__bfloat162float(h0), __bfloat162float(h1));
      il[e / 2] = pack2(__bfloat162float(l0), __bfloat162float(l1));
    }
    const uint32_t ohi = swz_offset(r, q * 8), olo = swz_offset(r, 32 + q * 8);
    *reinterpret_cast<uint4*>(out + ohi) = make_uint4(rh[0], rh[1], rh[2], rh[3]);
    *reinterpret_cast<uint4*>(out + olo) = make_uint4(rl[0], rl[1], rl[2], rl[3]);
    *reinterpret_cast<uint4*>(out + kTcBlock + ohi) = make_uint4(ih[0], ih[1], ih[2], ih[3]);
    *reinterpret_cast<uint4*>(out + kTcBlock + olo) = make_uint4(il[0], il[1], il[2], il[3]);
  }
}

// ------------------------------------------------------------------ the GEMM
struct TcShared {
  uint64_t full[kTcStages];
  uint64_t empty[kTcStages];
  uint64_t tfull[2];
  uint64_t tempty[2];
  uint32_t tmem_base;
  int abort_flag;
  int ninst;
  int epi_go;
  int32_t prefix[kTcMaxInst + 1];
};

__device__ __forceinline__ void epi_bar() {
  asm volatile("bar.sync %0, %1;" ::"n"(kTcNamedBar), "n"(kTcEpiThreads) : "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void red_add_tile(const void* map, int32_t x, int32_t y, uint32_t src) {
  asm volatile(
      "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2}], "
      "[%3];" ::"l"(map),
      "r"(x), "r"(y), "r"(src)
      : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_read1() {
  asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}
// 32 lanes x 8 consecutive 32-bit TMEM columns
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity, int* err,
                                        volatile int* abort_flag) {
  for (uint32_t it = 0; it < kSpinLimit; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 1023) == 1023 && *abort_flag) return false;
  }
  if (err) atomicExch(err, kErrTimeout);
  *abort_flag = 1;
  return false;
}

// tile t of the batch -> (instance, mt, nt); prefix[] holds cumulative tile counts
__device__ __forceinline__ void tile_coords(const TcShared& S, const TcGemmInst* insts,
                                            int64_t t, int* inst, int64_t* mt, int64_t* nt) {
  // largest instance i with prefix[i] <= t (empty instances are skipped over)
  int lo = 0, hi = S.ninst - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (S.prefix[mid] <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  const int64_t local = t - (int64_t)S.prefix[lo];
  const int64_t mtiles = (insts[lo].m + kTcM - 1) / kTcM;
  *inst = lo;
  *mt = local % mtiles;
  *nt = local / mtiles;
}

__global__ void __launch_bounds__(kTcThreads, 1)
    k_tc_cgemm(const TcGemmInst* __restrict__ insts, int ninst, int* err, int red) {
  extern __shared__ uint8_t smem_raw[];
  // 1024-byte aligned stage buffers (swizzle atoms), barriers after them
  uint8_t* base = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* red_smem = base + kTcStages * kTcStageBytes;  // 2 reduction staging buffers
  TcShared& S = *reinterpret_cast<TcShared*>(red_smem + 2 * kTcRedBytes);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kTcStages; ++s) {
      mbar_init(&S.full[s], 1);
      mbar_init(&S.empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&S.tfull[b], 1);
      mbar_init(&S.tempty[b], kTcEpiThreads);
    }
    S.abort_flag = 0;
    S.ninst = ninst;
    int32_t acc = 0;
    S.prefix[0] = 0;
    for (int i = 0; i < ninst; ++i) {
      const TcGemmInst& G = insts[i];
      const int64_t t = (G.active && G.m > 0 && G.n > 0 && G.kk > 0)
                            ? ((G.m + kTcM - 1) / kTcM) * ((G.n + kTcN - 1) / kTcN)
                            : 0;
      acc += (int32_t)t;
      S.prefix[i + 1] = acc;
    }
    mbar_fence_init();
  }
  if (warp == 1) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
            smem_addr(&S.tmem_base)),
        "r"(kTmemCols)
        : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem_base;
  const int64_t total = S.prefix[ninst];
  volatile int* abort_flag = &S.abort_flag;

  if (warp == 0) {
    // ------------------------------------------------ producer
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int armed[kTcStages];
      uint32_t armed_par[kTcStages];
      for (int s = 0; s < kTcStages; ++s) armed[s] = 0, armed_par[s] = 0;
      for (int64_t t = blockIdx.x; t < total && !*abort_flag; t += gridDim.x) {
        int inst;
        int64_t mt, nt;
        tile_coords(S, insts, t, &inst, &mt, &nt);
        const TcGemmInst& G = insts[inst];
        const int chunks = (G.kk + kTcKC - 1) / kTcKC;
        const uint8_t* pa = reinterpret_cast<const uint8_t*>(G.apack) +
                            (size_t)mt * chunks * 2 * kTcBlock;
        const uint8_t* pb = reinterpret_cast<const uint8_t*>(G.bpack) +
                            (size_t)nt * chunks * 2 * kTcBlock;
        for (int c = 0; c < chunks; ++c) {
          if (!tc_wait(&S.empty[stage], phase ^ 1, err, abort_flag)) break;
          uint8_t* dst = base + stage * kTcStageBytes;
          armed[stage] = 1;
          armed_par[stage] = phase;
          mbar_arrive_expect_tx(&S.full[stage], kTcStageBytes);
          bulk_g2s(dst, pa + (size_t)c * 2 * kTcBlock, 2 * kTcBlock, &S.full[stage]);
          bulk_g2s(dst + 2 * kTcBlock, pb + (size_t)c * 2 * kTcBlock, 2 * kTcBlock,
                   &S.full[stage]);
          if (++stage == kTcStages) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
      // drain: every copy this thread issued has landed before the CTA exits
      // (immediate in the normal path, bounded when a consumer gave up)
      for (int q = 0; q < kTcStages; ++q) {
        if (!armed[q]) continue;
        for (uint32_t it = 0; it < kSpinLimit; ++it)
          if (mbar_try_wait(&S.full[q], armed_par[q])) break;
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      int stage = 0, buf = 0;
      uint32_t phase = 0, bphase = 0;
      const uint32_t id_pos = idesc_bf16(false), id_neg = idesc_bf16(true);
      const uint32_t sbase = smem_addr(base);
      for (int64_t t = blockIdx.x; t < total && !*abort_flag; t += gridDim.x) {
        int inst;
        int64_t mt, nt;
        tile_coords(S, insts, t, &inst, &mt, &nt);
        const int chunks = (insts[inst].kk + kTcKC - 1) / kTcKC;
        if (!tc_wait(&S.tempty[buf], bphase ^ 1, err, abort_flag)) break;
        tc_fence_after();
        const uint32_t dr = tmem + (uint32_t)(buf * 256);
        const uint32_t di = dr + 128;
        bool ok = true;
        for (int c = 0; c < chunks; ++c) {
          if (!tc_wait(&S.full[stage], phase, err, abort_flag)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a_r = sbase + stage * kTcStageBytes;
          const uint32_t a_i = a_r + kTcBlock;
          const uint32_t b_r = a_r + 2 * kTcBlock;
          const uint32_t b_i = a_r + 3 * kTcBlock;
#pragma unroll
          for (int ks = 0; ks < 2; ++ks) {
            const uint32_t hi = ks * 32, lo = 64 + ks * 32;  // byte offsets in a row
            const uint32_t acc = (c > 0 || ks > 0) ? 1u : 0u;
            // Cr += Arh Brh + Arl Brh + Arh Brl - Aih Bih - Ail Bih - Aih Bil
            mma_bf16(dr, smem_desc(a_r + hi), smem_desc(b_r + hi), id_pos, acc);
            mma_bf16(dr, smem_desc(a_r + lo), smem_desc(b_r + hi), id_pos, 1u);
            mma_bf16(dr, smem_desc(a_r + hi), smem_desc(b_r + lo), id_pos, 1u);
            mma_bf16(dr, smem_desc(a_i + hi), smem_desc(b_i + hi), id_neg, 1u);
            mma_bf16(dr, smem_desc(a_i + lo), smem_desc(b_i + hi), id_neg, 1u);
            mma_bf16(dr, smem_desc(a_i + hi), smem_desc(b_i + lo), id_neg, 1u);
            // Ci += Arh Bih + Arl Bih + Arh Bil + Aih Brh + Ail Brh + Aih Brl
            mma_bf16(di, smem_desc(a_r + hi), smem_desc(b_i + hi), id_pos, acc);
            mma_bf16(di, smem_desc(a_r + lo), smem_desc(b_i + hi), id_pos, 1u);
            mma_bf16(di, smem_desc(a_r + hi), smem_desc(b_i + lo), id_pos, 1u);
            mma_bf16(di, smem_desc(a_i + hi), smem_desc(b_r + hi), id_pos, 1u);
            mma_bf16(di, smem_desc(a_i + lo), smem_desc(b_r + hi), id_pos, 1u);
            mma_bf16(di, smem_desc(a_i + hi), smem_desc(b_r + lo), id_pos, 1u);
          }
          mma_commit(&S.empty[stage]);  // stage reusable once these MMAs are done
          if (++stage == kTcStages) {
            stage = 0;
            phase ^= 1;
          }
        }
        if (!ok) break;
        mma_commit(&S.tfull[buf]);  // accumulators complete
        if (++buf == 2) {
          buf = 0;
          bphase ^= 1;
        }
      }
    }
  } else {
    // ------------------------------------------------ epilogue (warps 2..9)
    // Warp w reads TMEM lane quadrant w % 4 (hardware rule); warps 2..5 take tile
    // columns 0..63 and warps 6..9 columns 64..127.  The C values of a 16-column chunk
    // are loaded before they are needed (the first chunk before the accumulators are
    // ready), so each thread keeps 16 independent loads in flight.
    const int quad = warp & 3;
    const int half = (warp - 2) >> 2;
    const int row = quad * 32 + lane;
    const bool leader = threadIdx.x == 64;  // warp 2, lane 0: issues the reductions
    int buf = 0;
    uint32_t bphase = 0;
    if (red) {
      // ---- reduction epilogue: C += (-acc) through the TMA unit.  Every control
      // decision is taken by the leader and published through shared memory behind the
      // epilogue barrier, so the eight warps always pass the same barriers.
      int rchunk = 0;  // reduction chunks issued (selects the staging buffer)
      for (int64_t t = blockIdx.x; t < total; t += gridDim.x) {
        if (leader) S.epi_go = (!*abort_flag && tc_wait(&S.tfull[buf], bphase, err, abort_flag)) ? 1 : 0;
        epi_bar();
        if (!S.epi_go) break;
        tc_fence_after();
        int inst;
        int64_t mt, nt;
        tile_coords(S, insts, t, &inst, &mt, &nt);
        const TcGemmInst& G = insts[inst];
        const uint32_t tl = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * 256);
        const int32_t x0 = (int32_t)(2 * (G.c_r0 + mt * kTcM));
        const int64_t ncols = G.n - nt * kTcN;
        const int nchunks =
            (int)min((int64_t)(kTcN / kTcRedCols), (ncols + kTcRedCols - 1) / kTcRedCols);
#pragma unroll 1
        for (int cc = 0; cc < nchunks; ++cc, ++rchunk) {
          uint8_t* sb = red_smem + (rchunk & 1) * kTcRedBytes;
          if (leader) bulk_wait_read1();  // the reduction that used this buffer has read it
          epi_bar();
          const int j0 = cc * kTcRedCols + half * 8;
          float vr[8], vi[8];
          tmem_ld8(tl + (uint32_t)j0, vr);
          tmem_ld8(tl + 128u + (uint32_t)j0, vi);
          tmem_wait_ld();
#pragma unroll
          for (int j = 0; j < 8; ++j)
            *reinterpret_cast<float2*>(sb + ((half * 8 + j) * kTcM + row) * 8) =
                make_float2(-vr[j], -vi[j]);
          fence_async_smem();
          epi_bar();
          if (leader) {
            red_add_tile(G.cmap, x0, (int32_t)(G.c_c0 + nt * kTcN + cc * kTcRedCols),
                         smem_addr(sb));
            bulk_commit();
          }
        }
        tc_fence_before();
        mbar_arrive(&S.tempty[buf]);
        if (++buf == 2) {
          buf = 0;
          bphase ^= 1;
        }
      }
      if (leader) bulk_wait_all();  // every reduction performed before the CTA exits
    }
    for (int64_t t = blockIdx.x; !red && t < total && !*abort_flag; t += gridDim.x) {
      int inst;
      int64_t mt, nt;
      tile_coords(S, insts, t, &inst, &mt, &nt);
      const TcGemmInst& G = insts[inst];
      const int64_t gr = mt * kTcM + row;
      const bool row_ok = gr < G.m;
      float2* C = reinterpret_cast<float2*>(G.c);
      const int64_t ncols = G.n - nt * kTcN;
      const int64_t rbase = G.c_r0 + gr;
      const int64_t cbase = G.c_c0 + nt * kTcN;
      const int c0 = half * 64;
      float2 cur[16], nxt[16];
#pragma unroll
      for (int j = 0; j < 16; ++j)
        cur[j] = (row_ok && c0 + j < ncols) ? C[rbase + (cbase + c0 + j) * G.ldc]
                                            : make_float2(0.f, 0.f);
      if (!tc_wait(&S.tfull[buf], bphase, err, abort_flag)) break;
      tc_fence_after();
      const uint32_t tl = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * 256);
#pragma unroll 1
      for (int cc = 0; cc < 4; ++cc) {
        const int j0 = c0 + cc * 16;
        float vr[16], vi[16];
        tmem_ld16(tl + (uint32_t)j0, vr);
        tmem_ld16(tl + 128u + (uint32_t)j0, vi);
        tmem_wait_ld();
        if (cc < 3) {
#pragma unroll
          for (int j = 0; j < 16; ++j)
            nxt[j] = (row_ok && j0 + 16 + j < ncols)
                         ? C[rbase + (cbase + j0 + 16 + j) * G.ldc]
                         : make_float2(0.f, 0.f);
        }
        if (row_ok) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            if (j0 + j < ncols) {
              float2 v = cur[j];
              v.x -= vr[j];
              v.y -= vi[j];
              C[rbase + (cbase + j0 + j) * G.ldc] = v;
            }
          }
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) cur[j] = nxt[j];
      }
      tc_fence_before();
      mbar_arrive(&S.tempty[buf]);
      if (++buf == 2) {
        buf = 0;
        bphase ^= 1;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

// ------------------------------------------------------------------ host side
size_t tc_pack_bytes(int64_t rows, int kk) {
  const int64_t tiles = (rows + kTcM - 1) / kTcM;
  const int chunks = (kk + kTcKC - 1) / kTcKC;
  return (size_t)tiles * chunks * 2 * kTcBlock;
}

void launch_tc_pack(const Launch& L, const TcPackInst* d, int ninst, int64_t max_rows,
                    int max_kk) {
  if (ninst <= 0 || max_rows <= 0 || max_kk <= 0) return;
  dim3 grid((unsigned)((max_rows + kTcM - 1) / kTcM), (unsigned)((max_kk + kTcKC - 1) / kTcKC),
            (unsigned)ninst);
  k_tc_pack<<<grid, 256, 0, L.stream>>>(d);
  count_launch(1);
}

bool tc_encode_cmap(void* map, const void* c, int64_t ldc, int64_t rows, int64_t cols) {
  // the driver entry point is process-wide; a function-local static is initialised once,
  // thread-safely
  static const PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    cudaGetLastError();
    return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
  }();
  if (!encode || (ldc & 1) || rows <= 0 || cols <= 0 ||
      (reinterpret_cast<uintptr_t>(c) & 15) != 0)
    return false;
  const cuuint64_t dims[2] = {(cuuint64_t)(2 * rows), (cuuint64_t)cols};
  const cuuint64_t strides[1] = {(cuuint64_t)ldc * 8};
  const cuuint32_t box[2] = {2 * kTcM, kTcRedCols};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = encode(reinterpret_cast<CUtensorMap*>(map), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                      const_cast<void*>(c), dims, strides, box, estr,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

void launch_tc_cgemm(const Launch& L, const TcGemmInst* d, int ninst, int64_t total_tiles,
                     bool red) {
  if (ninst <= 0 || total_tiles <= 0) return;
  const size_t smem = 1024 + kTcStages * kTcStageBytes + 2 * kTcRedBytes + sizeof(TcShared);
  static PerDeviceOnce attr;
  attr.call([&] {
    cudaFuncSetAttribute(k_tc_cgemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  });
  const int64_t sms = device_sm_count();
  const int64_t grid = total_tiles < sms ? total_tiles : sms;
  k_tc_cgemm<<<(unsigned)grid, kTcThreads, smem, L.stream>>>(d, ninst, L.err_flag, red ? 1 : 0);
  count_launch(1);
}

}  // namespace bemgpu
