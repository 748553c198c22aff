// Batched dense complex linear algebra for the BEM systems (complex128 and complex64).
//
// Every kernel takes a device array of MatInst descriptors and handles all instances
// of a batch in one launch (blockIdx.z or blockIdx.y selects the instance); instances
// whose order is exhausted at the current step return at once, so batches of uneven
// size share one launch sequence.
//
// LU: right-looking blocked partial pivoting (LAPACK zgetrf semantics: pivot = first
// row of largest |re| + |im| in the column, P A = L U with unit lower L):
//   getf2   panel of kPanelNB columns, one CTA per instance, column by column;
//   laswp   the panel's row interchanges applied to the columns outside it;
//   trsm    U12 = L11^{-1} A12, one warp per column of A12;
//   gemm    A22 -= L21 U12 (SIMT tile kernel; the complex64 factor of the mixed path
//           uses the tensor-core kernel in gemm_tc.cu instead).
// getrs: row interchanges, then blocked triangular solves: a diagonal-block solve
// (one CTA per instance and right-hand side) followed by a rank-update of the rows
// still to solve, for L, U, U^H and L^H (the last two for condition estimation).
#include <cfloat>
#include <cstdio>

#include "bemgpu_internal.h"
#include <algorithm>

#include "linalg.cuh"

namespace bemgpu {

// ------------------------------------------------------------------ helpers
template <typename R>
__device__ __forceinline__ cx<R> ld(const void* base, int64_t idx) {
  if constexpr (sizeof(R) == 8) {
    double2 v = reinterpret_cast<const double2*>(base)[idx];
    return {v.x, v.y};
  } else {
    float2 v = reinterpret_cast<const float2*>(base)[idx];
    return {v.x, v.y};
  }
}
template <typename R>
__device__ __forceinline__ void st(void* base, int64_t idx, cx<R> v) {
  if constexpr (sizeof(R) == 8)
    reinterpret_cast<double2*>(base)[idx] = make_double2(v.x, v.y);
  else
    reinterpret_cast<float2*>(base)[idx] = make_float2(v.x, v.y);
}
template <typename R>
__device__ __forceinline__ R cabs1(cx<R> a) {
  return fabs(a.x) + fabs(a.y);
}
template <typename R>
__device__ __forceinline__ cx<R> cinv(cx<R> a) {
  R s = fmax(fabs(a.x), fabs(a.y));
  R ar = a.x / s, ai = a.y / s;
  R d = (ar * ar + ai * ai) * s;
  return {ar / d, -ai / d};
}
template <typename R>
__device__ __forceinline__ cx<R> cconj(cx<R> a) {
  return {a.x, -a.y};
}

// ------------------------------------------------------------------ getf2 (panel)
// One CTA per instance factors the nbe-column panel at k0 column by column.  The panel
// lives in global memory (L2); every pass issues independent loads in groups (4 rows
// in the pivot search, 8 columns in the update) before any dependent store, so each
// thread keeps several requests in flight.
template <typename R>
struct Getf2Cfg;
template <>
struct Getf2Cfg<float> {
  static constexpr int kThreads = 1024;
};
template <>
struct Getf2Cfg<double> {
  static constexpr int kThreads = 512;
};

template <typename R>
__global__ void __launch_bounds__(Getf2Cfg<R>::kThreads) k_getf2(const MatInst* __restrict__ insts,
                                                                int64_t k0, int nb) {
  constexpr int T = Getf2Cfg<R>::kThreads;
  const MatInst& M = insts[blockIdx.x];
  const int64_t n = M.n;
  if (!M.active || k0 >= n) return;
  const int nbe = (int)min((int64_t)nb, n - k0);
  const int64_t lda = M.lda;
  void* A = M.a;
  __shared__ R s_val[T / 32];
  __shared__ int64_t s_idx[T / 32];
  __shared__ cx<R> s_u[kPanelNB];
  __shared__ int64_t s_piv;
  __shared__ R s_pmax;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int c = 0; c < nbe; ++c) {
    const int64_t col = k0 + c;
    const void* colp = static_cast<const cx<R>*>(A) + col * lda;
    // pivot search: largest |re|+|im|, first index on ties
    R best = (R)-1;
    int64_t bidx = col;
    for (int64_t r = col + tid; r < n; r += 4 * T) {
      R v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t rr = r + (int64_t)u * T;
        v[u] = rr < n ? cabs1(ld<R>(colp, rr)) : (R)-1;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (v[u] > best) {
          best = v[u];
          bidx = r + (int64_t)u * T;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      R ov = __shfl_down_sync(0xffffffffu, best, off);
      int64_t oi = __shfl_down_sync(0xffffffffu, bidx, off);
      if (ov > best || (ov == best && oi < bidx)) {
        best = ov;
        bidx = oi;
      }
    }
    if (lane == 0) {
      s_val[wid] = best;
      s_idx[wid] = bidx;
    }
    __syncthreads();
    if (tid == 0) {
      R bv = s_val[0];
      int64_t bi = s_idx[0];
      for (int w = 1; w < T / 32; ++w)
        if (s_val[w] > bv || (s_val[w] == bv && s_idx[w] < bi)) {
          bv = s_val[w];
          bi = s_idx[w];
        }
      s_piv = bi;
      s_pmax = bv;
      M.ipiv[col] = (int32_t)bi;
      if (!(bv > (R)0) && *M.info == 0) *M.info = (int32_t)(col + 1);
    }
    __syncthreads();
    const int64_t piv = s_piv;
    const bool nonzero = s_pmax > (R)0;
    if (nonzero && piv != col && tid < nbe) {
      const int64_t cc = k0 + tid;
      cx<R> a = ld<R>(A, col + cc * lda), b = ld<R>(A, piv + cc * lda);
      st<R>(A, col + cc * lda, b);
      st<R>(A, piv + cc * lda, a);
    }
    __syncthreads();
    if (tid < nbe) s_u[tid] = ld<R>(A, col + (k0 + tid) * lda);
    __syncthreads();
    const cx<R> inv = nonzero ? cinv(s_u[c]) : cx<R>{(R)1, (R)0};
    for (int64_t r = col + 1 + tid; r < n; r += T) {
      cx<R> l = ld<R>(A, r + col * lda);
      if (nonzero) {
        l = l * inv;
        st<R>(A, r + col * lda, l);
      }
      for (int cc0 = c + 1; cc0 < nbe; cc0 += 8) {
        cx<R> a[8];
#pragma unroll
        for (int e = 0; e < 8; ++e)
          if (cc0 + e < nbe) a[e] = ld<R>(A, r + (k0 + cc0 + e) * lda);
#pragma unroll
        for (int e = 0; e < 8; ++e)
          if (cc0 + e < nbe) st<R>(A, r + (k0 + cc0 + e) * lda, a[e] - l * s_u[cc0 + e]);
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ getf2, left-looking
// Complex64 panel factorisation for the LU driver: column c is brought up to date only
// when it is reached (U[0:c, c] by one warp from the finished L11 rows cached in shared
// memory, then a[r, c] -= sum_j L[r, j] u_j for the rows below), and the pivot search is
// fused into that pass, as is the scaling of column c - 1 by its pivot's reciprocal.
// Each row of the panel is read about c + 2 times at column c instead of the
// right-looking 2 (31 - c) + 1, and a cluster of CS CTAs shares an instance's rows
// (fixed ownership: row k0 + g + t CS T belongs to cluster thread g), exchanging
// the pivot candidates through distributed shared memory.  Two cluster barriers per
// column order the global writes of one CTA before the reads of the other.  Pivoting
// rule, interchanges and the singular marker are those of the right-looking kernel.
constexpr int kGetf2T = 1024;
constexpr int kLLBatch = 16;  // L values per row in flight

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::
                   : "memory");
}
__device__ __forceinline__ uint32_t peer_smem(const void* p, unsigned rank) {
  uint32_t a = (uint32_t)__cvta_generic_to_shared(p), r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ float ld_peer_f32(uint32_t a) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ int32_t ld_peer_s32(uint32_t a) {
  int32_t v;
  asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
  return v;
}
template <typename V>
__device__ __forceinline__ void better32(V& bv, int32_t& bi, V ov, int32_t oi) {
  if (ov > bv || (ov == bv && oi < bi)) {
    bv = ov;
    bi = oi;
  }
}
__device__ __forceinline__ double ld_peer_f64(uint32_t a) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(a) : "memory");
  return v;
}
template <typename R>
__device__ __forceinline__ R ld_peer_real(uint32_t a) {
  if constexpr (sizeof(R) == 8)
    return ld_peer_f64(a);
  else
    return ld_peer_f32(a);
}
__device__ __forceinline__ long long ld_peer_s64(uint32_t a) {
  long long v;
  asm volatile("ld.shared::cluster.s64 %0, [%1];" : "=l"(v) : "r"(a) : "memory");
  return v;
}

__device__ __forceinline__ void better(float& bv, int64_t& bi, float ov, int64_t oi) {
  if (ov > bv || (ov == bv && oi < bi)) {
    bv = ov;
    bi = oi;
  }
}

template <typename R, int CS, int T, int BATCH>
__global__ void __launch_bounds__(T) k_getf2_ll(const MatInst* __restrict__ insts, int64_t k0,
                                                int nb) {
  using C = cx<R>;
  const unsigned rank = CS > 1 ? cluster_rank() : 0u;
  const MatInst& M = insts[blockIdx.x / CS];
  const int64_t n = M.n;
  if (!M.active || k0 >= n) return;  // the whole cluster (one instance) leaves together
  const int nbe = (int)min((int64_t)nb, n - k0);
  const int64_t lda = M.lda;
  void* A = M.a;
  __shared__ C sL[kPanelNB][kPanelNB + 1];  // finished L11 rows
  __shared__ C su[kPanelNB];                // U[0:c, c]
  __shared__ R w_val[T / 32];
  __shared__ int32_t w_idx[T / 32];         // rows as int32 (orders below 2^31)
  __shared__ R c_val;                       // this CTA's pivot candidate
  __shared__ int32_t c_idx;
  __shared__ C s_inv;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int64_t g = (int64_t)rank * T + tid;
  constexpr int64_t stride = (int64_t)CS * T;
  C inv_prev = {(R)1, (R)0};
  for (int c = 0; c < nbe; ++c) {
    const int64_t col = k0 + c;
    // (1) u = L11[0:c, 0:c]^{-1} a[k0:k0+c, col] (identical in every CTA)
    if (wid == 0) {
      C x = {(R)0, (R)0};
      if (lane < c) x = ld<R>(A, (k0 + lane) + col * lda);
      for (int i = 0; i + 1 < c; ++i) {
        C ui;
        ui.x = __shfl_sync(0xffffffffu, x.x, i);
        ui.y = __shfl_sync(0xffffffffu, x.y, i);
        if (lane > i && lane < c) x -= sL[lane][i] * ui;
      }
      if (lane < c) su[lane] = x;  // stored after the first cluster barrier (peers read
                                   // the original values of these rows first)
    }
    __syncthreads();
    // (2) rows >= col: finish L[., c - 1], update column c, pivot candidate
    R best = (R)-1;
    int32_t bidx = INT32_MAX;
    int64_t r = k0 + g;
    if (r < col) r += ((col - r + stride - 1) / stride) * stride;
    for (; r < n; r += stride) {
      C acc = ld<R>(A, r + col * lda);
      for (int j0 = 0; j0 < c; j0 += BATCH) {
        C lv[BATCH];
#pragma unroll
        for (int e = 0; e < BATCH; ++e) {
          lv[e] = C{(R)0, (R)0};
          if (j0 + e < c) lv[e] = ld<R>(A, r + (k0 + j0 + e) * lda);
        }
#pragma unroll
        for (int e = 0; e < BATCH; ++e) {
          if (j0 + e < c) {
            if (j0 + e == c - 1) {
              lv[e] = lv[e] * inv_prev;
              st<R>(A, r + (k0 + j0 + e) * lda, lv[e]);
            }
            acc -= lv[e] * su[j0 + e];
          }
        }
      }
      st<R>(A, r + col * lda, acc);
      better32(best, bidx, cabs1(acc), (int32_t)r);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const R ov = __shfl_down_sync(0xffffffffu, best, off);
      const int32_t oi = __shfl_down_sync(0xffffffffu, bidx, off);
      better32(best, bidx, ov, oi);
    }
    if (lane == 0) {
      w_val[wid] = best;
      w_idx[wid] = bidx;
    }
    __syncthreads();
    if (wid == 0) {  // the CTA's candidate: a shuffle tree over the 32 warps' candidates
      R bv = lane < T / 32 ? w_val[lane] : (R)-1;
      int32_t bi = lane < T / 32 ? w_idx[lane] : INT32_MAX;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const R ov = __shfl_xor_sync(0xffffffffu, bv, off);
        const int32_t oi = __shfl_xor_sync(0xffffffffu, bi, off);
        better32(bv, bi, ov, oi);
      }
      if (lane == 0) {
        c_val = bv;
        c_idx = bi;
      }
    }
    // (3) pivot of the cluster: only warp 0 needs it (the U row, the interchange over the
    // panel's <= 32 columns, the singular marker and the pivot's reciprocal are its work)
    if (CS > 1)
      cluster_sync_all();
    else
      __syncthreads();
    R pv = (R)-1;
    int32_t piv32 = INT32_MAX;
    if (wid == 0) {  // one lane per CTA of the cluster, all peer loads in flight
      if (lane < CS) {
        if (CS > 1 && (unsigned)lane != rank) {
          pv = ld_peer_real<R>(peer_smem(&c_val, (unsigned)lane));
          piv32 = ld_peer_s32(peer_smem(&c_idx, (unsigned)lane));
        } else {
          pv = c_val;
          piv32 = c_idx;
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {  // every lane gets the cluster's pivot
        const R ov = __shfl_xor_sync(0xffffffffu, pv, off);
        const int32_t oi = __shfl_xor_sync(0xffffffffu, piv32, off);
        better32(pv, piv32, ov, oi);
      }
    }
    int64_t piv = piv32;
    if (piv >= n) piv = col;  // no candidate rows (cannot happen for col < n)
    const bool nonzero = pv > (R)0;
    if (rank == 0) {
      if (tid < c) st<R>(A, (k0 + tid) + col * lda, su[tid]);
      if (tid == 0) {
        M.ipiv[col] = (int32_t)piv;
        if (!nonzero && *M.info == 0) *M.info = (int32_t)(col + 1);
      }
      if (piv != col && tid < nbe) {  // interchange over the panel's columns
        const int64_t cc = k0 + tid;
        const C a = ld<R>(A, col + cc * lda), b = ld<R>(A, piv + cc * lda);
        st<R>(A, col + cc * lda, b);
        st<R>(A, piv + cc * lda, a);
      }
    }
    if (CS > 1)
      cluster_sync_all();
    else
      __syncthreads();
    // (4) reciprocal of the pivot; cache the finished row of L11
    if (tid < c) sL[c][tid] = ld<R>(A, col + (k0 + tid) * lda);
    if (tid == 0) s_inv = nonzero ? cinv(ld<R>(A, col + col * lda)) : C{(R)1, (R)0};
    __syncthreads();
    inv_prev = s_inv;
  }
  // scale the last column below its pivot
  const int64_t colL = k0 + nbe - 1;
  int64_t r = k0 + g;
  if (r <= colL) r += ((colL + 1 - r + stride - 1) / stride) * stride;
  for (; r < n; r += stride) st<R>(A, r + colL * lda, ld<R>(A, r + colL * lda) * inv_prev);
}

// ------------------------------------------------------------------ laswp
// Interchanges of rows k0 .. k0 + nbe - 1 (LAPACK's sequential order: row k0 + c with
// ipiv[k0 + c] for c = 0, 1, ...) applied to the columns j in [c_lo, min(c_hi, n)) that
// lie outside [s_lo, s_hi).  The sequence is first resolved, once per CTA, into the
// permutation of the rows it touches (destination row <- source row); then one warp per
// column loads every moved element (one per lane and slot, all loads in flight), meets at a
// warp barrier and stores them at their destinations.
constexpr int kSwpMaxNb = 128;   // interchanges per launch
constexpr int kSwpWarps = 8;
constexpr int kSwpCols = 128;    // columns per CTA
constexpr int kSwpHash = 512;    // open-addressing table of touched rows beyond the block

template <typename R>
__global__ void __launch_bounds__(kSwpWarps * 32) k_laswp(const MatInst* __restrict__ insts,
                                                         int64_t k0, int nb, int64_t c_lo,
                                                         int64_t c_hi, int64_t s_lo,
                                                         int64_t s_hi) {
  const MatInst& M = insts[blockIdx.y];
  const int64_t n = M.n;
  if (!M.active || k0 >= n) return;
  const int nbe = (int)min((int64_t)nb, n - k0);
  const int64_t skip = s_hi - s_lo;
  auto column = [&](int64_t q) {  // compacted column index -> matrix column (or -1)
    int64_t j = c_lo + q;
    if (j >= s_lo) j += skip;
    return (j >= n || j >= c_hi) ? (int64_t)-1 : j;
  };
  const int64_t q0 = (int64_t)blockIdx.x * kSwpCols;
  if (column(q0) < 0) return;  // uniform per CTA
  __shared__ int32_t piv[kSwpMaxNb];
  __shared__ int32_t pos[2 * kSwpMaxNb], src[2 * kSwpMaxNb];  // slot: row, its source row
  __shared__ int32_t hkey[kSwpHash];
  __shared__ int16_t hslot[kSwpHash];
  __shared__ int32_t mpos[2 * kSwpMaxNb], msrc[2 * kSwpMaxNb];
  __shared__ int nmove;
  const int tid = threadIdx.x;
  for (int c = tid; c < nbe; c += blockDim.x) piv[c] = M.ipiv[k0 + c];
  for (int h = tid; h < kSwpHash; h += blockDim.x) hkey[h] = -1;
  __syncthreads();
  if (tid == 0) {
    int ns = nbe;
    for (int c = 0; c < nbe; ++c) pos[c] = src[c] = (int32_t)(k0 + c);
    for (int c = 0; c < nbe; ++c) {
      const int32_t p = piv[c];
      if (p == (int32_t)(k0 + c)) continue;
      int sp;
      if (p < (int32_t)(k0 + nbe)) {
        sp = p - (int32_t)k0;
      } else {
        int h = (int)(((uint32_t)p * 2654435761u) >> 23) & (kSwpHash - 1);
        while (hkey[h] != -1 && hkey[h] != p) h = (h + 1) & (kSwpHash - 1);
        if (hkey[h] == -1) {
          hkey[h] = p;
          hslot[h] = (int16_t)ns;
          pos[ns] = src[ns] = p;
          ++ns;
        }
        sp = hslot[h];
      }
      const int32_t t = src[c];
      src[c] = src[sp];
      src[sp] = t;
    }
    int nm = 0;
    for (int t = 0; t < ns; ++t)
      if (src[t] != pos[t]) {
        mpos[nm] = pos[t];
        msrc[nm] = src[t];
        ++nm;
      }
    nmove = nm;
  }
  __syncthreads();
  const int nm = nmove;
  if (nm == 0) return;
  const int lane = tid & 31, wid = tid >> 5;
  const int64_t lda = M.lda;
  constexpr int kPer = 2 * kSwpMaxNb / 32;
  for (int q = wid; q < kSwpCols; q += kSwpWarps) {
    const int64_t j = column(q0 + q);
    if (j < 0) break;
    cx<R> v[kPer];
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int t = lane + 32 * u;
      if (t < nm) v[u] = ld<R>(M.a, msrc[t] + j * lda);
    }
    __syncwarp();  // every load of this column is performed before any store
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int t = lane + 32 * u;
      if (t < nm) st<R>(M.a, mpos[t] + j * lda, v[u]);
    }
  }
}

// ------------------------------------------------------------------ trsm (U12)
// U12 = L11^{-1} A12 for the columns [c_lo, min(c_hi, n)); L11 = unit lower nbe x nbe
// block at (k0, k0), staged once per CTA in shared memory; each warp solves TrsmCols<R>
// columns (column = warp + kTrsmWarps * t), lane r holding rows r, r + 32, ...
// complex128 takes fewer columns per warp: its FP64 solve is about 8x slower per column,
// and more CTAs spread the few trailing columns of small orders over the SMs.
constexpr int kTrsmWarps = 8;
template <typename R>
struct TrsmCols {
  static constexpr int value = sizeof(R) == 4 ? 16 : 2;
};

template <typename R, int NB>
__global__ void __launch_bounds__(kTrsmWarps * 32) k_trsm_panel(const MatInst* __restrict__ insts,
                                                               int64_t k0, int64_t c_lo,
                                                               int64_t c_hi) {
  constexpr int kTrsmCols = TrsmCols<R>::value;
  const MatInst& M = insts[blockIdx.y];
  const int64_t n = M.n;
  if (!M.active || k0 >= n) return;
  const int nbe = (int)min((int64_t)NB, n - k0);
  const int64_t lda = M.lda;
  const int64_t c_end = min(c_hi, n);
  const int64_t cta0 = c_lo + (int64_t)blockIdx.x * kTrsmWarps * kTrsmCols;
  if (cta0 >= c_end) return;  // uniform per CTA
  extern __shared__ __align__(16) unsigned char trsm_smem[];
  cx<R>* sL = reinterpret_cast<cx<R>*>(trsm_smem);  // [NB][NB + 1]
  for (int t = threadIdx.x; t < nbe * nbe; t += blockDim.x) {
    int r = t % nbe, c = t / nbe;
    sL[r * (NB + 1) + c] = ld<R>(M.a, (k0 + r) + (k0 + c) * lda);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int kPer = NB / 32;
  for (int tcol = 0; tcol < kTrsmCols; ++tcol) {
    const int64_t j = cta0 + wid + (int64_t)kTrsmWarps * tcol;
    if (j >= c_end) break;
    cx<R> x[kPer];
#pragma unroll
    for (int t = 0; t < kPer; ++t) {
      int r = lane + 32 * t;
      x[t] = r < nbe ? ld<R>(M.a, (k0 + r) + j * lda) : cx<R>{0, 0};
    }
#pragma unroll
    for (int t = 0; t < kPer; ++t) {
      for (int cl = 0; cl < 32; ++cl) {
        const int c = 32 * t + cl;
        if (c >= nbe) break;
        cx<R> xc;
        xc.x = __shfl_sync(0xffffffffu, x[t].x, cl);
        xc.y = __shfl_sync(0xffffffffu, x[t].y, cl);
#pragma unroll
        for (int u = t; u < kPer; ++u) {
          int r = lane + 32 * u;
          if (r > c && r < nbe) x[u] -= sL[r * (NB + 1) + c] * xc;
        }
      }
    }
#pragma unroll
    for (int t = 0; t < kPer; ++t) {
      int r = lane + 32 * t;
      if (r < nbe) st<R>(M.a, (k0 + r) + j * lda, x[t]);
    }
  }
}

// ------------------------------------------------------------------ SIMT gemm update
// C(m x m') -= A(m x kk) B(kk x m') with A = L21, B = U12, C = A22 of each instance.
constexpr int kGT = 64;   // tile edge
constexpr int kGK = 8;    // k chunk
constexpr int kGThreads = 256;

// Rows [k0 + nbe, n), columns [c_lo, min(c_hi, n)).
template <typename R>
__global__ void __launch_bounds__(kGThreads) k_gemm_update(const MatInst* __restrict__ insts,
                                                          int64_t k0, int nb, int64_t c_lo,
                                                          int64_t c_hi) {
  const MatInst& M = insts[blockIdx.y];
  const int64_t n = M.n;
  if (!M.active || k0 >= n) return;
  const int nbe = (int)min((int64_t)nb, n - k0);
  const int64_t s = k0 + nbe;  // first trailing row
  const int64_t m = n - s;
  const int64_t c_end = min(c_hi, n);
  const int64_t w = c_end - c_lo;
  if (m <= 0 || w <= 0) return;
  const int64_t tiles_m = (m + kGT - 1) / kGT, tiles_n = (w + kGT - 1) / kGT;
  const int64_t t = blockIdx.x;
  if (t >= tiles_m * tiles_n) return;
  const int64_t ti = t % tiles_m, tj = t / tiles_m;
  const int64_t r0 = s + ti * kGT, c0 = c_lo + tj * kGT;
  const int64_t lda = M.lda;
  __shared__ cx<R> sA[kGK][kGT + 1];
  __shared__ cx<R> sB[kGK][kGT + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  cx<R> acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = cx<R>{0, 0};
  for (int kc = 0; kc < nbe; kc += kGK) {
    for (int e = threadIdx.x; e < kGK * kGT; e += kGThreads) {
      int rr = e % kGT, kk = e / kGT;
      int64_t gr = r0 + rr, gk = k0 + kc + kk;
      sA[kk][rr] = (gr < n && kc + kk < nbe) ? ld<R>(M.a, gr + gk * lda) : cx<R>{0, 0};
      int kb = e % kGK;
      int cc = e / kGK;
      int64_t gc = c0 + cc, gkb = k0 + kc + kb;
      sB[kb][cc] = (gc < c_end && kc + kb < nbe) ? ld<R>(M.a, gkb + gc * lda) : cx<R>{0, 0};
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kGK; ++kk) {
      cx<R> av[4], bv[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) av[a] = sA[kk][tx + 16 * a];
#pragma unroll
      for (int b = 0; b < 4; ++b) bv[b] = sB[kk][ty + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] += av[a] * bv[b];
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      int64_t gr = r0 + tx + 16 * a, gc = c0 + ty + 16 * b;
      if (gr < n && gc < c_end) {
        int64_t idx = gr + gc * lda;
        st<R>(M.a, idx, ld<R>(M.a, idx) - acc[a][b]);
      }
    }
}

// ------------------------------------------------------------------ getrs pieces
// Row interchanges on the right-hand sides (forward: ipiv in order; back: reverse).
template <typename R>
__global__ void k_rhs_swap(const MatInst* __restrict__ insts, int reverse) {
  const MatInst& M = insts[blockIdx.y];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (!M.active || r >= M.nrhs) return;
  const int64_t n = M.n;
  void* X = M.x;
  const int64_t off = (int64_t)r * M.ldx;
  if (!reverse) {
    for (int64_t i = 0; i < n; ++i) {
      int64_t p = M.ipiv[i];
      if (p != i) {
        cx<R> a = ld<R>(X, off + i), b = ld<R>(X, off + p);
        st<R>(X, off + i, b);
        st<R>(X, off + p, a);
      }
    }
  } else {
    for (int64_t i = n - 1; i >= 0; --i) {
      int64_t p = M.ipiv[i];
      if (p != i) {
        cx<R> a = ld<R>(X, off + i), b = ld<R>(X, off + p);
        st<R>(X, off + i, b);
        st<R>(X, off + p, a);
      }
    }
  }
}

// element (r, c) of op(A): A or A^H
template <typename R, bool TRANS>
__device__ __forceinline__ cx<R> opel(const void* A, int64_t lda, int64_t r, int64_t c) {
  if (TRANS) return cconj(ld<R>(A, c + r * lda));
  return ld<R>(A, r + c * lda);
}

// Diagonal block solve: rows [r0, r0 + nbs) of op(T) x = x, op(T) lower when
// EFF_LOWER.  One CTA (kTrsvNB threads) per (rhs, instance).
template <typename R, bool EFF_LOWER, bool TRANS, bool UNIT>
__global__ void __launch_bounds__(kTrsvNB) k_trsv_block(const MatInst* __restrict__ insts,
                                                        int64_t r0) {
  const MatInst& M = insts[blockIdx.y];
  const int rhs = blockIdx.x;
  const int64_t n = M.n;
  if (!M.active || rhs >= M.nrhs || r0 >= n) return;
  const int nbs = (int)min((int64_t)kTrsvNB, n - r0);
  const int64_t lda = M.lda, off = (int64_t)rhs * M.ldx;
  __shared__ cx<R> sx[kTrsvNB];
  const int t = threadIdx.x;
  if (t < nbs) sx[t] = ld<R>(M.x, off + r0 + t);
  __syncthreads();
  if (EFF_LOWER) {
    for (int c = 0; c < nbs; ++c) {
      if (!UNIT && t == c) sx[c] = sx[c] * cinv(opel<R, TRANS>(M.a, lda, r0 + c, r0 + c));
      __syncthreads();
      if (t > c && t < nbs) sx[t] -= opel<R, TRANS>(M.a, lda, r0 + t, r0 + c) * sx[c];
      __syncthreads();
    }
  } else {
    for (int c = nbs - 1; c >= 0; --c) {
      if (!UNIT && t == c) sx[c] = sx[c] * cinv(opel<R, TRANS>(M.a, lda, r0 + c, r0 + c));
      __syncthreads();
      if (t < c) sx[t] -= opel<R, TRANS>(M.a, lda, r0 + t, r0 + c) * sx[c];
      __syncthreads();
    }
  }
  if (t < nbs) st<R>(M.x, off + r0 + t, sx[t]);
}

// Update of the unsolved rows by the solved block [r0, r0 + nbs): thread per row.
template <typename R, bool EFF_LOWER, bool TRANS>
__global__ void __launch_bounds__(256) k_trsv_update(const MatInst* __restrict__ insts,
                                                     int64_t r0) {
  const MatInst& M = insts[blockIdx.z];
  const int rhs = blockIdx.y;
  const int64_t n = M.n;
  if (!M.active || rhs >= M.nrhs || r0 >= n) return;
  const int nbs = (int)min((int64_t)kTrsvNB, n - r0);
  const int64_t lda = M.lda, off = (int64_t)rhs * M.ldx;
  __shared__ cx<R> sx[kTrsvNB];
  if (threadIdx.x < nbs) sx[threadIdx.x] = ld<R>(M.x, off + r0 + threadIdx.x);
  __syncthreads();
  int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (EFF_LOWER)
    row += r0 + nbs;
  if (EFF_LOWER ? row >= n : row >= r0) return;
  cx<R> acc = {0, 0};
  for (int c = 0; c < nbs; ++c) acc += opel<R, TRANS>(M.a, lda, row, r0 + c) * sx[c];
  st<R>(M.x, off + row, ld<R>(M.x, off + row) - acc);
}

// Whole triangular solve in one launch: one CTA per (rhs, instance) holds the
// right-hand side in shared memory, walks the 32-row diagonal blocks (warp 0 solves a
// block with shuffles) and lets all threads update the unsolved rows after each block.
// SWAP 1: LAPACK's forward row interchanges before the solve; 2: the reverse
// interchanges after it (the P^T of A^H x = b); 0: none.
constexpr int kTrsvThreads = 512;

template <typename R, bool EFF_LOWER, bool TRANS, bool UNIT, int SWAP>
__global__ void __launch_bounds__(kTrsvThreads) k_trsv_full(const MatInst* __restrict__ insts) {
  const MatInst& M = insts[blockIdx.y];
  const int rhs = blockIdx.x;
  if (!M.active || rhs >= M.nrhs) return;
  const int64_t n = M.n, lda = M.lda, off = (int64_t)rhs * M.ldx;
  extern __shared__ __align__(16) unsigned char trsv_smem[];
  cx<R>* sx = reinterpret_cast<cx<R>*>(trsv_smem);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int64_t i = tid; i < n; i += kTrsvThreads) sx[i] = ld<R>(M.x, off + i);
  __syncthreads();
  if (SWAP == 1 && tid == 0) {
    for (int64_t i = 0; i < n; ++i) {
      const int64_t p = M.ipiv[i];
      if (p != i) {
        cx<R> t = sx[i];
        sx[i] = sx[p];
        sx[p] = t;
      }
    }
  }
  __syncthreads();
  const int64_t nblk = (n + 31) / 32;
  for (int64_t bb = 0; bb < nblk; ++bb) {
    const int64_t b = EFF_LOWER ? bb : nblk - 1 - bb;
    const int64_t r0 = b * 32;
    const int nb = (int)min((int64_t)32, n - r0);
    if (warp == 0) {
      cx<R> x = lane < nb ? sx[r0 + lane] : cx<R>{0, 0};
      if (EFF_LOWER) {
        for (int c = 0; c < nb; ++c) {
          if (!UNIT && lane == c) x = x * cinv(opel<R, TRANS>(M.a, lda, r0 + c, r0 + c));
          cx<R> xc;
          xc.x = __shfl_sync(0xffffffffu, x.x, c);
          xc.y = __shfl_sync(0xffffffffu, x.y, c);
          if (lane > c && lane < nb) x -= opel<R, TRANS>(M.a, lda, r0 + lane, r0 + c) * xc;
        }
      } else {
        for (int c = nb - 1; c >= 0; --c) {
          if (!UNIT && lane == c) x = x * cinv(opel<R, TRANS>(M.a, lda, r0 + c, r0 + c));
          cx<R> xc;
          xc.x = __shfl_sync(0xffffffffu, x.x, c);
          xc.y = __shfl_sync(0xffffffffu, x.y, c);
          if (lane < c) x -= opel<R, TRANS>(M.a, lda, r0 + lane, r0 + c) * xc;
        }
      }
      if (lane < nb) sx[r0 + lane] = x;
    }
    __syncthreads();
    const int64_t lo = EFF_LOWER ? r0 + nb : 0, hi = EFF_LOWER ? n : r0;
    for (int64_t r = lo + tid; r < hi; r += kTrsvThreads) {
      cx<R> acc = {0, 0};
#pragma unroll
      for (int h = 0; h < 32; h += 16) {
        cx<R> lv[16];  // 16 independent loads in flight per thread
#pragma unroll
        for (int c = 0; c < 16; ++c)
          lv[c] = (h + c < nb) ? opel<R, TRANS>(M.a, lda, r, r0 + h + c) : cx<R>{0, 0};
#pragma unroll
        for (int c = 0; c < 16; ++c)
          if (h + c < nb) acc += lv[c] * sx[r0 + h + c];
      }
      sx[r] -= acc;
    }
    __syncthreads();
  }
  if (SWAP == 2 && tid == 0) {
    for (int64_t i = n - 1; i >= 0; --i) {
      const int64_t p = M.ipiv[i];
      if (p != i) {
        cx<R> t = sx[i];
        sx[i] = sx[p];
        sx[p] = t;
      }
    }
  }
  __syncthreads();
  for (int64_t i = tid; i < n; i += kTrsvThreads) st<R>(M.x, off + i, sx[i]);
}

template <typename R, bool EL, bool TR, bool UN, int SW>
static void trsv_full_t(const Launch& L, const MatInst* d, int ninst, int64_t nmax,
                        int32_t max_rhs) {
  const size_t smem = (size_t)nmax * sizeof(cx<R>);
  static PerDeviceOnce attr;
  attr.call([] {
    cudaFuncSetAttribute(k_trsv_full<R, EL, TR, UN, SW>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  });
  k_trsv_full<R, EL, TR, UN, SW><<<dim3((unsigned)max_rhs, (unsigned)ninst), kTrsvThreads, smem,
                                   L.stream>>>(d);
  count_launch(1);
}

// largest order whose right-hand side fits the shared memory of one CTA
static int64_t trsv_full_max(int prec) { return (int64_t)(220 * 1024) / (prec == 1 ? 8 : 16); }

// ------------------------------------------------------------------ -(L11^{-1} - I)
// For the tensor-core U12 solve: with L11^{-1} = I + N (N strictly lower),
// U12 = L11^{-1} A12 = A12 - (-N) A12.  One CTA per instance stages the unit lower
// block L11 (nbe x nbe at (k0, k0)) in shared memory and solves L11 x = e_j for every
// column j (one warp per column); out (ld kLinvB, complex64) receives -N.
constexpr int kLinvB = 128;

__global__ void __launch_bounds__(256) k_linv_neg(const MatInst* __restrict__ insts, int64_t k0,
                                                  float2* const* outs) {
  const MatInst& M = insts[blockIdx.x];
  const int64_t n = M.n;
  if (!M.active || k0 >= n) return;
  const int nbe = (int)min((int64_t)kLinvB, n - k0);
  const int64_t lda = M.lda;
  extern __shared__ __align__(16) unsigned char linv_smem[];
  cx<float>* sL = reinterpret_cast<cx<float>*>(linv_smem);  // [kLinvB][kLinvB + 1]
  for (int t = threadIdx.x; t < nbe * nbe; t += blockDim.x) {
    int r = t % nbe, c = t / nbe;
    sL[r * (kLinvB + 1) + c] = ld<float>(M.a, (k0 + r) + (k0 + c) * lda);
  }
  __syncthreads();
  float2* out = outs[blockIdx.x];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int kPer = kLinvB / 32;
  for (int j = wid; j < kLinvB; j += 8) {
    cx<float> x[kPer];
#pragma unroll
    for (int t = 0; t < kPer; ++t) {
      const int r = lane + 32 * t;
      x[t] = cx<float>{(r == j && j < nbe) ? 1.f : 0.f, 0.f};
    }
    if (j < nbe) {
#pragma unroll
      for (int t = 0; t < kPer; ++t) {
        for (int cl = 0; cl < 32; ++cl) {
          const int c = 32 * t + cl;
          if (c >= nbe) break;
          if (c < j) continue;
          cx<float> xc;
          xc.x = __shfl_sync(0xffffffffu, x[t].x, cl);
          xc.y = __shfl_sync(0xffffffffu, x[t].y, cl);
#pragma unroll
          for (int u = t; u < kPer; ++u) {
            const int r = lane + 32 * u;
            if (r > c && r < nbe) x[u] -= sL[r * (kLinvB + 1) + c] * xc;
          }
        }
      }
    }
#pragma unroll
    for (int t = 0; t < kPer; ++t) {
      const int r = lane + 32 * t;
      const bool strict = r > j && r < nbe && j < nbe;
      out[r + (int64_t)j * kLinvB] = strict ? make_float2(-x[t].x, -x[t].y) : make_float2(0.f, 0.f);
    }
  }
}

void launch_linv_neg(const Launch& L, const MatInst* d, int ninst, int64_t k0, float2* const* outs) {
  const size_t smem = (size_t)kLinvB * (kLinvB + 1) * sizeof(cx<float>);
  static PerDeviceOnce attr;
  attr.call([&] {
    cudaFuncSetAttribute(k_linv_neg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  });
  k_linv_neg<<<ninst, 256, smem, L.stream>>>(d, k0, outs);
  count_launch(1);
}

// ------------------------------------------------------------------ blocked solves
// Two-level triangular solve: diagonal blocks of kBigB rows are solved by one CTA per
// (rhs, instance) holding the block's slice of the vector in shared memory; the rows
// outside the block are then updated by a full-GPU product kernel.  About 2 n / kBigB
// launches per triangle.
//
// Inside a diagonal block the 32 x 32 triangle of each sub-block is staged in shared
// memory (double-buffered: the next sub-block's triangle is fetched while warp 0 solves
// the current one from shared memory with shuffles), then all warps update the rest of
// the block.  op(A) = A^H reads A along its columns in both phases (a warp per row,
// lanes along the column), so every global access is coalesced.
constexpr int kBigB = 512;
constexpr int kDiagThreads = 512;
constexpr int kTilePad = 33;
constexpr int kPre = 32;  // prefetched update operands per thread
static_assert(kBigB - 32 <= kDiagThreads, "one update row per thread");
static_assert((kBigB - 32 + (kDiagThreads / 32) * 4 - 1) / ((kDiagThreads / 32) * 4) * 4 <= kPre,
              "transposed update rows per lane");

template <typename R>
constexpr size_t diag_smem_bytes() {
  return sizeof(cx<R>) * (kBigB + 2 * 32 * kTilePad + 2 * 32);
}

template <typename R, bool EFF_LOWER, bool TRANS, bool UNIT>
__global__ void __launch_bounds__(kDiagThreads) k_trsv_diag(const MatInst* __restrict__ insts,
                                                            int64_t r0) {
  const MatInst& M = insts[blockIdx.y];
  const int rhs = blockIdx.x;
  if (!M.active || rhs >= M.nrhs || r0 >= M.n) return;
  const int64_t n = M.n, lda = M.lda, off = (int64_t)rhs * M.ldx;
  const int nbs = (int)min((int64_t)kBigB, n - r0);
  extern __shared__ __align__(16) unsigned char diag_smem[];
  cx<R>* sx = reinterpret_cast<cx<R>*>(diag_smem);
  cx<R>* tiles = sx + kBigB;  // [2][32][kTilePad], tile[i][j] = op(A)[s0 + i, s0 + j]
  cx<R>* dinv = tiles + 2 * 32 * kTilePad;  // [2][32] reciprocals of the tiles' diagonals
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nsub = (nbs + 31) / 32;
  auto sub_of = [&](int bb) { return EFF_LOWER ? bb : nsub - 1 - bb; };
  // stage the triangle of sub-block b in tile buffer buf (threads [t0, kDiagThreads))
  auto stage = [&](int buf, int b, int t0) {
    const int s0 = b * 32, nb = min(32, nbs - s0);
    cx<R>* T = tiles + buf * 32 * kTilePad;
    for (int e = tid - t0; e < 1024; e += kDiagThreads - t0) {
      const int p = e & 31, q = e >> 5;  // physical A[s0 + p, s0 + q], coalesced in p
      cx<R> v = {0, 0};
      if (p < nb && q < nb) v = ld<R>(M.a, (r0 + s0 + p) + (r0 + s0 + q) * lda);
      if (TRANS)
        T[q * kTilePad + p] = cconj(v);
      else
        T[p * kTilePad + q] = v;
      if (!UNIT && p == q && p < nb) dinv[buf * 32 + p] = cinv(TRANS ? cconj(v) : v);
    }
  };
  for (int i = tid; i < nbs; i += kDiagThreads) sx[i] = ld<R>(M.x, off + r0 + i);
  stage(0, sub_of(0), 0);
  __syncthreads();
  for (int bb = 0; bb < nsub; ++bb) {
    const int b = sub_of(bb);
    const int s0 = b * 32;
    const int nb = min(32, nbs - s0);
    const cx<R>* T = tiles + (bb & 1) * 32 * kTilePad;
    const cx<R>* DI = dinv + (bb & 1) * 32;
    // this sub-block's update operands, loaded before the solve so that their memory
    // latency overlaps it (one row of 32 values per thread, or 32 column values per
    // lane for op(A) = A^H)
    constexpr int kP = sizeof(R) == 4 ? kPre : kPre / 2;  // FP64: half, rest on demand
    cx<R> pre[kP];
    {
      const int lo = EFF_LOWER ? s0 + nb : 0, hi = EFF_LOWER ? nbs : s0;
      if (!TRANS) {
        const int r = lo + tid;
#pragma unroll
        for (int c = 0; c < kP; ++c)
          pre[c] = (r < hi && c < nb) ? ld<R>(M.a, (r0 + r) + (r0 + s0 + c) * lda) : cx<R>{0, 0};
      } else {
#pragma unroll
        for (int q = 0; q < kP; ++q) {
          const int r = lo + warp * 4 + (q & 3) + (q >> 2) * (kDiagThreads / 32) * 4;
          pre[q] = (r < hi && lane < nb) ? ld<R>(M.a, (r0 + s0 + lane) + (r0 + r) * lda)
                                         : cx<R>{0, 0};
        }
      }
    }
    if (warp == 0) {
      cx<R> x = lane < nb ? sx[s0 + lane] : cx<R>{0, 0};
      if (EFF_LOWER) {
        for (int c = 0; c < nb; ++c) {
          if (!UNIT && lane == c) x = x * DI[c];
          cx<R> xc;
          xc.x = __shfl_sync(0xffffffffu, x.x, c);
          xc.y = __shfl_sync(0xffffffffu, x.y, c);
          if (lane > c && lane < nb) x -= T[lane * kTilePad + c] * xc;
        }
      } else {
        for (int c = nb - 1; c >= 0; --c) {
          if (!UNIT && lane == c) x = x * DI[c];
          cx<R> xc;
          xc.x = __shfl_sync(0xffffffffu, x.x, c);
          xc.y = __shfl_sync(0xffffffffu, x.y, c);
          if (lane < c) x -= T[lane * kTilePad + c] * xc;
        }
      }
      if (lane < nb) sx[s0 + lane] = x;
    } else if (bb + 1 < nsub) {
      stage((bb + 1) & 1, sub_of(bb + 1), 32);
    }
    __syncthreads();
    const int lo = EFF_LOWER ? s0 + nb : 0, hi = EFF_LOWER ? nbs : s0;
    if (!TRANS) {
      // one row per thread (the block's rows outside the sub-block fit in kDiagThreads)
      const int r = lo + tid;
      if (r < hi) {
        cx<R> acc = {0, 0};
#pragma unroll
        for (int c = 0; c < kP; ++c)
          if (c < nb) acc += pre[c] * sx[s0 + c];
#pragma unroll
        for (int c = kP; c < 32; ++c)
          if (c < nb) acc += ld<R>(M.a, (r0 + r) + (r0 + s0 + c) * lda) * sx[s0 + c];
        sx[r] -= acc;
      }
    } else {
      // op(A)[r, s0 + c] = conj(A[s0 + c, r]): lanes along c, 4 rows per warp pass
      const cx<R> xv = lane < nb ? sx[s0 + lane] : cx<R>{0, 0};
#pragma unroll
      for (int q = 0; q < kPre; ++q) {
        const cx<R> av =
            q < kP ? pre[q < kP ? q : 0]
                   : [&] {
                       const int rr = lo + warp * 4 + (q & 3) + (q >> 2) * (kDiagThreads / 32) * 4;
                       return (rr < hi && lane < nb) ? ld<R>(M.a, (r0 + s0 + lane) + (r0 + rr) * lda)
                                                     : cx<R>{0, 0};
                     }();
        cx<R> t = cconj(av) * xv;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          t.x += __shfl_xor_sync(0xffffffffu, t.x, o);
          t.y += __shfl_xor_sync(0xffffffffu, t.y, o);
        }
        const int r = lo + warp * 4 + (q & 3) + (q >> 2) * (kDiagThreads / 32) * 4;
        if (lane == 0 && r < hi) sx[r] -= t;
      }
    }
    __syncthreads();
  }
  for (int i = tid; i < nbs; i += kDiagThreads) st<R>(M.x, off + r0 + i, sx[i]);
}

// Rows outside the solved block [r0, r0 + kBigB): x_r -= sum_c op(A)[r, c] x_c, one
// thread per row, the block's solution in shared memory (op(A) = A, coalesced along r).
// RG right-hand sides per CTA share every matrix element a thread loads, so a sweep's
// many right-hand sides read the factor once per group instead of once each.
template <typename R, int RG>
constexpr size_t upd_smem_bytes() {
  return sizeof(cx<R>) * (size_t)RG * kBigB;
}

// Rows [lo, hi) (absolute, clamped to the instance: beyond its block for the lower solve,
// before it for the upper one) are updated from the solution of block [r0, r0 + kBigB).
template <typename R, bool EFF_LOWER, bool TRANS, int RG>
__global__ void __launch_bounds__(256) k_trsv_big_update(const MatInst* __restrict__ insts,
                                                         int64_t r0, int64_t lo, int64_t hi) {
  const MatInst& M = insts[blockIdx.z];
  const int rg0 = blockIdx.y * RG;
  const int64_t n = M.n;
  if (!M.active || rg0 >= M.nrhs || r0 >= n) return;
  const int nr = min(RG, M.nrhs - rg0);
  const int nbs = (int)min((int64_t)kBigB, n - r0);
  const int64_t lda = M.lda, ldx = M.ldx;
  extern __shared__ __align__(16) unsigned char upd_smem[];
  cx<R>* sx = reinterpret_cast<cx<R>*>(upd_smem);  // [RG][kBigB]
  for (int r = 0; r < nr; ++r)
    for (int i = threadIdx.x; i < nbs; i += blockDim.x)
      sx[r * kBigB + i] = ld<R>(M.x, (int64_t)(rg0 + r) * ldx + r0 + i);
  __syncthreads();
  const int64_t row = lo + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= hi || (EFF_LOWER ? (row < r0 + nbs || row >= n) : row >= r0)) return;
  cx<R> acc[RG];
#pragma unroll
  for (int r = 0; r < RG; ++r) acc[r] = cx<R>{0, 0};
  for (int c0 = 0; c0 < nbs; c0 += 8) {
    cx<R> lv[8];
#pragma unroll
    for (int c = 0; c < 8; ++c)
      lv[c] = (c0 + c < nbs) ? opel<R, TRANS>(M.a, lda, row, r0 + c0 + c) : cx<R>{0, 0};
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      if (c0 + c < nbs) {
#pragma unroll
        for (int r = 0; r < RG; ++r)
          if (r < nr) acc[r] += lv[c] * sx[r * kBigB + c0 + c];
      }
    }
  }
#pragma unroll
  for (int r = 0; r < RG; ++r) {
    if (r < nr) {
      const int64_t o = (int64_t)(rg0 + r) * ldx + row;
      st<R>(M.x, o, ld<R>(M.x, o) - acc[r]);
    }
  }
}

// The same update for op(A) = A^H: x_r -= sum_c conj(A[c, r]) x_c reads column r of A,
// so a warp takes 4 rows with its lanes along c (coalesced), then reduces by shuffles.
constexpr int kTrUpRows = 32;  // rows per 256-thread CTA (8 warps x 4)
template <typename R, bool EFF_LOWER, int RG>
__global__ void __launch_bounds__(256) k_trsv_big_update_h(const MatInst* __restrict__ insts,
                                                           int64_t r0, int64_t lo, int64_t hi) {
  const MatInst& M = insts[blockIdx.z];
  const int rg0 = blockIdx.y * RG;
  const int64_t n = M.n;
  if (!M.active || rg0 >= M.nrhs || r0 >= n) return;
  const int nr = min(RG, M.nrhs - rg0);
  const int nbs = (int)min((int64_t)kBigB, n - r0);
  const int64_t lda = M.lda, ldx = M.ldx;
  extern __shared__ __align__(16) unsigned char upd_smem[];
  cx<R>* sx = reinterpret_cast<cx<R>*>(upd_smem);  // [RG][kBigB]
  for (int r = 0; r < nr; ++r)
    for (int i = threadIdx.x; i < nbs; i += blockDim.x)
      sx[r * kBigB + i] = ld<R>(M.x, (int64_t)(rg0 + r) * ldx + r0 + i);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t row0 = lo + (int64_t)blockIdx.x * kTrUpRows + warp * 4;
  const int64_t lim = min(hi, EFF_LOWER ? n : r0);
  if (row0 >= lim || (EFF_LOWER && row0 < r0 + nbs)) return;  // lo is a multiple of 4 rows
  cx<R> acc[4][RG];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int r = 0; r < RG; ++r) acc[u][r] = cx<R>{0, 0};
  for (int c = lane; c < nbs; c += 32) {
    cx<R> v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
      v[u] = (row0 + u < lim) ? cconj(ld<R>(M.a, (r0 + c) + (row0 + u) * lda)) : cx<R>{0, 0};
#pragma unroll
    for (int r = 0; r < RG; ++r) {
      if (r < nr) {
        const cx<R> xv = sx[r * kBigB + c];
#pragma unroll
        for (int u = 0; u < 4; ++u) acc[u][r] += v[u] * xv;
      }
    }
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
#pragma unroll
    for (int r = 0; r < RG; ++r) {
      if (r < nr) {
        cx<R> t = acc[u][r];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          t.x += __shfl_xor_sync(0xffffffffu, t.x, o);
          t.y += __shfl_xor_sync(0xffffffffu, t.y, o);
        }
        if (lane == 0 && row0 + u < lim) {
          const int64_t o2 = (int64_t)(rg0 + r) * ldx + row0 + u;
          st<R>(M.x, o2, ld<R>(M.x, o2) - t);
        }
      }
    }
  }
}

// x[i] = y[perm[i]] (forward interchanges as one gather; y holds a copy of x)
template <typename R>
__global__ void k_gather_perm(const MatInst* __restrict__ insts) {
  const MatInst& M = insts[blockIdx.z];
  const int rhs = blockIdx.y;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (!M.active || rhs >= M.nrhs || i >= M.n) return;
  const int64_t off = (int64_t)rhs * M.ldx;
  st<R>(M.x, off + i, ld<R>(M.y, off + M.perm[i]));
}

// (P^T w): x[perm[i]] = y[i] for every stream, then the caller's x holds the result.
template <typename R>
__global__ void k_scatter_perm(const MatInst* __restrict__ insts, int max_rhs) {
  const MatInst& M = insts[blockIdx.z];
  const int rhs = blockIdx.y;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (!M.active || rhs >= M.nrhs || i >= M.n) return;
  const int64_t off = (int64_t)rhs * M.ldx;
  st<R>(M.x, off + M.perm[i], ld<R>(M.y, off + i));
}

// x -> y copy (both ld ldx)
template <typename R>
__global__ void k_copy_xy(const MatInst* __restrict__ insts, int to_y) {
  const MatInst& M = insts[blockIdx.z];
  const int rhs = blockIdx.y;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (!M.active || rhs >= M.nrhs || i >= M.n) return;
  const int64_t off = (int64_t)rhs * M.ldx;
  if (to_y)
    st<R>(M.y, off + i, ld<R>(M.x, off + i));
  else
    st<R>(M.x, off + i, ld<R>(M.y, off + i));
}

// perm from LAPACK pivots: apply the interchanges in order to the identity, in shared
// memory (SMEM, orders up to the shared-memory capacity) or in place in global memory.
template <bool SMEM>
__global__ void __launch_bounds__(256) k_make_perm(const MatInst* __restrict__ insts) {
  const MatInst& M = insts[blockIdx.x];
  if (!M.active || !M.perm) return;
  extern __shared__ int32_t sperm_smem[];
  int32_t* sperm = SMEM ? sperm_smem : M.perm;
  const int64_t n = M.n;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) sperm[i] = (int32_t)i;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int64_t i = 0; i < n; ++i) {
      const int32_t p = M.ipiv[i];
      const int32_t t = sperm[i];
      sperm[i] = sperm[p];
      sperm[p] = t;
    }
  __syncthreads();
  if (SMEM)
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) M.perm[i] = sperm[i];
}

// ------------------------------------------------------------------ launch wrappers
static int prec_is_single(int prec) { return prec == 1; }

// CTAs per instance of the left-looking panel kernel: as many as keep the batch on the
// SMs in one wave (a power of two, 2..8: the portable cluster limit).
static int getf2_cluster(int ninst) {
  const int sms = device_sm_count();
  int cs = 2;
  while (cs < 8 && (int64_t)ninst * cs * 2 <= sms) cs *= 2;
  return cs;
}

// complex64: 1024 threads, 16 L values in flight per row; complex128: 512 threads and 8
// (the 64-register budget of 1024 threads would spill the FP64 values)
template <typename R>
struct LLCfg {
  static constexpr int kT = sizeof(R) == 4 ? kGetf2T : kGetf2T / 2;
  static constexpr int kBatch = sizeof(R) == 4 ? kLLBatch : kLLBatch / 2;
};

template <typename R, int CS>
static void getf2_ll_t(const Launch& L, const MatInst* d, int ninst, int64_t k0, int nb) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(ninst * CS));
  cfg.blockDim = dim3(LLCfg<R>::kT);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = L.stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CS;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_getf2_ll<R, CS, LLCfg<R>::kT, LLCfg<R>::kBatch>, d, k0, nb);
}

void launch_getf2(const Launch& L, const MatInst* d, int ninst, int64_t k0, int nb, int prec,
                  int cs) {
  // left-looking, one thread-block cluster per instance
  const int csel = cs > 0 ? cs : getf2_cluster(ninst);
  if (prec_is_single(prec)) {
    switch (csel) {
      case 8: getf2_ll_t<float, 8>(L, d, ninst, k0, nb); break;
      case 4: getf2_ll_t<float, 4>(L, d, ninst, k0, nb); break;
      default: getf2_ll_t<float, 2>(L, d, ninst, k0, nb); break;
    }
  } else {
    switch (csel) {
      case 8: getf2_ll_t<double, 8>(L, d, ninst, k0, nb); break;
      case 4: getf2_ll_t<double, 4>(L, d, ninst, k0, nb); break;
      default: getf2_ll_t<double, 2>(L, d, ninst, k0, nb); break;
    }
  }
  count_launch(1);
}

void launch_laswp(const Launch& L, const MatInst* d, int ninst, int64_t k0, int nb, int64_t c_lo,
                  int64_t c_hi, int64_t s_lo, int64_t s_hi, int prec) {
  const int64_t cols = (c_hi - c_lo) - (s_hi - s_lo);
  if (cols <= 0) return;
  dim3 grid((unsigned)((cols + kSwpCols - 1) / kSwpCols), (unsigned)ninst);
  for (int b0 = 0; b0 < nb; b0 += kSwpMaxNb) {  // sequential chunks of interchanges
    const int nbc = std::min(kSwpMaxNb, nb - b0);
    if (prec_is_single(prec))
      k_laswp<float><<<grid, kSwpWarps * 32, 0, L.stream>>>(d, k0 + b0, nbc, c_lo, c_hi, s_lo,
                                                              s_hi);
    else
      k_laswp<double><<<grid, kSwpWarps * 32, 0, L.stream>>>(d, k0 + b0, nbc, c_lo, c_hi, s_lo,
                                                               s_hi);
    count_launch(1);
  }
}

template <typename R, int NB>
static void trsm_t(const Launch& L, const MatInst* d, int ninst, int64_t k0, int64_t c_lo,
                   int64_t c_hi) {
  const size_t smem = (size_t)NB * (NB + 1) * sizeof(cx<R>);
  static PerDeviceOnce attr;
  if (smem > 48 * 1024)
    attr.call([&] {
      cudaFuncSetAttribute(k_trsm_panel<R, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem);
    });
  const int64_t per = (int64_t)kTrsmWarps * TrsmCols<R>::value;
  dim3 grid((unsigned)((c_hi - c_lo + per - 1) / per), (unsigned)ninst);
  k_trsm_panel<R, NB><<<grid, kTrsmWarps * 32, smem, L.stream>>>(d, k0, c_lo, c_hi);
  count_launch(1);
}

void launch_trsm_panel(const Launch& L, const MatInst* d, int ninst, int64_t k0, int nb,
                       int64_t c_lo, int64_t c_hi, int prec) {
  if (c_hi <= c_lo) return;
  if (nb <= 32) {
    if (prec_is_single(prec))
      trsm_t<float, 32>(L, d, ninst, k0, c_lo, c_hi);
    else
      trsm_t<double, 32>(L, d, ninst, k0, c_lo, c_hi);
  } else {
    if (prec_is_single(prec))
      trsm_t<float, 128>(L, d, ninst, k0, c_lo, c_hi);
    else
      trsm_t<double, 128>(L, d, ninst, k0, c_lo, c_hi);
  }
}

void launch_gemm_update(const Launch& L, const MatInst* d, int ninst, int64_t k0, int nb,
                        int64_t nmax, int64_t c_lo, int64_t c_hi, int prec) {
  const int64_t m = nmax - k0 - nb;
  const int64_t w = c_hi - c_lo;
  if (m <= 0 || w <= 0) return;
  const int64_t tiles = ((m + kGT - 1) / kGT) * ((w + kGT - 1) / kGT);
  dim3 grid((unsigned)tiles, (unsigned)ninst);
  if (prec_is_single(prec))
    k_gemm_update<float><<<grid, kGThreads, 0, L.stream>>>(d, k0, nb, c_lo, c_hi);
  else
    k_gemm_update<double><<<grid, kGThreads, 0, L.stream>>>(d, k0, nb, c_lo, c_hi);
  count_launch(1);
}

void launch_rhs_swap(const Launch& L, const MatInst* d, int ninst, int32_t max_rhs, int reverse,
                     int prec) {
  dim3 grid((unsigned)((max_rhs + 63) / 64), (unsigned)ninst);
  if (prec_is_single(prec))
    k_rhs_swap<float><<<grid, 64, 0, L.stream>>>(d, reverse);
  else
    k_rhs_swap<double><<<grid, 64, 0, L.stream>>>(d, reverse);
  count_launch(1);
}

template <typename R, bool EL, bool TR, bool UN>
static void trsv_t(const Launch& L, const MatInst* d, int ninst, int64_t nmax, int32_t max_rhs) {
  const int64_t nblk = (nmax + kTrsvNB - 1) / kTrsvNB;
  for (int64_t b = 0; b < nblk; ++b) {
    const int64_t blk = EL ? b : nblk - 1 - b;
    const int64_t r0 = blk * kTrsvNB;
    k_trsv_block<R, EL, TR, UN><<<dim3((unsigned)max_rhs, (unsigned)ninst), kTrsvNB, 0,
                                  L.stream>>>(d, r0); count_launch(1);
    const int64_t rows = EL ? (nmax - r0 - kTrsvNB) : r0;
    if (rows > 0) {
      k_trsv_update<R, EL, TR><<<dim3((unsigned)((rows + 255) / 256), (unsigned)max_rhs,
                                      (unsigned)ninst),
                                 256, 0, L.stream>>>(d, r0);
      count_launch(1);
    }
  }
}

template <typename R, bool EL, bool TR, bool UN>
static void trsv_big_t(const Launch& L, const MatInst* d, int ninst, int64_t nmax,
                       int32_t max_rhs) {
  constexpr size_t smem = diag_smem_bytes<R>();
  static PerDeviceOnce attr;
  attr.call([&] {
    cudaFuncSetAttribute(k_trsv_diag<R, EL, TR, UN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
  });
  // right-hand sides per update CTA: one, or a group sharing the matrix loads
  constexpr int RG = sizeof(R) == 4 ? 8 : 4;
  static PerDeviceOnce uattr;
  uattr.call([] {
    cudaFuncSetAttribute(k_trsv_big_update<R, EL, TR, RG>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)upd_smem_bytes<R, RG>());
    cudaFuncSetAttribute(k_trsv_big_update_h<R, EL, RG>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)upd_smem_bytes<R, RG>());
  });
  const int64_t nblk = (nmax + kBigB - 1) / kBigB;
  const unsigned gy = max_rhs >= 4 ? (unsigned)((max_rhs + RG - 1) / RG) : (unsigned)max_rhs;
  auto diag = [&](cudaStream_t s, int64_t r0) {
    k_trsv_diag<R, EL, TR, UN><<<dim3((unsigned)max_rhs, (unsigned)ninst), kDiagThreads, smem, s>>>(
        d, r0);
    count_launch(1);
  };
  auto update = [&](cudaStream_t s, int64_t r0, int64_t lo, int64_t hi) {  // rows [lo, hi)
    if (hi <= lo) return;
    const int64_t rows = hi - lo;
    if (TR) {
      const dim3 g((unsigned)((rows + kTrUpRows - 1) / kTrUpRows), gy, (unsigned)ninst);
      if (max_rhs >= 4)
        k_trsv_big_update_h<R, EL, RG><<<g, 256, upd_smem_bytes<R, RG>(), s>>>(d, r0, lo, hi);
      else
        k_trsv_big_update_h<R, EL, 1><<<g, 256, upd_smem_bytes<R, 1>(), s>>>(d, r0, lo, hi);
    } else {
      const dim3 g((unsigned)((rows + 255) / 256), gy, (unsigned)ninst);
      if (max_rhs >= 4)
        k_trsv_big_update<R, EL, TR, RG><<<g, 256, upd_smem_bytes<R, RG>(), s>>>(d, r0, lo, hi);
      else
        k_trsv_big_update<R, EL, TR, 1><<<g, 256, upd_smem_bytes<R, 1>(), s>>>(d, r0, lo, hi);
    }
    count_launch(1);
  };
  auto block_row = [&](int64_t b) { return (EL ? b : nblk - 1 - b) * kBigB; };
  if (!L.side || nblk < 3 || L.n_events < 2 * (int)nblk + 1) {
    for (int64_t b = 0; b < nblk; ++b) {
      const int64_t r0 = block_row(b);
      diag(L.stream, r0);
      if (EL)
        update(L.stream, r0, r0 + kBigB, nmax);
      else
        update(L.stream, r0, 0, r0);
    }
    return;
  }
  // Look-ahead: the main stream updates only the next block's rows and solves that block
  // while the side stream updates every later row from the same solved block.  Both write
  // x by read-modify-write, so the main stream's next-block update waits for the side
  // stream's previous update (which also covered those rows), and the side stream's update
  // waits for the block it reads.
  cudaEvent_t* ev = L.events;
  cudaEventRecord(ev[0], L.stream);  // the side stream starts after the main stream's work
  cudaStreamWaitEvent(L.side, ev[0], 0);
  diag(L.stream, block_row(0));
  for (int64_t b = 0; b < nblk; ++b) {
    const int64_t r0 = block_row(b);
    cudaEvent_t e_diag = ev[1 + 2 * b], e_big = ev[2 + 2 * b];
    cudaEventRecord(e_diag, L.stream);
    if (b + 1 < nblk) {
      const int64_t rn = block_row(b + 1);  // the next block in solve order
      if (b > 0) cudaStreamWaitEvent(L.stream, ev[2 + 2 * (b - 1)], 0);
      update(L.stream, r0, rn, rn + kBigB);
      diag(L.stream, rn);
    }
    cudaStreamWaitEvent(L.side, e_diag, 0);
    if (EL)
      update(L.side, r0, r0 + 2 * kBigB, nmax);
    else
      update(L.side, r0, 0, r0 - kBigB);
    cudaEventRecord(e_big, L.side);
  }
  cudaStreamWaitEvent(L.stream, ev[2 + 2 * (nblk - 1)], 0);  // join before returning
}

template <typename R>
static void getrs_big_t(const Launch& L, const MatInst* d, int ninst, int64_t nmax,
                        int32_t max_rhs, int trans, int swaps) {
  dim3 g((unsigned)((nmax + 255) / 256), (unsigned)max_rhs, (unsigned)ninst);
  if (!trans) {
    if (swaps) {
      k_copy_xy<R><<<g, 256, 0, L.stream>>>(d, 1);
      k_gather_perm<R><<<g, 256, 0, L.stream>>>(d);
      count_launch(2);
    }
    trsv_big_t<R, true, false, true>(L, d, ninst, nmax, max_rhs);
    trsv_big_t<R, false, false, false>(L, d, ninst, nmax, max_rhs);
  } else {
    trsv_big_t<R, true, true, false>(L, d, ninst, nmax, max_rhs);
    trsv_big_t<R, false, true, true>(L, d, ninst, nmax, max_rhs);
    if (swaps) {
      k_copy_xy<R><<<g, 256, 0, L.stream>>>(d, 1);
      k_scatter_perm<R><<<g, 256, 0, L.stream>>>(d, max_rhs);
      count_launch(2);
    }
  }
}

void launch_make_perm(const Launch& L, const MatInst* d, int ninst, int64_t nmax) {
  constexpr size_t kMaxSmem = 227 * 1024;
  const size_t smem = (size_t)nmax * sizeof(int32_t);
  if (smem > kMaxSmem) {  // beyond 58112 unknowns: interchanges in global memory
    k_make_perm<false><<<ninst, 256, 0, L.stream>>>(d);
    count_launch(1);
    return;
  }
  static PerDeviceOnce attr;
  attr.call([] {
    cudaFuncSetAttribute(k_make_perm<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kMaxSmem);
  });
  k_make_perm<true><<<ninst, 256, smem, L.stream>>>(d);
  count_launch(1);
}

// Solve op(LU) x = b in place on MatInst.x.  trans = 0: A x = b; trans = 1: A^H x = b.
// swaps = 0 leaves out the row interchanges (the (LU)^{-1} and (LU)^{-H} products that
// LAPACK's condition estimator applies).
void launch_getrs(const Launch& L, const MatInst* d, int ninst, int64_t nmax, int32_t max_rhs,
                  int trans, int prec, int swaps, const TrsvWork* work) {
  if (nmax <= 0 || ninst <= 0 || max_rhs <= 0) return;
  if (work) {  // blocked two-level solve; needs MatInst.y and MatInst.perm
    if (prec_is_single(prec))
      getrs_big_t<float>(L, d, ninst, nmax, max_rhs, trans, swaps);
    else
      getrs_big_t<double>(L, d, ninst, nmax, max_rhs, trans, swaps);
    return;
  }
  if (nmax <= trsv_full_max(prec)) {
    const bool sp = prec_is_single(prec);
    if (!trans) {
      if (sp) {
        if (swaps)
          trsv_full_t<float, true, false, true, 1>(L, d, ninst, nmax, max_rhs);
        else
          trsv_full_t<float, true, false, true, 0>(L, d, ninst, nmax, max_rhs);
        trsv_full_t<float, false, false, false, 0>(L, d, ninst, nmax, max_rhs);
      } else {
        if (swaps)
          trsv_full_t<double, true, false, true, 1>(L, d, ninst, nmax, max_rhs);
        else
          trsv_full_t<double, true, false, true, 0>(L, d, ninst, nmax, max_rhs);
        trsv_full_t<double, false, false, false, 0>(L, d, ninst, nmax, max_rhs);
      }
    } else {
      if (sp) {
        trsv_full_t<float, true, true, false, 0>(L, d, ninst, nmax, max_rhs);
        if (swaps)
          trsv_full_t<float, false, true, true, 2>(L, d, ninst, nmax, max_rhs);
        else
          trsv_full_t<float, false, true, true, 0>(L, d, ninst, nmax, max_rhs);
      } else {
        trsv_full_t<double, true, true, false, 0>(L, d, ninst, nmax, max_rhs);
        if (swaps)
          trsv_full_t<double, false, true, true, 2>(L, d, ninst, nmax, max_rhs);
        else
          trsv_full_t<double, false, true, true, 0>(L, d, ninst, nmax, max_rhs);
      }
    }
    return;
  }
  if (!trans) {
    if (swaps) launch_rhs_swap(L, d, ninst, max_rhs, 0, prec);
    if (prec_is_single(prec)) {
      trsv_t<float, true, false, true>(L, d, ninst, nmax, max_rhs);
      trsv_t<float, false, false, false>(L, d, ninst, nmax, max_rhs);
    } else {
      trsv_t<double, true, false, true>(L, d, ninst, nmax, max_rhs);
      trsv_t<double, false, false, false>(L, d, ninst, nmax, max_rhs);
    }
  } else {
    // A^H = U^H L^H P: solve U^H (lower, non-unit), then L^H (upper, unit), then P^T.
    if (prec_is_single(prec)) {
      trsv_t<float, true, true, false>(L, d, ninst, nmax, max_rhs);
      trsv_t<float, false, true, true>(L, d, ninst, nmax, max_rhs);
    } else {
      trsv_t<double, true, true, false>(L, d, ninst, nmax, max_rhs);
      trsv_t<double, false, true, true>(L, d, ninst, nmax, max_rhs);
    }
    if (swaps) launch_rhs_swap(L, d, ninst, max_rhs, 1, prec);
  }
}

// Full SIMT LU of a batch (used by the complex128 path and by the complex64 path when
// the tensor-core trailing update is not selected).
void launch_getrf_simt(const Launch& L, const MatInst* d, int ninst, int64_t nmax, int prec) {
  for (int64_t k0 = 0; k0 < nmax; k0 += kPanelNB) {
    launch_getf2(L, d, ninst, k0, kPanelNB, prec);
    launch_laswp(L, d, ninst, k0, kPanelNB, 0, nmax, k0, k0 + kPanelNB, prec);
    launch_trsm_panel(L, d, ninst, k0, kPanelNB, k0 + kPanelNB, nmax, prec);
    launch_gemm_update(L, d, ninst, k0, kPanelNB, nmax, k0 + kPanelNB, nmax, prec);
  }
}

}  // namespace bemgpu
