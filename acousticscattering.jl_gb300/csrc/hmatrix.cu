// Hierarchical-matrix operators and batched restarted GMRES on the device.
//
// Compressed operators (the reference's compression=(method=:hmatrix, tol) of
// solvers/bem/full.jl:89-97, which builds Inti operators compressed by HMatrices.jl):
//  * admissible blocks: adaptive cross approximation with partial pivoting, one CTA per
//    block, the matrix entries evaluated on demand by the same regular 7-point rule as
//    the dense assembly (admissible blocks hold no near pair, so the regular rule is the
//    entry), stopped when |u_r| |v_r| <= tol |S_r|_F with the Frobenius norm of the
//    running approximation updated exactly from the projections of the new cross;
//  * full leaf blocks: the regular kernel here, then the near-pair kernel of the dense
//    assembly writing into block storage (AsmInst.near_dst);
//  * products: coefficients V^T x of every admissible block (one warp per rank column),
//    then one CTA per row leaf that sums, in the fixed order of its block list, the full
//    blocks and the U (V^T x) terms covering its rows.  No atomics: every output element
//    has one writer and a fixed summation order.
// GMRES (IterativeSolvers.gmres as called by solvers/bem/full.jl:153-154: x0 = 0,
// stopping when the residual estimate <= max(reltol |b|, abstol), restart and maxiter in
// Arnoldi steps): classical Gram-Schmidt with one reorthogonalisation (CGS2: the same
// Krylov basis as modified Gram-Schmidt up to rounding, with the projections as
// parallel dot products), complex Givens rotations, an explicit residual at each restart.
// Right-hand sides iterate in lock step; one that converges is frozen by its state word,
// so its iterates do not depend on the others.
#include <type_traits>

#include "hmatrix.cuh"
#include "quad_math.cuh"
#include "quad_regular.cuh"

namespace bemgpu {

namespace {

__device__ __forceinline__ cd ldc(const double* p, int64_t i) {
  const double2 v = reinterpret_cast<const double2*>(p)[i];
  return cd{v.x, v.y};
}
__device__ __forceinline__ void stc(double* p, int64_t i, cd v) {
  reinterpret_cast<double2*>(p)[i] = make_double2(v.x, v.y);
}
// conj(a) b
__device__ __forceinline__ cd conjmul(cd a, cd b) {
  return cd{a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double abs2(cd a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ cd cdiv_real(cd a, double s) { return cd{a.x / s, a.y / s}; }
__device__ __forceinline__ cd crecip(cd a) {
  const double d = a.x * a.x + a.y * a.y;
  return cd{a.x / d, -a.y / d};
}
__device__ __forceinline__ cd warp_sum(cd v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, off);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, off);
  }
  return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}
template <typename V>
__device__ __forceinline__ void amax(V& v, int32_t& i, V ov, int32_t oi) {
  if (ov > v || (ov == v && oi < i)) {
    v = ov;
    i = oi;
  }
}

// Entry (i, j) of M1 (op 0) or M2 (op 1) of a rigid/soft assembly kind at panels pi != pj
// by the regular rule in precision R (FP32 on the records relative to the mesh centre, as
// the dense mixed-precision assembly), combined as in the dense regular kernel.
template <typename R, int KIND, int OP>
__device__ __forceinline__ cx<R> hm_entry(const R* __restrict__ recs, int32_t pi, int32_t pj,
                                          R k, cx<R> al) {
  constexpr int kRec = Prec<R>::kRec;
  const R* ri = recs + (int64_t)pi * kRec;
  const R x[3] = {ri[0], ri[1], ri[2]}, nx[3] = {ri[3], ri[4], ri[5]};
  Acc<R> a;
  a.S = a.D = a.K = a.H = cx<R>{0, 0};
  regular_panel<R, KIND == kAsmBM>(recs + (int64_t)pj * kRec, x, nx, k, a);
  if (OP == 0) {
    cx<R> m1 = cx<R>{-a.D.x, -a.D.y};
    if (KIND == kAsmBM) m1 -= al * a.H;
    return m1;
  }
  cx<R> m2 = a.S;
  if (KIND == kAsmBM) m2 += al * a.K;
  return m2;
}

template <typename R>
__device__ __forceinline__ cx<R> cconjmul(cx<R> a, cx<R> b) {  // conj(a) b
  return cx<R>{a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x};
}
template <typename R>
__device__ __forceinline__ cx<R> cwarp_sum(cx<R> v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, off);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, off);
  }
  return v;
}
template <typename R>
__device__ __forceinline__ cx<R> to(cd v) {
  return cx<R>{(R)v.x, (R)v.y};
}
// element i of a vector held in the operator's precision (complex128 or complex64)
template <typename R>
__device__ __forceinline__ cx<R> ldv(const void* p, int64_t i) {
  return static_cast<const cx<R>*>(p)[i];
}

constexpr int kAcaT = 256;
constexpr int kAcaW = kAcaT / 32;

// block-wide argmax over NW warps (largest value, then smallest index); every thread gets
// the result
template <int NW, typename V>
__device__ __forceinline__ void block_argmax(V& v, int32_t& i, V* rv, int32_t* ri) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const V ov = __shfl_xor_sync(0xffffffffu, v, off);
    const int32_t oi = __shfl_xor_sync(0xffffffffu, i, off);
    amax(v, i, ov, oi);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) {
    rv[w] = v;
    ri[w] = i;
  }
  __syncthreads();
  v = rv[0];
  i = ri[0];
  for (int q = 1; q < NW; ++q) amax(v, i, rv[q], ri[q]);
}

}  // namespace

// ------------------------------------------------------------------ cross approximation
// NT threads per CTA (512 for the largest blocks, whose serial rank steps set the
// kernel's duration; 256 otherwise); list: the blocks of this launch.
template <typename R, int KIND, int OP, int NT>
__global__ void __launch_bounds__(NT) k_hm_aca(HmLR* __restrict__ lrs,
                                              const int32_t* __restrict__ list, void* Up,
                                              void* Vp, const R* __restrict__ recs,
                                              const int32_t* __restrict__ perm, double k_,
                                              double a_re, double a_im, double tol) {
  using C = cx<R>;
  constexpr int NW = NT / 32;
  HmLR& B = lrs[list[blockIdx.x]];
  const int m = B.m, n = B.n, kmax = B.kmax;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  C* U = static_cast<C*>(Up) + B.uoff;
  C* V = static_cast<C*>(Vp) + B.voff;
  const int32_t* prow = perm + B.rlo;
  const int32_t* pcol = perm + B.clo;
  const C al = {(R)a_re, (R)a_im};
  const R k = (R)k_;
  extern __shared__ uint32_t used[];  // pivot rows taken, (m + 31) / 32 words
  __shared__ R rv[NW];
  __shared__ int32_t ri[NW];
  __shared__ C su[kHmMaxRank], sv[kHmMaxRank];    // U[i*, l], V[j*, l]
  __shared__ C cu[kHmMaxRank], cv[kHmMaxRank];    // projections of the new cross
  __shared__ C s_piv;
  __shared__ double s_s2;
  __shared__ int s_stop;
  const int words = (m + 31) >> 5;
  for (int w = tid; w < words; w += NT) used[w] = 0u;
  if (tid == 0) s_s2 = 0.0;
  int rank = 0, conv = 0;
  int32_t istar = 0;
  __syncthreads();
  for (int it = 0; rank < kmax && it < m; ++it) {
    if (tid < rank) su[tid] = U[istar + (int64_t)tid * m];
    if (tid == 0) used[istar >> 5] |= 1u << (istar & 31);
    __syncthreads();
    // residual row i*: A[i*, :] - sum_l U[i*, l] V[:, l]
    R bv = -1;
    int32_t bj = INT32_MAX;
    const int32_t pi = prow[istar];
    for (int j = tid; j < n; j += NT) {
      C v = hm_entry<R, KIND, OP>(recs, pi, pcol[j], k, al);
      for (int l = 0; l < rank; ++l) v -= su[l] * V[j + (int64_t)l * n];
      V[j + (int64_t)rank * n] = v;
      amax(bv, bj, v.x * v.x + v.y * v.y, j);
    }
    block_argmax<NW>(bv, bj, rv, ri);
    if (!(bv > 0)) {  // the residual row vanishes: continue from the next unused row
      R fv = -1;
      int32_t fi = INT32_MAX;
      for (int i = tid; i < m; i += NT)
        if (!((used[i >> 5] >> (i & 31)) & 1u)) {
          amax(fv, fi, (R)1, i);
          break;
        }
      block_argmax<NW>(fv, fi, rv, ri);
      if (fv < 0) {  // every row was a pivot row: the approximation is exact
        conv = 1;
        break;
      }
      istar = fi;
      continue;
    }
    const int32_t jstar = bj;
    if (tid == 0) s_piv = V[jstar + (int64_t)rank * n];
    if (tid < rank) sv[tid] = V[jstar + (int64_t)tid * n];
    __syncthreads();
    const R pd = s_piv.x * s_piv.x + s_piv.y * s_piv.y;
    const C inv = {s_piv.x / pd, -s_piv.y / pd};
    // residual column j*: A[:, j*] - sum_l U[:, l] V[j*, l]; next pivot row
    R cb = -1;
    int32_t ci = INT32_MAX;
    const int32_t pj = pcol[jstar];
    for (int i = tid; i < m; i += NT) {
      C u = hm_entry<R, KIND, OP>(recs, prow[i], pj, k, al);
      for (int l = 0; l < rank; ++l) u -= U[i + (int64_t)l * m] * sv[l];
      U[i + (int64_t)rank * m] = u;
      if (!((used[i >> 5] >> (i & 31)) & 1u)) amax(cb, ci, u.x * u.x + u.y * u.y, i);
    }
    for (int j = tid; j < n; j += NT) V[j + (int64_t)rank * n] = V[j + (int64_t)rank * n] * inv;
    __syncthreads();
    // projections U_l^H U_r and V_l^H V_r, l = 0..rank (one warp per l, fixed order)
    for (int l = wid; l <= rank; l += NW) {
      C a = {0, 0}, b = {0, 0};
      for (int i = lane; i < m; i += 32)
        a += cconjmul(U[i + (int64_t)l * m], U[i + (int64_t)rank * m]);
      for (int j = lane; j < n; j += 32)
        b += cconjmul(V[j + (int64_t)l * n], V[j + (int64_t)rank * n]);
      a = cwarp_sum(a);
      b = cwarp_sum(b);
      if (lane == 0) {
        cu[l] = a;
        cv[l] = b;
      }
    }
    block_argmax<NW>(cb, ci, rv, ri);
    if (tid == 0) {
      // |S_r|^2 = |S_{r-1}|^2 + |u_r|^2 |v_r|^2 + 2 Re sum_{l<r} (U_l^H u_r)(V_l^H v_r)
      const double uv2 = (double)cu[rank].x * (double)cv[rank].x;
      double s = s_s2 + uv2;
      for (int l = 0; l < rank; ++l)
        s += 2.0 * ((double)cu[l].x * cv[l].x - (double)cu[l].y * cv[l].y);
      s_s2 = s;
      s_stop = uv2 <= tol * tol * s ? 1 : 0;
    }
    __syncthreads();
    ++rank;
    if (s_stop || cb < 0) {  // converged, or every row was a pivot row (exact)
      conv = 1;
      break;
    }
    istar = ci;
  }
  if (tid == 0) {
    B.rank = rank;
    B.conv = conv;
  }
}

void launch_hm_aca(const Launch& L, HmLR* lr, const int32_t* normal, int32_t n_normal,
                   int32_t max_m, const int32_t* large, int32_t n_large, int32_t max_m_large,
                   void* U, void* V, const void* recs, bool f32, const int32_t* perm, int kind,
                   int op, double k, double a_re, double a_im, double tol) {
  // the large blocks' launch runs beside the others (on the side stream when there is one):
  // its few long CTAs are the critical path, the many short ones fill the GPU around them
  const bool two = L.side && L.n_events >= 2 && n_large > 0 && n_normal > 0;
  const cudaStream_t sl = two ? L.side : L.stream;
  if (two) {
    cudaEventRecord(L.events[0], L.stream);
    cudaStreamWaitEvent(L.side, L.events[0], 0);
  }
  auto go = [&](auto kern, auto kern_l, auto rec) {
    const size_t smem = (size_t)((max_m + 31) / 32) * 4;
    const size_t smem_l = (size_t)((max_m_large + 31) / 32) * 4;
    if (n_large > 0) {
      if (smem_l > 48 * 1024)
        cudaFuncSetAttribute(kern_l, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_l);
      kern_l<<<(unsigned)n_large, 2 * kAcaT, smem_l, sl>>>(lr, large, U, V, rec, perm, k, a_re,
                                                           a_im, tol);
      count_launch(1);
    }
    if (n_normal > 0) {
      if (smem > 48 * 1024)
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      kern<<<(unsigned)n_normal, kAcaT, smem, L.stream>>>(lr, normal, U, V, rec, perm, k, a_re,
                                                         a_im, tol);
      count_launch(1);
    }
  };
  const float* rf = static_cast<const float*>(recs);
  const double* rd = static_cast<const double*>(recs);
  constexpr int T1 = kAcaT, T2 = 2 * kAcaT;
  const int sel = (f32 ? 4 : 0) + (kind == kAsmBM ? 2 : 0) + op;
  switch (sel) {
    case 0: go(k_hm_aca<double, kAsmCBIE, 0, T1>, k_hm_aca<double, kAsmCBIE, 0, T2>, rd); break;
    case 1: go(k_hm_aca<double, kAsmCBIE, 1, T1>, k_hm_aca<double, kAsmCBIE, 1, T2>, rd); break;
    case 2: go(k_hm_aca<double, kAsmBM, 0, T1>, k_hm_aca<double, kAsmBM, 0, T2>, rd); break;
    case 3: go(k_hm_aca<double, kAsmBM, 1, T1>, k_hm_aca<double, kAsmBM, 1, T2>, rd); break;
    case 4: go(k_hm_aca<float, kAsmCBIE, 0, T1>, k_hm_aca<float, kAsmCBIE, 0, T2>, rf); break;
    case 5: go(k_hm_aca<float, kAsmCBIE, 1, T1>, k_hm_aca<float, kAsmCBIE, 1, T2>, rf); break;
    case 6: go(k_hm_aca<float, kAsmBM, 0, T1>, k_hm_aca<float, kAsmBM, 0, T2>, rf); break;
    default: go(k_hm_aca<float, kAsmBM, 1, T1>, k_hm_aca<float, kAsmBM, 1, T2>, rf); break;
  }
  if (two) {  // join
    cudaEventRecord(L.events[1], L.side);
    cudaStreamWaitEvent(L.stream, L.events[1], 0);
  }
}

// ------------------------------------------------------------------ pool compaction
__global__ void __launch_bounds__(256) k_hm_compact(const HmCopy* __restrict__ cp,
                                                    const uint2* __restrict__ src,
                                                    uint2* __restrict__ dst) {
  const HmCopy c = cp[blockIdx.x];
  for (int64_t w = threadIdx.x; w < c.words; w += blockDim.x) dst[c.dst + w] = src[c.src + w];
}

void launch_hm_compact(const Launch& L, const HmCopy* d, int32_t count, const void* src,
                       void* dst) {
  if (count <= 0) return;
  k_hm_compact<<<(unsigned)count, 256, 0, L.stream>>>(d, static_cast<const uint2*>(src),
                                                        static_cast<uint2*>(dst));
  count_launch(1);
}

// ------------------------------------------------------------------ full blocks
template <typename R, int KIND>
__global__ void __launch_bounds__(256) k_hm_dense(const HmDense* __restrict__ dn, void* D1,
                                                  void* D2, const R* __restrict__ recs,
                                                  const int32_t* __restrict__ perm, double k_,
                                                  double a_re, double a_im) {
  constexpr int kRec = Prec<R>::kRec;
  const HmDense B = dn[blockIdx.x];
  const int64_t cnt = (int64_t)B.m * B.n;
  const cx<R> al = {(R)a_re, (R)a_im};
  const R k = (R)k_;
  cx<R>* o1 = static_cast<cx<R>*>(D1) + B.off;
  cx<R>* o2 = static_cast<cx<R>*>(D2) + B.off;
  for (int64_t e = (int64_t)blockIdx.y * blockDim.x + threadIdx.x; e < cnt;
       e += (int64_t)blockDim.x * gridDim.y) {
    const int i = (int)(e % B.m), j = (int)(e / B.m);
    const int32_t pi = perm[B.rlo + i], pj = perm[B.clo + j];
    if (pi == pj) continue;  // self pair: near kernel
    const R* ri = recs + (int64_t)pi * kRec;
    const R x[3] = {ri[0], ri[1], ri[2]}, nx[3] = {ri[3], ri[4], ri[5]};
    Acc<R> a;
    a.S = a.D = a.K = a.H = cx<R>{0, 0};
    regular_panel<R, KIND == kAsmBM>(recs + (int64_t)pj * kRec, x, nx, k, a);
    cx<R> m1 = cx<R>{-a.D.x, -a.D.y}, m2 = a.S;
    if (KIND == kAsmBM) {
      m1 -= al * a.H;
      m2 += al * a.K;
    }
    o1[e] = m1;
    o2[e] = m2;
  }
}

void launch_hm_dense(const Launch& L, const HmDense* dn, int32_t n_dense, void* D1, void* D2,
                     const void* recs, bool f32, const int32_t* perm, int kind, double k,
                     double a_re, double a_im) {
  if (n_dense <= 0) return;
  dim3 g((unsigned)n_dense, 4);
  const float* rf = static_cast<const float*>(recs);
  const double* rd = static_cast<const double*>(recs);
  if (f32) {
    if (kind == kAsmBM)
      k_hm_dense<float, kAsmBM><<<g, 256, 0, L.stream>>>(dn, D1, D2, rf, perm, k, a_re, a_im);
    else
      k_hm_dense<float, kAsmCBIE><<<g, 256, 0, L.stream>>>(dn, D1, D2, rf, perm, k, a_re, a_im);
  } else {
    if (kind == kAsmBM)
      k_hm_dense<double, kAsmBM><<<g, 256, 0, L.stream>>>(dn, D1, D2, rd, perm, k, a_re, a_im);
    else
      k_hm_dense<double, kAsmCBIE><<<g, 256, 0, L.stream>>>(dn, D1, D2, rd, perm, k, a_re, a_im);
  }
  count_launch(1);
}

// ------------------------------------------------------------------ products
// Operators stored in precision R (complex128 / complex64) are applied in that precision;
// the vectors stay complex128.
__device__ __forceinline__ bool rhs_on(const GmState* st, int r, int mode) {
  if (mode == 0 || !st) return true;
  return mode == 1 ? st[r].active != 0 : st[r].done == 0;
}

// Products over RB right-hand sides per CTA (each stored block element is read once for
// all of them); every right-hand side keeps the same summation order whatever RB is, so
// results do not depend on how many right-hand sides share a launch.
__device__ __forceinline__ bool group_on(const GmState* st, int r0, int rb, int nr, int mode) {
  for (int q = 0; q < rb && r0 + q < nr; ++q)
    if (rhs_on(st, r0 + q, mode)) return true;
  return false;
}

// Coefficients of one column chunk of a compressed block: T[toff + c kmax + l] =
// sum over the chunk of V[j, l] x[clo + j]; one warp per l, four independent accumulators
// per lane and right-hand side (added in a fixed order).
template <typename R, int RB>
__global__ void __launch_bounds__(256) k_hm_vt(HmOp A, const void* __restrict__ X, int64_t ldx,
                                               int32_t nr, const GmState* st, int mode,
                                               const int32_t* jptr, int64_t jstride) {
  using C = cx<R>;
  const int r0 = blockIdx.y * RB;
  if (!group_on(st, r0, RB, nr, mode)) return;
  if (jptr) X = static_cast<const C*>(X) + (int64_t)*jptr * jstride;
  const HmItem it = A.vt_items[blockIdx.x];
  const HmLR B = A.lr[it.blk];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const C* V = static_cast<const C*>(A.V) + B.voff;
  const C* x[RB];
#pragma unroll
  for (int q = 0; q < RB; ++q)
    x[q] = static_cast<const C*>(X) + (int64_t)min(r0 + q, nr - 1) * ldx + B.clo;
  const int j0 = it.lo, j1 = it.lo + it.cnt;
  for (int l = wid; l < B.rank; l += 8) {
    const C* v = V + (int64_t)l * B.n;
    C s[RB][4];
#pragma unroll
    for (int q = 0; q < RB; ++q) s[q][0] = s[q][1] = s[q][2] = s[q][3] = C{0, 0};
    int j = j0 + lane;
    for (; j + 96 < j1; j += 128) {
      const C v0 = v[j], v1 = v[j + 32], v2 = v[j + 64], v3 = v[j + 96];
#pragma unroll
      for (int q = 0; q < RB; ++q) {
        s[q][0] += v0 * x[q][j];
        s[q][1] += v1 * x[q][j + 32];
        s[q][2] += v2 * x[q][j + 64];
        s[q][3] += v3 * x[q][j + 96];
      }
    }
    for (; j < j1; j += 32) {
      const C v0 = v[j];
#pragma unroll
      for (int q = 0; q < RB; ++q) s[q][0] += v0 * x[q][j];
    }
#pragma unroll
    for (int q = 0; q < RB; ++q) {
      const C t = cwarp_sum(((s[q][0] + s[q][1]) + s[q][2]) + s[q][3]);
      if (lane == 0 && r0 + q < nr) {
        double* T = A.T + 2 * ((int64_t)(r0 + q) * A.tstride + B.toff + (int64_t)it.c * B.kmax);
        stc(T, l, cd{(double)t.x, (double)t.y});
      }
    }
  }
}

constexpr int kLeafRows = 64;
constexpr int kLeafSlices = 4;

// Partial rows of every full block: P[poff + i] = sum_j D[i, j] x[clo + j] (64 rows x 4
// column slices per pass, slices added in a fixed order), RB right-hand sides per CTA.
template <typename R, int RB>
__global__ void __launch_bounds__(kLeafRows * kLeafSlices) k_hm_dblk(
    HmOp A, const void* __restrict__ X, int64_t ldx, int32_t nr, const GmState* st, int mode,
    const int32_t* jptr, int64_t jstride) {
  using C = cx<R>;
  const int r0 = blockIdx.y * RB;
  if (!group_on(st, r0, RB, nr, mode)) return;
  if (jptr) X = static_cast<const C*>(X) + (int64_t)*jptr * jstride;
  const HmDense& B = A.dn[blockIdx.x];
  const int row = threadIdx.x % kLeafRows, s = threadIdx.x / kLeafRows;
  __shared__ C part[RB][kLeafSlices][kLeafRows];
  const C* D = static_cast<const C*>(A.D) + B.off;
  const C* x[RB];
#pragma unroll
  for (int q = 0; q < RB; ++q)
    x[q] = static_cast<const C*>(X) + (int64_t)min(r0 + q, nr - 1) * ldx + B.clo;
  auto store = [&](int i) {
#pragma unroll
    for (int q = 0; q < RB; ++q)
      if (r0 + q < nr)
        static_cast<C*>(A.P)[(int64_t)(r0 + q) * A.pstride + B.poff + i] =
            ((part[q][0][row] + part[q][1][row]) + part[q][2][row]) + part[q][3][row];
  };
  if (B.m == kLeafRows && B.n == kLeafRows) {  // leaf x leaf block: all loads in flight
    constexpr int kPer = kLeafRows / kLeafSlices;
    C d[kPer];
#pragma unroll
    for (int u = 0; u < kPer; ++u) d[u] = D[row + (int64_t)(s + u * kLeafSlices) * kLeafRows];
#pragma unroll
    for (int q = 0; q < RB; ++q) {
      C a = d[0] * x[q][s];
#pragma unroll
      for (int u = 1; u < kPer; ++u) a += d[u] * x[q][s + u * kLeafSlices];
      part[q][s][row] = a;
    }
    __syncthreads();
    if (s == 0) store(row);
    return;
  }
  for (int rr = 0; rr < B.m; rr += kLeafRows) {
    const int i = rr + row;
#pragma unroll
    for (int q = 0; q < RB; ++q) {
      C a0 = {0, 0}, a1 = {0, 0};
      if (i < B.m) {
        int j = s;
        for (; j + kLeafSlices < B.n; j += 2 * kLeafSlices) {
          a0 += D[i + (int64_t)j * B.m] * x[q][j];
          a1 += D[i + (int64_t)(j + kLeafSlices) * B.m] * x[q][j + kLeafSlices];
        }
        for (; j < B.n; j += kLeafSlices) a0 += D[i + (int64_t)j * B.m] * x[q][j];
      }
      part[q][s][row] = a0 + a1;
    }
    __syncthreads();
    if (s == 0 && i < B.m) store(i);
    __syncthreads();
  }
}

// Partial rows of one row chunk of a compressed block: P[poff + i] = sum_l U[i, l] t[l],
// t = the block's coefficient chunks added in order; RB right-hand sides per CTA.
template <typename R, int RB>
__global__ void __launch_bounds__(kHmRowChunk) k_hm_lblk(HmOp A, int32_t nr, const GmState* st,
                                                        int mode) {
  using C = cx<R>;
  const int r0 = blockIdx.y * RB;
  if (!group_on(st, r0, RB, nr, mode)) return;
  const HmItem it = A.lb_items[blockIdx.x];
  const HmLR B = A.lr[it.blk];
  __shared__ C t[RB][kHmMaxRank];
  if (threadIdx.x < B.rank) {
#pragma unroll
    for (int q = 0; q < RB; ++q) {
      const double* T = A.T + 2 * ((int64_t)min(r0 + q, nr - 1) * A.tstride + B.toff);
      cd v = ldc(T, threadIdx.x);
      for (int c = 1; c < B.nvc; ++c) v += ldc(T, (int64_t)c * B.kmax + threadIdx.x);
      t[q][threadIdx.x] = to<R>(v);
    }
  }
  __syncthreads();
  const int i = it.lo + threadIdx.x;
  if (threadIdx.x >= it.cnt) return;
  const C* U = static_cast<const C*>(A.U) + B.uoff + i;
  C a[RB][4];
#pragma unroll
  for (int q = 0; q < RB; ++q) a[q][0] = a[q][1] = a[q][2] = a[q][3] = C{0, 0};
  int l = 0;
  for (; l + 3 < B.rank; l += 4) {
    const C u0 = U[(int64_t)l * B.m], u1 = U[(int64_t)(l + 1) * B.m],
            u2 = U[(int64_t)(l + 2) * B.m], u3 = U[(int64_t)(l + 3) * B.m];
#pragma unroll
    for (int q = 0; q < RB; ++q) {
      a[q][0] += u0 * t[q][l];
      a[q][1] += u1 * t[q][l + 1];
      a[q][2] += u2 * t[q][l + 2];
      a[q][3] += u3 * t[q][l + 3];
    }
  }
  for (; l < B.rank; ++l) {
    const C u0 = U[(int64_t)l * B.m];
#pragma unroll
    for (int q = 0; q < RB; ++q) a[q][0] += u0 * t[q][l];
  }
#pragma unroll
  for (int q = 0; q < RB; ++q)
    if (r0 + q < nr)
      static_cast<C*>(A.P)[(int64_t)(r0 + q) * A.pstride + B.poff + i] =
          ((a[q][0] + a[q][1]) + a[q][2]) + a[q][3];
}

// Y = sb B + sa (sum of the partial rows covering each row, in the leaf's list order, the
// list split over 4 slices added in a fixed order)
template <typename R>
__global__ void __launch_bounds__(kLeafRows * kLeafSlices) k_hm_gather(
    HmOp A, double* __restrict__ Y, int64_t ldy, const double* __restrict__ Bv, int64_t ldb,
    double sb, double sa, const GmState* st, int mode) {
  using C = cx<R>;
  const int r = blockIdx.y;
  if (!rhs_on(st, r, mode)) return;
  const int leaf = blockIdx.x;
  const int32_t lo = A.leaf_lo[leaf], rows = A.leaf_lo[leaf + 1] - lo;
  const int row = threadIdx.x % kLeafRows, s = threadIdx.x / kLeafRows;
  __shared__ C part[kLeafSlices][kLeafRows];
  const C* P = static_cast<const C*>(A.P) + (int64_t)r * A.pstride;
  C acc = {0, 0};
  if (row < rows) {
    const int32_t e1 = A.leaf_ptr[leaf + 1];
    for (int e = A.leaf_ptr[leaf] + s; e < e1; e += kLeafSlices) {
      const int32_t b = A.leaf_ent[e];
      int64_t q;
      if (b >= 0) {
        const HmDense& B = A.dn[b];
        q = B.poff + (lo + row - B.rlo);
      } else {
        const HmLR& B = A.lr[-b - 1];
        q = B.poff + (lo + row - B.rlo);
      }
      acc += P[q];
    }
  }
  part[s][row] = acc;
  __syncthreads();
  if (s == 0 && row < rows) {
    const C y = ((part[0][row] + part[1][row]) + part[2][row]) + part[3][row];
    const int64_t i = lo + row;
    cd out = sa * cd{(double)y.x, (double)y.y};
    if (Bv) out += sb * ldc(Bv, (int64_t)r * ldb + i);
    stc(Y, (int64_t)r * ldy + i, out);
  }
}

// complex128 -> complex64 copy of the input vectors (one rounding per element)
__global__ void k_hm_to_f32(const double* __restrict__ X, int64_t ldx, cf* __restrict__ Xf,
                            int64_t n, const GmState* st, int mode, const int32_t* jptr,
                            int64_t jstride) {
  const int r = blockIdx.y;
  if (!rhs_on(st, r, mode)) return;
  if (jptr) X += 2 * (int64_t)*jptr * jstride;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) Xf[(int64_t)r * n + i] = to<float>(ldc(X, (int64_t)r * ldx + i));
}

void launch_hm_matvec(const Launch& L, const HmOp& A, const double* X, int64_t ldx, double* Y,
                      int64_t ldy, const double* B, int64_t ldb, double sb, double sa, int32_t nr,
                      const GmState* act, int mode, const int32_t* jptr, int64_t jstride) {
  if (nr <= 0) return;
  constexpr int kRB = 4;  // right-hand sides per CTA of the block products
  const int rb = nr >= kRB ? kRB : 1;
  const unsigned ng = (unsigned)((nr + rb - 1) / rb);
  const dim3 gv((unsigned)A.n_vt, ng), gb((unsigned)A.n_lb, ng), gd((unsigned)A.n_dense, ng),
      gl((unsigned)A.n_leaf, (unsigned)nr);
  constexpr int TL = kLeafRows * kLeafSlices;
  int launches = 1;
  const void* Xr = X;  // the input in the operator's precision
  int64_t ldr = ldx;
  if (A.f32) {
    k_hm_to_f32<<<dim3((unsigned)((A.n + 255) / 256), (unsigned)nr), 256, 0, L.stream>>>(
        X, ldx, static_cast<cf*>(A.Xf), A.n, act, mode, jptr, jstride);
    ++launches;
    Xr = A.Xf;
    ldr = A.n;
    jptr = nullptr;  // the copy is already the step's vector
  }
  auto blocks = [&](auto tag, auto rbt) {
    using R = decltype(tag);
    constexpr int RB = decltype(rbt)::value;
    if (A.n_lr > 0) {
      k_hm_vt<R, RB><<<gv, 256, 0, L.stream>>>(A, Xr, ldr, nr, act, mode, jptr, jstride);
      k_hm_lblk<R, RB><<<gb, kHmRowChunk, 0, L.stream>>>(A, nr, act, mode);
      launches += 2;
    }
    if (A.n_dense > 0) {
      k_hm_dblk<R, RB><<<gd, TL, 0, L.stream>>>(A, Xr, ldr, nr, act, mode, jptr, jstride);
      ++launches;
    }
  };
  auto run = [&](auto tag) {
    using R = decltype(tag);
    if (rb == kRB)
      blocks(tag, std::integral_constant<int, kRB>{});
    else
      blocks(tag, std::integral_constant<int, 1>{});
    k_hm_gather<R><<<gl, TL, 0, L.stream>>>(A, Y, ldy, B, ldb, sb, sa, act, mode);
  };
  if (A.f32)
    run(float{});
  else
    run(double{});
  count_launch(launches);
}

__global__ void k_hm_permute(const double* __restrict__ src, int64_t lds, double* __restrict__ dst,
                             int64_t ldd, const int32_t* __restrict__ idx, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (i >= n) return;
  stc(dst, (int64_t)r * ldd + i, ldc(src, (int64_t)r * lds + idx[i]));
}

void launch_hm_permute(const Launch& L, const double* src, int64_t lds, double* dst, int64_t ldd,
                       const int32_t* idx, int64_t n, int32_t nr) {
  if (n <= 0 || nr <= 0) return;
  k_hm_permute<<<dim3((unsigned)((n + 255) / 256), (unsigned)nr), 256, 0, L.stream>>>(src, lds, dst,
                                                                                     ldd, idx, n);
  count_launch(1);
}

// ------------------------------------------------------------------ GMRES
constexpr int kGmT = 256;

namespace {
__device__ __forceinline__ int32_t jval(const GmWork& w, int32_t j) { return j >= 0 ? j : *w.jcur; }
__device__ __forceinline__ double* vcol(const GmWork& w, int r, int l) {
  return w.Vb + 2 * (((int64_t)r * (w.restart + 1) + l) * w.n);
}
__device__ __forceinline__ int64_t hidx(const GmWork& w, int r, int i, int j) {
  return (int64_t)r * (w.restart + 1) * w.restart + i + (int64_t)j * (w.restart + 1);
}
__device__ __forceinline__ double* partp(const GmWork& w, int r, int chunk) {
  return w.part + 2 * (((int64_t)r * w.chunks + chunk) * (w.restart + 1));
}
}  // namespace

// part[r][chunk][l] = sum over the chunk of conj(V_l) w; one warp per basis vector l
// (blockIdx.y selects 8 of them), lanes over the chunk's rows
__global__ void __launch_bounds__(kGmT) k_gm_dot(GmWork w, int32_t j) {
  const int r = blockIdx.z, chunk = blockIdx.x;
  if (!w.st[r].active) return;
  j = jval(w, j);
  const int lane = threadIdx.x & 31;
  const int l = blockIdx.y * (kGmT / 32) + (threadIdx.x >> 5);
  if (l > j) return;
  const int64_t i0 = (int64_t)chunk * kGmChunk, i1 = min(w.n, i0 + kGmChunk);
  const double* wr = w.w + 2 * (int64_t)r * w.n;
  const double* v = vcol(w, r, l);
  cd s0 = {0.0, 0.0}, s1 = s0, s2 = s0, s3 = s0;
  int64_t i = i0 + lane;
  for (; i + 96 < i1; i += 128) {
    s0 += conjmul(ldc(v, i), ldc(wr, i));
    s1 += conjmul(ldc(v, i + 32), ldc(wr, i + 32));
    s2 += conjmul(ldc(v, i + 64), ldc(wr, i + 64));
    s3 += conjmul(ldc(v, i + 96), ldc(wr, i + 96));
  }
  for (; i < i1; i += 32) s0 += conjmul(ldc(v, i), ldc(wr, i));
  const cd s = warp_sum(((s0 + s1) + s2) + s3);
  if (lane == 0) stc(partp(w, r, chunk), l, s);
}

// hc[r][l] = sum over chunks (in order); pass 0 stores H[l, j], pass 1 adds to it
__global__ void k_gm_dot_finish(GmWork w, int32_t j, int pass) {
  const int r = blockIdx.x;
  if (!w.st[r].active) return;
  j = jval(w, j);
  for (int l = threadIdx.x; l <= j; l += blockDim.x) {
    cd s0 = {0.0, 0.0}, s1 = s0;
    int c = 0;
    for (; c + 1 < w.chunks; c += 2) {
      s0 += ldc(partp(w, r, c), l);
      s1 += ldc(partp(w, r, c + 1), l);
    }
    if (c < w.chunks) s0 += ldc(partp(w, r, c), l);
    const cd s = s0 + s1;
    stc(w.hc, (int64_t)r * (w.restart + 1) + l, s);
    const int64_t h = hidx(w, r, l, j);
    stc(w.H, h, pass == 0 ? s : ldc(w.H, h) + s);
  }
}

// w -= sum_{l <= j} V_l hc_l: 64 rows per CTA, the basis vectors split over 4 slices
// of threads whose partial sums are added in a fixed order
constexpr int kOrthRows = 64;
constexpr int kOrthSlices = kGmT / kOrthRows;

__global__ void __launch_bounds__(kGmT) k_gm_orth(GmWork w, int32_t j) {
  const int r = blockIdx.y;
  if (!w.st[r].active) return;
  j = jval(w, j);
  __shared__ cd h[512];
  __shared__ cd part[kOrthSlices][kOrthRows];
  const cd* hc = reinterpret_cast<const cd*>(w.hc) + (int64_t)r * (w.restart + 1);
  for (int l = threadIdx.x; l <= j; l += blockDim.x) h[l] = hc[l];
  __syncthreads();
  const int row = threadIdx.x % kOrthRows, sl = threadIdx.x / kOrthRows;
  const int64_t i = (int64_t)blockIdx.x * kOrthRows + row;
  cd s0 = {0.0, 0.0}, s1 = s0, s2 = s0, s3 = s0;
  if (i < w.n) {
    int l = sl;
    for (; l + 3 * kOrthSlices <= j; l += 4 * kOrthSlices) {
      s0 += ldc(vcol(w, r, l), i) * h[l];
      s1 += ldc(vcol(w, r, l + kOrthSlices), i) * h[l + kOrthSlices];
      s2 += ldc(vcol(w, r, l + 2 * kOrthSlices), i) * h[l + 2 * kOrthSlices];
      s3 += ldc(vcol(w, r, l + 3 * kOrthSlices), i) * h[l + 3 * kOrthSlices];
    }
    for (; l <= j; l += kOrthSlices) s0 += ldc(vcol(w, r, l), i) * h[l];
  }
  part[sl][row] = ((s0 + s1) + s2) + s3;
  __syncthreads();
  if (sl == 0 && i < w.n) {
    double* wr = w.w + 2 * (int64_t)r * w.n;
    const cd t = ((part[0][row] + part[1][row]) + part[2][row]) + part[3][row];
    stc(wr, i, ldc(wr, i) - t);
  }
}

// part[r][chunk][0].x = sum over the chunk of |w_i|^2 (mode 1: active, 2: not done)
__global__ void __launch_bounds__(kGmT) k_gm_norm(GmWork w, int mode) {
  const int r = blockIdx.y, chunk = blockIdx.x;
  if (!rhs_on(w.st, r, mode)) return;
  __shared__ double red[kGmT / 32];
  const int64_t i0 = (int64_t)chunk * kGmChunk, i1 = min(w.n, i0 + kGmChunk);
  const double* wr = w.w + 2 * (int64_t)r * w.n;
  double s = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += kGmT) s += abs2(ldc(wr, i));
  s = warp_sum_d(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < kGmT / 32; ++q) t += red[q];
    stc(partp(w, r, chunk), 0, cd{t, 0.0});
  }
}

__device__ __forceinline__ double chunk_norm(const GmWork& w, int r) {
  double t = 0.0;
  for (int c = 0; c < w.chunks; ++c) t += partp(w, r, c)[0];
  return sqrt(t);
}

// V_{j+1} = w / |w|, H[j + 1, j] = |w|
__global__ void __launch_bounds__(kGmT) k_gm_normalize(GmWork w, int32_t j) {
  const int r = blockIdx.y;
  if (!w.st[r].active) return;
  j = jval(w, j);
  const double hn = chunk_norm(w, r);
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (blockIdx.x == 0 && threadIdx.x == 0) stc(w.H, hidx(w, r, j + 1, j), cd{hn, 0.0});
  if (i >= w.n) return;
  const cd v = ldc(w.w + 2 * (int64_t)r * w.n, i);
  stc(vcol(w, r, j + 1), i, hn > 0.0 ? cdiv_real(v, hn) : cd{0.0, 0.0});
}

void launch_gm_arnoldi(const Launch& L, const GmWork& w, int32_t j) {
  const dim3 gc((unsigned)w.chunks, (unsigned)w.nr);
  const int32_t jg = j >= 0 ? j : w.restart - 1;  // device step: the largest grid
  const dim3 gd((unsigned)w.chunks, (unsigned)((jg + 1 + kGmT / 32 - 1) / (kGmT / 32)),
                (unsigned)w.nr);
  const dim3 go((unsigned)((w.n + kOrthRows - 1) / kOrthRows), (unsigned)w.nr);
  const dim3 gv((unsigned)((w.n + kGmT - 1) / kGmT), (unsigned)w.nr);
  for (int pass = 0; pass < 2; ++pass) {
    k_gm_dot<<<gd, kGmT, 0, L.stream>>>(w, j);
    k_gm_dot_finish<<<(unsigned)w.nr, 128, 0, L.stream>>>(w, j, pass);
    k_gm_orth<<<go, kGmT, 0, L.stream>>>(w, j);
  }
  k_gm_norm<<<gc, kGmT, 0, L.stream>>>(w, 1);
  k_gm_normalize<<<gv, kGmT, 0, L.stream>>>(w, j);
  count_launch(8);
}

// Givens rotations of column j, residual estimate, stopping tests (one warp per
// right-hand side: the column and the rotations are staged in shared memory, lane 0 applies
// them in order); nact = active right-hand sides afterwards.
constexpr int kRotWarps = 2;  // 40 KB of static shared memory per CTA

__global__ void __launch_bounds__(kRotWarps * 32) k_gm_rotate(GmWork w, int32_t j, int32_t* cnt) {
  j = jval(w, j);
  __shared__ cd col[kRotWarps][512];
  __shared__ cd ssn[kRotWarps][512];
  __shared__ double scs[kRotWarps][512];
  const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
  const int r = blockIdx.x * kRotWarps + wq;
  bool act = false;
  if (r < w.nr && w.st[r].active) {
    cd* H = reinterpret_cast<cd*>(w.H);
    cd* g = reinterpret_cast<cd*>(w.g) + (int64_t)r * (w.restart + 1);
    double* cs = w.cs + (int64_t)r * w.restart;
    cd* sn = reinterpret_cast<cd*>(w.sn) + (int64_t)r * w.restart;
    for (int i = lane; i <= j + 1; i += 32) col[wq][i] = H[hidx(w, r, i, j)];
    for (int i = lane; i < j; i += 32) {
      ssn[wq][i] = sn[i];
      scs[wq][i] = cs[i];
    }
    __syncwarp();
    if (lane == 0) {
      GmState& S = w.st[r];
      cd* cc = col[wq];
      for (int i = 0; i < j; ++i) {
        const cd a = cc[i], b = cc[i + 1], s = ssn[wq][i];
        cc[i] = scs[wq][i] * a + s * b;
        cc[i + 1] = scs[wq][i] * b - conjmul(s, a);
      }
      const cd a = cc[j], b = cc[j + 1];
      const double aa = hypot(a.x, a.y), bb = hypot(b.x, b.y);
      double c;
      cd s, rr;
      if (aa == 0.0) {
        c = 0.0;
        s = cd{1.0, 0.0};
        rr = b;
      } else {
        const double t = hypot(aa, bb);
        const cd ph = cd{a.x / aa, a.y / aa};
        c = aa / t;
        s = ph * cd{b.x / t, -b.y / t};
        rr = cd{ph.x * t, ph.y * t};
      }
      cs[j] = c;
      sn[j] = s;
      cc[j] = rr;
      cc[j + 1] = cd{0.0, 0.0};
      const cd gj = g[j];
      g[j + 1] = cd{0.0, 0.0} - conjmul(s, gj);
      g[j] = c * gj;
      const double res = hypot(g[j + 1].x, g[j + 1].y);
      S.res = res;
      S.kdim = j + 1;
      if (S.iters < w.maxiter) w.hist[(int64_t)r * w.maxiter + S.iters] = res;
      S.iters += 1;
      if (res <= S.tol) {
        S.converged = 1;
        S.done = 1;
        S.active = 0;
      } else if (S.iters >= w.maxiter) {
        S.done = 1;
        S.active = 0;
      } else if (j + 1 == w.restart) {
        S.active = 0;
      }
    }
    __syncwarp();
    for (int i = lane; i <= j + 1; i += 32) H[hidx(w, r, i, j)] = col[wq][i];
    act = w.st[r].active != 0;
  }
  const int c = __syncthreads_count(act && lane == 0);
  if (threadIdx.x == 0) cnt[blockIdx.x] = c;
}

// nact = sum of the per-CTA counts (fixed order); a device step index advances
__global__ void k_gm_count(GmWork w, const int32_t* cnt, int nb, int advance) {
  if (threadIdx.x != 0) return;
  int t = 0;
  for (int b = 0; b < nb; ++b) t += cnt[b];
  *w.nact = t;
  if (advance) *w.jcur += 1;
}

void launch_gm_rotate(const Launch& L, const GmWork& w, int32_t j) {
  const int nb = (w.nr + kRotWarps - 1) / kRotWarps;
  int32_t* cnt = w.nact + 1;  // nact is followed by room for one count per CTA
  k_gm_rotate<<<(unsigned)nb, kRotWarps * 32, 0, L.stream>>>(w, j, cnt);
  k_gm_count<<<1, 32, 0, L.stream>>>(w, cnt, nb, j < 0 ? 1 : 0);
  count_launch(2);
}

// y = H[0:kdim, 0:kdim]^{-1} g (back substitution, one warp per right-hand side) into hc
__global__ void k_gm_solve_y(GmWork w) {
  const int r = blockIdx.x;
  const int kd = w.st[r].kdim;
  if (kd <= 0) return;
  const int lane = threadIdx.x;
  const cd* H = reinterpret_cast<const cd*>(w.H);
  const cd* g = reinterpret_cast<const cd*>(w.g) + (int64_t)r * (w.restart + 1);
  cd* y = reinterpret_cast<cd*>(w.hc) + (int64_t)r * (w.restart + 1);
  for (int i = kd - 1; i >= 0; --i) {
    cd s = {0.0, 0.0};
    for (int l = i + 1 + lane; l < kd; l += 32) s += H[hidx(w, r, i, l)] * y[l];
    s = warp_sum(s);
    if (lane == 0) {
      const cd d = H[hidx(w, r, i, i)];
      y[i] = (d.x == 0.0 && d.y == 0.0) ? cd{0.0, 0.0} : (g[i] - s) * crecip(d);
    }
    __syncwarp();
  }
}

// x += V y for every right-hand side that iterated in this cycle
__global__ void __launch_bounds__(kGmT) k_gm_xupd(GmWork w) {
  const int r = blockIdx.y;
  const int kd = w.st[r].kdim;
  if (kd <= 0) return;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= w.n) return;
  const cd* y = reinterpret_cast<const cd*>(w.hc) + (int64_t)r * (w.restart + 1);
  double* x = w.x + 2 * (int64_t)r * w.n;
  cd s = ldc(x, i);
  for (int l = 0; l < kd; ++l) s += ldc(vcol(w, r, l), i) * y[l];
  stc(x, i, s);
}

void launch_gm_update_x(const Launch& L, const GmWork& w) {
  k_gm_solve_y<<<(unsigned)w.nr, 32, 0, L.stream>>>(w);
  k_gm_xupd<<<dim3((unsigned)((w.n + kGmT - 1) / kGmT), (unsigned)w.nr), kGmT, 0, L.stream>>>(w);
  count_launch(2);
}

// New cycle from the residual in w (its chunk norms already in part): state, then V_0.
__global__ void k_gm_start_state(GmWork w, double reltol, double abstol, int first) {
  int total = 0;
  for (int base = 0; base < w.nr; base += blockDim.x) {
    const int r = base + threadIdx.x;
    bool act = false;
    if (r < w.nr) {
      GmState& S = w.st[r];
      S.kdim = 0;
      if (first) {
        const double beta = chunk_norm(w, r);
        S.bnorm = beta;
        S.tol = fmax(reltol * beta, abstol);
        S.iters = 0;
        S.converged = 0;
        S.done = 0;
      }
      if (!S.done) {
        const double beta = chunk_norm(w, r);
        S.res = beta;
        if (beta <= S.tol) {
          S.converged = 1;
          S.done = 1;
          S.active = 0;
        } else if (S.iters >= w.maxiter) {
          S.done = 1;
          S.active = 0;
        } else {
          S.active = 1;
          cd* g = reinterpret_cast<cd*>(w.g) + (int64_t)r * (w.restart + 1);
          g[0] = cd{beta, 0.0};
        }
      } else {
        S.active = 0;
      }
      act = S.active != 0;
    }
    total += __syncthreads_count(act);
  }
  if (threadIdx.x == 0) {
    *w.nact = total;
    if (w.jcur) *w.jcur = 0;
  }
}

__global__ void __launch_bounds__(kGmT) k_gm_start_vec(GmWork w) {
  const int r = blockIdx.y;
  if (!w.st[r].active) return;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= w.n) return;
  const double beta = w.st[r].res;
  stc(vcol(w, r, 0), i, cdiv_real(ldc(w.w + 2 * (int64_t)r * w.n, i), beta));
}

void launch_gm_start(const Launch& L, const GmWork& w, double reltol, double abstol, int first) {
  const dim3 gc((unsigned)w.chunks, (unsigned)w.nr);
  k_gm_norm<<<gc, kGmT, 0, L.stream>>>(w, first ? 0 : 2);
  k_gm_start_state<<<1, 1024, 0, L.stream>>>(w, reltol, abstol, first);
  k_gm_start_vec<<<dim3((unsigned)((w.n + kGmT - 1) / kGmT), (unsigned)w.nr), kGmT, 0, L.stream>>>(
      w);
  count_launch(3);
}

}  // namespace bemgpu
