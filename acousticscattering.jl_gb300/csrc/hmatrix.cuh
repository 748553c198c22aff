// Device descriptors and launchers of the hierarchical-matrix operators and the batched
// restarted GMRES (hmatrix.cu).  All vectors are complex128 in the permuted panel order
// of the cluster tree; every reduction runs in a fixed order, so results do not depend on
// scheduling or on how many right-hand sides share a launch.
#pragma once

#include "bemgpu_internal.h"

namespace bemgpu {

constexpr int kHmMaxRank = 64;  // rank capacity of a compressed block
constexpr int kGmChunk = 1024;  // rows per GMRES partial sum

// Admissible block: rows [rlo, rlo + m), columns [clo, clo + n) of the permuted order,
// approximated by U V^T with U (m x rank) and V (n x rank) column-major.
struct HmLR {
  int32_t rlo, m, clo, n;
  int64_t uoff, voff;  // complex offsets of U (m x kmax) and V (n x kmax) in the pools
  int64_t toff;        // offset of the block's coefficients in the coefficient scratch:
                       // nvc partial sums of V^T x over column chunks, kmax each
  int32_t kmax;        // rank capacity
  int32_t rank;        // rank reached by the cross approximation
  int32_t conv;        // 1: converged to the tolerance within kmax
  int32_t nvc;         // column chunks of the coefficient products
  int64_t poff;        // offset of the block's m partial rows in the row scratch
};

// Work items of the compressed-block products: a column chunk of V^T x (c: chunk index)
// or a row chunk of U t.
constexpr int kHmColChunk = 256;
constexpr int kHmRowChunk = 256;
struct HmItem {
  int32_t blk, lo, cnt, c;
};

// Full block (column-major m x n at complex offset off of the dense pool).
struct HmDense {
  int32_t rlo, m, clo, n;
  int64_t off;
  int64_t poff;        // offset of the block's m partial rows in the row scratch
};

// One compressed operator (U, V and the full blocks complex128, or complex64 when f32).
struct HmOp {
  const HmLR* lr;
  const HmDense* dn;
  const void* U;
  const void* V;
  const void* D;
  const int32_t* leaf_lo;   // n_leaf + 1 row boundaries
  const int32_t* leaf_ptr;  // n_leaf + 1
  const int32_t* leaf_ent;  // dense block b as b, low-rank block b as -(b + 1)
  int32_t n_lr, n_dense, n_leaf, f32;
  const HmItem* vt_items;   // column chunks of every compressed block
  const HmItem* lb_items;   // row chunks of every compressed block
  int32_t n_vt, n_lb;
  double* T;                // coefficient scratch: per right-hand side tstride complex128
  int64_t tstride;
  void* P;                  // partial-row scratch: per right-hand side pstride complex
  int64_t pstride;          // (complex64 when f32)
  void* Xf;                 // f32: the input vectors rounded once to complex64 (n x nr)
  int64_t n;                // order
};

// Batched GMRES state of one right-hand side.
struct GmState {
  int32_t active;     // iterating in the current restart cycle
  int32_t done;       // converged or out of iterations
  int32_t converged;
  int32_t kdim;       // Krylov vectors of the current cycle
  int32_t iters;      // Arnoldi steps so far
  int32_t pad;
  double tol;         // max(reltol ||b||, abstol)
  double res;         // current residual estimate
  double bnorm;
};

// GMRES work arrays of a group of right-hand sides (device pointers).
struct GmWork {
  GmState* st;
  double* Vb;     // basis: [r][restart + 1][n] complex
  double* H;      // Hessenberg: [r][(restart + 1) x restart] complex, column-major
  double* cs;     // rotation cosines [r][restart]
  double* sn;     // rotation sines [r][restart] complex
  double* g;      // least-squares right side [r][restart + 1] complex
  double* hc;     // current projection coefficients [r][restart + 1] complex
  double* part;   // chunk partial sums [r][chunks][restart + 1] complex
  double* hist;   // residual estimates [r][maxiter]
  double* x;      // solutions [r][n] complex
  const double* b;  // right-hand sides [r][n] complex
  double* w;      // work vector [r][n] complex
  int64_t n;
  int32_t nr, restart, maxiter, chunks;
  int32_t* nact;  // active right-hand sides after the last rotation step
  int32_t* jcur;  // the current Arnoldi step on the device (kernels given j < 0 read it;
                  // the rotation step advances it, a new cycle resets it)
};

#ifdef __CUDACC__
// Cross approximation of every admissible block of op (0: M1, 1: M2 of the assembly
// kind); f32: FP32 entries (records: FP32 panel records) into complex64 U, V, else FP64.
// normal / large: the blocks for 256- and 512-thread CTAs (large: m + n >= kHmAcaLarge),
// max_m / max_m_large their largest row counts.
constexpr int kHmAcaLarge = 1024;
void launch_hm_aca(const Launch& L, HmLR* lr, const int32_t* normal, int32_t n_normal,
                   int32_t max_m, const int32_t* large, int32_t n_large, int32_t max_m_large,
                   void* U, void* V, const void* recs, bool f32, const int32_t* perm, int kind,
                   int op, double k, double a_re, double a_im, double tol);
// One contiguous copy per descriptor (the first rank columns of a block's U or V moved into
// pools sized by the ranks reached); sizes and offsets in 8-byte words.
struct HmCopy {
  int64_t src, dst, words;
};
void launch_hm_compact(const Launch& L, const HmCopy* d, int32_t count, const void* src,
                       void* dst);
// Regular-rule entries of the full blocks of both operators (self pairs left to the near
// kernel, which writes them through AsmInst.near_dst), precision as launch_hm_aca.
void launch_hm_dense(const Launch& L, const HmDense* dn, int32_t n_dense, void* D1, void* D2,
                     const void* recs, bool f32, const int32_t* perm, int kind, double k,
                     double a_re, double a_im);
// Y[:, r] = sb B[:, r] + sa (A X)[:, r] for every right-hand side r < nr with
// (act == null or act[r].active), the operands in permuted order.
// jptr (optional): X is offset by (*jptr) * jstride complex entries, read on the device
// (the Arnoldi vector of the current step, so that a captured graph replays any step).
void launch_hm_matvec(const Launch& L, const HmOp& A, const double* X, int64_t ldx, double* Y,
                      int64_t ldy, const double* B, int64_t ldb, double sb, double sa, int32_t nr,
                      const GmState* act, int mode, const int32_t* jptr = nullptr,
                      int64_t jstride = 0);

// GMRES steps (hmatrix.cu describes each); j < 0: the step index is read from w.jcur.
void launch_gm_start(const Launch& L, const GmWork& w, double reltol, double abstol, int first);
void launch_gm_arnoldi(const Launch& L, const GmWork& w, int32_t j);
void launch_gm_rotate(const Launch& L, const GmWork& w, int32_t j);
void launch_gm_update_x(const Launch& L, const GmWork& w);
// permuted <-> panel order of nr complex vectors of length n
void launch_hm_permute(const Launch& L, const double* src, int64_t lds, double* dst,
                       int64_t ldd, const int32_t* idx, int64_t n, int32_t nr);
#endif

}  // namespace bemgpu
