// Large dense LU with partial pivoting (one matrix, n up to tens of
// thousands) and its solve, in FP64 (the plain form of nalgebra's `m.lu()` /
// `.solve(&b)`, src/linalg/lu.rs:93-122, 221-260) and in FP32 (the factor of
// the mixed-precision form, see gesv_mixed.cu).
//
// Blocked right-looking LU, panels of NB columns:
//   1. panel factorization, partial pivoting with nalgebra's icamax rule
//      (largest |x|, first index on ties, src/base/min_max.rs:221-240; an
//      all-zero column is skipped, lu.rs:107-110), by one cooperative kernel
//      whose CTAs own row blocks of the panel and meet at two grid barriers per
//      column (candidate pivots published; pivot row swapped);
//   2. the panel's row swaps applied to the columns left and right of it;
//   3. U12 = L11^-1 A12 (unit lower triangular solve, one thread per column);
//   4. A22 -= L21 U12 by the GEMM kernels (FP64 DFMA, or the BF16-split
//      tensor-core GEMM for the FP32 factor).
// The triangular solves for the right-hand side run as one cooperative kernel
// per triangle: the diagonal block of each step is solved by CTA 0 while all
// CTAs then apply it to the remaining rows (coalesced GEMV), one grid barrier
// per phase.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace nacu {

// ---------------------------------------------------------------------------
// panel factorization (cooperative, the panel resident in shared memory)
// ---------------------------------------------------------------------------
constexpr int kPanelThreads = 256;
constexpr int kPanelMaxG = 256;          // CTAs of one panel launch
constexpr int kPanelMaxNb = 128;         // panel width
constexpr int kPanelRowsPerCta = 64;     // rows per CTA aimed for
constexpr size_t kPanelMaxSmem = 200 * 1024;

// What each column step publishes to the other CTAs, double-buffered by the
// column's parity (a slot is rewritten two steps later, after every CTA has
// passed the barrier between): each CTA's pivot candidate (|x| key, row) and
// that row's panel values, and the current values of row c.
template <typename T>
struct PanelPub {
  unsigned long long key[2][kPanelMaxG];
  int idx[2][kPanelMaxG];
  T row[2][kPanelMaxG][kPanelMaxNb];
  T diag[2][kPanelMaxNb];
  // the panel's swaps as one row mapping: row pdst[k] takes old row psrc[k]
  int npairs;
  int pdst[2 * kPanelMaxNb];
  int psrc[2 * kPanelMaxNb];
};

template <typename T>
struct PanelArgs {
  int n;        // matrix order
  T* A;         // column-major, lda
  int64_t lda;
  int j0, nb;   // panel columns [j0, j0 + nb)
  int chunk;    // rows per CTA (CTA b owns rows j0 + b*chunk ...)
  int32_t* ipiv;   // per-step pivots (0-based rows)
  int32_t* info;   // first zero pivot (1-based), atomicMin
  PanelPub<T>* pub;
};

// The cluster form gives each CTA a copy of every CTA's publication slots in
// its own shared memory: each CTA pushes its candidate (key, row index, row)
// and, when it owns it, row c into all CTAs of the cluster with remote
// stores before the cluster barrier, so that after it the pivot decision and
// the pivot row are local reads.  The header is followed by
// T row[2][kClusterMaxCtas][nb] and T diag[2][nb].
constexpr int kClusterMaxCtas = 16;
struct ClusterPub {
  unsigned long long key[2][kClusterMaxCtas];
  int idx[2][kClusterMaxCtas];
};
constexpr size_t kClusterPubHead = (sizeof(ClusterPub) + 15) & ~(size_t)15;
// Rows are stored with a stride of nb rounded up to 16 bytes (vector pushes).
template <typename T>
__host__ __device__ constexpr int cpub_stride(int nb) {
  return (nb + (int)(16 / sizeof(T)) - 1) & ~((int)(16 / sizeof(T)) - 1);
}
template <typename T>
__host__ __device__ constexpr size_t cluster_pub_bytes(int nb) {
  return kClusterPubHead + (size_t)(2 * kClusterMaxCtas + 2) * cpub_stride<T>(nb) * sizeof(T);
}
template <typename T>
__device__ __forceinline__ T* cpub_row(ClusterPub* p, int nb, int par, int q) {
  return reinterpret_cast<T*>(reinterpret_cast<unsigned char*>(p) + kClusterPubHead) +
         (size_t)(par * kClusterMaxCtas + q) * cpub_stride<T>(nb);
}
template <typename T>
__device__ __forceinline__ T* cpub_diag(ClusterPub* p, int nb, int par) {
  return reinterpret_cast<T*>(reinterpret_cast<unsigned char*>(p) + kClusterPubHead) +
         (size_t)(2 * kClusterMaxCtas + par) * cpub_stride<T>(nb);
}
// Row r of the panel (columns 0..nb) into dst in 16-byte vectors: 16 threads
// per destination (sub = 0..15), the tail element by element.
template <typename T>
__device__ __forceinline__ void push_row(T* dst, const T* P, int ldp, int r, int nb, int sub) {
  constexpr int kV = 16 / sizeof(T);
  const int nv = nb / kV;
  for (int v = sub; v < nv; v += 16) {
    T x[kV];
#pragma unroll
    for (int i = 0; i < kV; ++i) x[i] = P[(v * kV + i) * ldp + r];
    if constexpr (kV == 4) {
      *reinterpret_cast<float4*>(dst + v * kV) = make_float4(x[0], x[1], x[2], x[3]);
    } else {
      *reinterpret_cast<double2*>(dst + v * kV) = make_double2(x[0], x[1]);
    }
  }
  for (int t = nv * kV + sub; t < nb; t += 16) dst[t] = P[t * ldp + r];
}

// Composes the panel's swaps into one mapping for the columns outside it
// (one CTA): slots 0..nb-1 are rows j0.., slot nb + i the first swap partner
// ipiv[j0+i] below the panel.
template <typename T>
__device__ void panel_compose_swaps(const PanelArgs<T>& g, int nb, int tid) {
  PanelPub<T>* pub = g.pub;
  __shared__ int s_slot[kPanelMaxNb];
  __shared__ int s_row[2 * kPanelMaxNb];
  __shared__ int s_src[2 * kPanelMaxNb];
  for (int i = tid; i < nb; i += kPanelThreads) {
    const int p = g.ipiv[g.j0 + i];
    int slot = p - g.j0;
    if (p >= g.j0 + nb) {
      int f = i;
      for (int q = 0; q < i; ++q)
        if (g.ipiv[g.j0 + q] == p) {
          f = q;
          break;
        }
      slot = nb + f;
    }
    s_slot[i] = slot;
    s_row[i] = g.j0 + i;
    s_row[nb + i] = p;
  }
  for (int sl = tid; sl < 2 * nb; sl += kPanelThreads) s_src[sl] = sl;
  __syncthreads();
  if (tid == 0) {
    for (int i = 0; i < nb; ++i) {
      const int o = s_slot[i];
      const int t = s_src[i];
      s_src[i] = s_src[o];
      s_src[o] = t;
    }
    int k = 0;
    for (int sl = 0; sl < 2 * nb; ++sl)
      if (s_src[sl] != sl) {
        pub->pdst[k] = s_row[sl];
        pub->psrc[k] = s_row[s_src[sl]];
        ++k;
      }
    pub->npairs = k;
  }
}

// The grid form (the panel's rows spread over a cooperative grid, for panels
// too tall for one cluster's shared memory).  One grid barrier per column:
// the candidates and the candidate rows are published in global memory before
// it, so after it every CTA knows the pivot row's values without a second
// exchange; row c and the pivot row are swapped by their owners (nalgebra
// swaps whole rows, lu.rs:111-116; the columns outside the panel are swapped
// afterwards by lu_swap_kernel).
// The panel's pivot reciprocal, on its serial per-column path: the Newton
// form in FP64 (rcp_nr), a division in FP32.
__device__ __forceinline__ double pivot_rcp(double d) { return rcp_nr(d); }
__device__ __forceinline__ float pivot_rcp(float d) { return 1.0f / d; }

template <typename T>
__global__ void __launch_bounds__(kPanelThreads) lu_panel_grid_kernel(PanelArgs<T> g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* P = reinterpret_cast<T*>(smem_raw);  // P[t * ldp + r]
  __shared__ uint64_t s_key[kPanelThreads / 32];
  __shared__ int s_idx[kPanelThreads / 32];
  __shared__ T s_prow[kPanelMaxNb];
  __shared__ T s_drow[kPanelMaxNb];
  __shared__ int s_win, s_piv, s_wcta;
  __shared__ T s_inv;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int G = gridDim.x, b = blockIdx.x;
  const int nb = g.nb, ldp = g.chunk | 1;  // odd: row walks (t varies) hit distinct banks
  const int rb = g.j0 + b * g.chunk;
  const int nr = max(0, min(g.n, rb + g.chunk) - rb);
  T* A = g.A;
  const int64_t lda = g.lda;
  PanelPub<T>* pub = g.pub;
  for (int e = tid; e < nb * nr; e += kPanelThreads) {
    const int t = e / nr, r = e - t * nr;
    P[t * ldp + r] = A[(size_t)(g.j0 + t) * lda + rb + r];
  }
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    const int c = g.j0 + j, par = j & 1;
    // 1. my candidate: the largest |x| of column j over my rows >= c
    //    (icamax, src/base/min_max.rs:221-240: first index on ties)
    uint64_t key = 0;
    int idx = 0x7fffffff;
    for (int r = max(0, c - rb) + tid; r < nr; r += kPanelThreads) {
      const uint64_t k = pivot_key(P[j * ldp + r], rb + r == c);
      if (idx == 0x7fffffff || k > key) {
        key = k;
        idx = rb + r;
      }
    }
    warp_argmax(key, idx);
    if (lane == 0) {
      s_key[warp] = key;
      s_idx[warp] = idx;
    }
    __syncthreads();
    if (warp == 0) {
      key = lane < kPanelThreads / 32 ? s_key[lane] : 0ull;
      idx = lane < kPanelThreads / 32 ? s_idx[lane] : 0x7fffffff;
      warp_argmax(key, idx);
      if (lane == 0) {
        s_win = idx;
        pub->key[par][b] = key;
        pub->idx[par][b] = (idx == 0x7fffffff) ? -1 : idx;
      }
    }
    __syncthreads();
    // 2. publish my candidate row and, if I own it, row c
    {
      const int w = s_win;
      T* prow_out = pub->row[par][b];
      T* diag_out = pub->diag[par];
      if (w != 0x7fffffff)
        for (int t = tid; t < nb; t += kPanelThreads) prow_out[t] = P[t * ldp + (w - rb)];
      if (c >= rb && c < rb + nr)
        for (int t = tid; t < nb; t += kPanelThreads) diag_out[t] = P[t * ldp + (c - rb)];
    }
    cg::this_grid().sync();
    // 3. the pivot: every CTA reduces the G candidates the same way
    if (warp == 0) {
      uint64_t bk = 0;
      int bi = 0x7fffffff, bw = 0;
      for (int q = lane; q < G; q += 32) {
        const int ri = pub->idx[par][q];
        const uint64_t kk = pub->key[par][q];
        if (ri < 0) continue;
        if (bi == 0x7fffffff || kk > bk || (kk == bk && ri < bi)) {
          bk = kk;
          bi = ri;
          bw = q;
        }
      }
      {  // the winner's CTA: the lane holding the winning row (rows have one owner)
        const int myi = bi;
        warp_argmax(bk, bi);
        const unsigned holder = __ballot_sync(0xffffffffu, myi == bi);
        bw = __shfl_sync(0xffffffffu, bw, __ffs(holder) - 1);
      }
      if (lane == 0) {
        const bool zero = (bi == 0x7fffffff || bk == 0);  // all |x| == 0: skipped, lu.rs:107-110
        s_piv = zero ? -1 : bi;
        s_wcta = bw;
        if (b == 0) {
          g.ipiv[c] = zero ? c : bi;
          if (zero) atomicMin(g.info, c + 1);
        }
      }
    }
    __syncthreads();
    const int piv = s_piv;
    if (piv < 0) continue;
    // 4. swap rows c and piv (their owners), from the published copies
    const bool own_c = (c >= rb && c < rb + nr), own_p = (piv >= rb && piv < rb + nr);
    {
      const T* win_row = pub->row[par][s_wcta];
      const T* c_row = pub->diag[par];
      for (int t = tid; t < nb; t += kPanelThreads) {
        s_prow[t] = win_row[t];
        if (own_p && piv != c) s_drow[t] = c_row[t];
      }
      if (tid == 0) s_inv = pivot_rcp(win_row[j]);
    }
    __syncthreads();
    if (piv != c) {
      for (int t = tid; t < nb; t += kPanelThreads) {
        if (own_c) P[t * ldp + (c - rb)] = s_prow[t];
        if (own_p) P[t * ldp + (piv - rb)] = s_drow[t];
      }
      __syncthreads();
    }
    // 5. multipliers of column j below row c; their elimination from the
    //    panel's remaining columns (gauss_step, lu.rs:340-357)
    const int r0 = max(0, c + 1 - rb);
    const T inv = s_inv;
    for (int r = r0 + tid; r < nr; r += kPanelThreads) P[j * ldp + r] *= inv;
    __syncthreads();
    if (j + 1 < nb && r0 < nr) {
      const int tr = tid & 63, tc = tid >> 6;  // rows r0 + tr + 64 i, columns j + 1 + tc + 4 k
      for (int r = r0 + tr; r < nr; r += 64) {
        const T l = P[j * ldp + r];
        int t = j + 1 + tc;
        for (; t + 12 < nb; t += 16) {
          const T p0 = P[t * ldp + r], p1 = P[(t + 4) * ldp + r], p2 = P[(t + 8) * ldp + r],
                  p3 = P[(t + 12) * ldp + r];
          const T q0 = s_prow[t], q1 = s_prow[t + 4], q2 = s_prow[t + 8], q3 = s_prow[t + 12];
          P[t * ldp + r] = axpy1<false>(p0, -q0, l);
          P[(t + 4) * ldp + r] = axpy1<false>(p1, -q1, l);
          P[(t + 8) * ldp + r] = axpy1<false>(p2, -q2, l);
          P[(t + 12) * ldp + r] = axpy1<false>(p3, -q3, l);
        }
        for (; t < nb; t += 4) P[t * ldp + r] = axpy1<false>(P[t * ldp + r], -s_prow[t], l);
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < nb * nr; e += kPanelThreads) {
    const int t = e / nr, r = e - t * nr;
    A[(size_t)(g.j0 + t) * lda + rb + r] = P[t * ldp + r];
  }
  __syncthreads();  // the pivots thread 0 wrote, for the composition
  if (b == 0) panel_compose_swaps(g, nb, tid);
}

__device__ __forceinline__ void cluster_arrive_release() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_wait_acquire() {
  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// The cluster form with look-ahead inside the panel.  Column j's rank-1
// update is split: the next column (j+1) is updated at once, so that its
// pivot search can start, and the rest (columns j+2..) is deferred into the
// next column's exchange, between the cluster barrier's arrive and wait, where
// it hides the barrier's latency.  The candidate rows pushed for column j+1
// therefore still lack column j's update of columns j+2..; every CTA applies
// it to its copies with the same operands (fma(-u_t, l, x)), so the copies
// stay bit-identical to the rows their owners update.  The pivot decision and
// the pivot row are local reads (rows pushed into every CTA before the
// barrier: no remote reads).
template <typename T>
__global__ void __launch_bounds__(kPanelThreads) lu_panel_cluster_kernel(PanelArgs<T> g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ClusterPub* cpub = reinterpret_cast<ClusterPub*>(smem_raw);
  T* P = reinterpret_cast<T*>(smem_raw + cluster_pub_bytes<T>(g.nb));  // P[t * ldp + r]
  constexpr int kWarps = kPanelThreads / 32;
  __shared__ uint64_t s_key[kWarps];
  __shared__ int s_idx[kWarps];
  __shared__ T s_prev[kPanelMaxNb];  // the last eliminated column's pivot row (complete)
  __shared__ uint64_t s_ckey;
  __shared__ int s_win, s_piv, s_wcta;
  __shared__ T s_inv;
  cg::cluster_group cl = cg::this_cluster();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int G = (int)cl.num_blocks(), b = (int)cl.block_rank();
  const int nb = g.nb, ldp = g.chunk | 1;
  const int rb = g.j0 + b * g.chunk;
  const int nr = max(0, min(g.n, rb + g.chunk) - rb);
  T* A = g.A;
  const int64_t lda = g.lda;
  for (int e = tid; e < nb * nr; e += kPanelThreads) {
    const int t = e / nr, r = e - t * nr;
    P[t * ldp + r] = A[(size_t)(g.j0 + t) * lda + rb + r];
  }
  __syncthreads();
  bool pend = false;  // column j-1 was eliminated and its update of columns j+1.. is pending
  for (int j = 0; j < nb; ++j) {
    const int c = g.j0 + j, par = j & 1;
    // 1. my candidate: the largest |x| of column j over my rows >= c
    //    (icamax, src/base/min_max.rs:221-240: first index on ties)
    uint64_t key = 0;
    int idx = 0x7fffffff;
    for (int r = max(0, c - rb) + tid; r < nr; r += kPanelThreads) {
      const uint64_t k = pivot_key(P[j * ldp + r], rb + r == c);
      if (idx == 0x7fffffff || k > key) {
        key = k;
        idx = rb + r;
      }
    }
    warp_argmax(key, idx);
    if (lane == 0) {
      s_key[warp] = key;
      s_idx[warp] = idx;
    }
    __syncthreads();
    if (warp == 0) {
      key = lane < kWarps ? s_key[lane] : 0ull;
      idx = lane < kWarps ? s_idx[lane] : 0x7fffffff;
      warp_argmax(key, idx);
      if (lane == 0) {
        s_win = idx;
        s_ckey = key;
      }
    }
    __syncthreads();
    // 2. push my candidate (key, row index, row) and, if I own it, row c into
    //    every CTA of the cluster
    {
      const int w = s_win;
      if (tid < G) {
        ClusterPub* dst = cl.map_shared_rank(cpub, tid);
        dst->key[par][b] = s_ckey;
        dst->idx[par][b] = (w == 0x7fffffff) ? -1 : w;
      }
      const int q = tid >> 4;  // 16 threads per destination CTA
      if (q < G) {
        ClusterPub* dst = cl.map_shared_rank(cpub, q);
        if (w != 0x7fffffff) push_row<T>(cpub_row<T>(dst, nb, par, b), P, ldp, w - rb, nb, tid & 15);
        if (c >= rb && c < rb + nr) push_row<T>(cpub_diag<T>(dst, nb, par), P, ldp, c - rb, nb, tid & 15);
      }
    }
    __syncthreads();  // the rows are read out before the deferred update changes them
    cluster_arrive_release();
    // 3. deferred: column j-1's update of columns j+1.. (rows >= c; gauss_step,
    //    lu.rs:340-357), while the other CTAs arrive
    if (pend && j + 1 < nb) {
      const int tr = tid & 63, tc = tid >> 6;  // rows r0 + tr + 64 i, columns j + 1 + tc + 4 k
      for (int r = max(0, c - rb) + tr; r < nr; r += 64) {
        const T l = P[(j - 1) * ldp + r];
        int t = j + 1 + tc;
        for (; t + 12 < nb; t += 16) {
          const T p0 = P[t * ldp + r], p1 = P[(t + 4) * ldp + r], p2 = P[(t + 8) * ldp + r],
                  p3 = P[(t + 12) * ldp + r];
          const T q0 = s_prev[t], q1 = s_prev[t + 4], q2 = s_prev[t + 8], q3 = s_prev[t + 12];
          P[t * ldp + r] = axpy1<false>(p0, -q0, l);
          P[(t + 4) * ldp + r] = axpy1<false>(p1, -q1, l);
          P[(t + 8) * ldp + r] = axpy1<false>(p2, -q2, l);
          P[(t + 12) * ldp + r] = axpy1<false>(p3, -q3, l);
        }
        for (; t < nb; t += 4) P[t * ldp + r] = axpy1<false>(P[t * ldp + r], -s_prev[t], l);
      }
    }
    cluster_wait_acquire();
    // 4. the pivot, from the local copies of the G candidates
    if (warp == 0) {
      uint64_t bk = 0;
      int bi = 0x7fffffff, bw = 0;
      if (lane < G) {
        const int ri = cpub->idx[par][lane];
        if (ri >= 0) {
          bk = cpub->key[par][lane];
          bi = ri;
          bw = lane;
        }
      }
      const int myi = bi;
      warp_argmax(bk, bi);
      const unsigned holder = __ballot_sync(0xffffffffu, myi == bi);
      bw = __shfl_sync(0xffffffffu, bw, __ffs(holder) - 1);
      if (lane == 0) {
        const bool zero = (bi == 0x7fffffff || bk == 0);  // all |x| == 0: skipped, lu.rs:107-110
        s_piv = zero ? -1 : bi;
        s_wcta = bw;
        if (b == 0) {
          g.ipiv[c] = zero ? c : bi;
          if (zero) atomicMin(g.info, c + 1);
        }
        if (!zero) s_inv = pivot_rcp(cpub_row<T>(cpub, nb, par, bw)[j]);  // column j: complete in the copy
      }
    }
    __syncthreads();
    const int piv = s_piv;
    if (piv < 0) {  // nothing to eliminate; column j+1 already has every earlier update
      pend = false;
      continue;
    }
    // 5. complete the copies (column j-1's pending update), keep the pivot row
    //    for the next column, and swap rows c and piv (their owners)
    {
      const T* prow = cpub_row<T>(cpub, nb, par, s_wcta);
      const T* crow = cpub_diag<T>(cpub, nb, par);
      const bool own_c = (c >= rb && c < rb + nr), own_p = (piv >= rb && piv < rb + nr);
      const bool swap = (piv != c);
      const bool need_c = swap && own_p;
      const T lp = pend ? prow[j - 1] : T(0);
      const T lc = (pend && need_c) ? crow[j - 1] : T(0);
      for (int t = tid; t < nb; t += kPanelThreads) {
        T pv = prow[t];
        T cv = need_c ? crow[t] : T(0);
        if (pend && t > j) {
          const T u = s_prev[t];
          pv = axpy1<false>(pv, -u, lp);
          if (need_c) cv = axpy1<false>(cv, -u, lc);
        }
        s_prev[t] = pv;
        if (swap) {
          if (own_c) P[t * ldp + (c - rb)] = pv;
          if (own_p) P[t * ldp + (piv - rb)] = cv;
        }
      }
    }
    __syncthreads();
    // 6. multipliers of column j below row c, and their update of column j+1
    //    (the look-ahead column); the rest of the update is deferred
    {
      const T inv = s_inv;
      const T u = (j + 1 < nb) ? s_prev[j + 1] : T(0);
      for (int r = max(0, c + 1 - rb) + tid; r < nr; r += kPanelThreads) {
        const T l = P[j * ldp + r] * inv;
        P[j * ldp + r] = l;
        if (j + 1 < nb) P[(j + 1) * ldp + r] = axpy1<false>(P[(j + 1) * ldp + r], -u, l);
      }
    }
    pend = true;
    __syncthreads();
  }
  for (int e = tid; e < nb * nr; e += kPanelThreads) {
    const int t = e / nr, r = e - t * nr;
    A[(size_t)(g.j0 + t) * lda + rb + r] = P[t * ldp + r];
  }
  __syncthreads();  // the pivots thread 0 wrote, for the composition
  if (b == 0) panel_compose_swaps(g, nb, tid);
  cl.sync();  // every remote access to this CTA's shared memory is over
}

// ---------------------------------------------------------------------------
// row swaps of the panel applied to the other columns; unit-lower TRSM
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) lu_swap_kernel(int n, T* A, int64_t lda, const PanelPub<T>* __restrict__ pub,
                                                      int j0, int nb) {
  __shared__ int s_dst[2 * kPanelMaxNb], s_src[2 * kPanelMaxNb];
  const int np = pub->npairs;
  for (int k = threadIdx.x; k < np; k += blockDim.x) {
    s_dst[k] = pub->pdst[k];
    s_src[k] = pub->psrc[k];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int c = blockIdx.x * 8 + warp;  // a warp per column outside the panel
  if (c >= j0) c += nb;
  if (np == 0 || c >= n) return;
  T* col = A + (size_t)c * lda;
  constexpr int U = 2 * kPanelMaxNb / 32;
  T v[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int k = lane + 32 * u;
    if (k < np) v[u] = col[s_src[k]];
  }
  __syncwarp();
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int k = lane + 32 * u;
    if (k < np) col[s_dst[k]] = v[u];
  }
}

// U12 = L11^-1 A12 (unit lower L11, NB x NB, in shared memory) for the columns
// right of the panel: a warp owns kTrsmCols columns, lane l holding rows
// l, l + 32, ... of each in registers; row k's final value is broadcast by a
// shuffle and eliminated from the rows below (solve_lower_triangular_with_diag,
// src/linalg/solve.rs:106-133, column-oriented).
constexpr int kTrsmCols = 4;
template <typename T, int NB>
__global__ void __launch_bounds__(256) lu_trsm_kernel(int n, T* A, int64_t lda, int j0) {
  constexpr int M = NB / 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* L = reinterpret_cast<T*>(smem_raw);  // L[k * NB + i] = A[j0 + i][j0 + k]
  for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) {
    const int k = e / NB, i = e - k * NB;
    L[e] = A[(size_t)(j0 + k) * lda + j0 + i];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cbase = j0 + NB + (blockIdx.x * 8 + warp) * kTrsmCols;
  if (cbase >= n) return;
  T v[kTrsmCols][M];
#pragma unroll
  for (int c = 0; c < kTrsmCols; ++c) {
    const int col = min(cbase + c, n - 1);
#pragma unroll
    for (int m = 0; m < M; ++m) v[c][m] = A[(size_t)col * lda + j0 + m * 32 + lane];
  }
#pragma unroll
  for (int mb = 0; mb < M; ++mb) {
#pragma unroll 4
    for (int kk = 0; kk < 32; ++kk) {
      const int k = mb * 32 + kk;
      T lk[M];
#pragma unroll
      for (int m = mb; m < M; ++m) lk[m] = L[k * NB + m * 32 + lane];
#pragma unroll
      for (int c = 0; c < kTrsmCols; ++c) {
        const T xk = __shfl_sync(0xffffffffu, v[c][mb], kk);
#pragma unroll
        for (int m = mb; m < M; ++m)
          if (m > mb || lane > kk) v[c][m] = axpy1<false>(v[c][m], -lk[m], xk);
      }
    }
  }
#pragma unroll
  for (int c = 0; c < kTrsmCols; ++c) {
    const int col = cbase + c;
    if (col < n)
#pragma unroll
      for (int m = 0; m < M; ++m) A[(size_t)col * lda + j0 + m * 32 + lane] = v[c][m];
  }
}

// The same for a panel width without a register-tiled instance: L11 in shared
// memory, one thread per column, the column kept in shared memory.
template <typename T>
__global__ void __launch_bounds__(64) lu_trsm_generic_kernel(int n, T* A, int64_t lda, int j0, int nb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* L = reinterpret_cast<T*>(smem_raw);  // nb x nb
  T* X = L + (size_t)nb * nb;             // nb x 64 (column-major per thread)
  const int tid = threadIdx.x;
  for (int e = tid; e < nb * nb; e += blockDim.x) {
    const int cc = e / nb, r = e - cc * nb;
    L[e] = A[(size_t)(j0 + cc) * lda + j0 + r];
  }
  const int c = j0 + nb + blockIdx.x * 64 + tid;
  const bool valid = c < n;
  T* col = A + (size_t)(valid ? c : j0) * lda + j0;
  for (int i = 0; i < nb; ++i) X[(size_t)i * 64 + tid] = valid ? col[i] : T(0);
  __syncthreads();
  for (int i = 1; i < nb; ++i) {
    T x = X[(size_t)i * 64 + tid];
    for (int k = 0; k < i; ++k) x = axpy1<false>(x, -L[(size_t)k * nb + i], X[(size_t)k * 64 + tid]);
    X[(size_t)i * 64 + tid] = x;
  }
  if (valid)
    for (int i = 0; i < nb; ++i) col[i] = X[(size_t)i * 64 + tid];
}

template <typename T, int NB>
cudaError_t launch_trsm_tiled(int n, T* A, int64_t lda, int j0, int rest, cudaStream_t s) {
  const size_t smem = (size_t)NB * NB * sizeof(T);
  cudaError_t e = ensure_dynamic_smem(lu_trsm_kernel<T, NB>, smem);
  if (e != cudaSuccess) return e;
  const int per_cta = 8 * kTrsmCols;
  lu_trsm_kernel<T, NB><<<(rest + per_cta - 1) / per_cta, 256, smem, s>>>(n, A, lda, j0);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_trsm(int n, T* A, int64_t lda, int j0, int jb, int rest, cudaStream_t s) {
  if (jb == 64) return launch_trsm_tiled<T, 64>(n, A, lda, j0, rest, s);
  if (jb == 128) return launch_trsm_tiled<T, 128>(n, A, lda, j0, rest, s);
  const size_t smem = (size_t)jb * jb * sizeof(T) + (size_t)jb * 64 * sizeof(T);
  if (smem > 48 * 1024) {
    cudaError_t e = ensure_dynamic_smem(lu_trsm_generic_kernel<T>, smem);
    if (e != cudaSuccess) return e;
  }
  lu_trsm_generic_kernel<T><<<(rest + 63) / 64, 64, smem, s>>>(n, A, lda, j0, jb);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// triangular solves for one right-hand side (one CTA per row block, ready flags)
// ---------------------------------------------------------------------------
constexpr int kTrsvThreads = 256;
constexpr int kTrsvInfoTimeout = -1000;  // info value when a wait ran out
template <typename T>
struct TrsvTile {
  static constexpr int BS = sizeof(T) == 4 ? 128 : 64;  // rows per block
  static constexpr int NC = kTrsvThreads / BS;          // column parts per row
  static constexpr int CW = BS / NC;                    // columns per part
};

template <typename T>
struct TrsvArgs {
  int n;
  const T* A;
  int64_t lda;
  T* x;
  int lower;
  int32_t* info;
  int* sync;  // [0] ticket, [1] timeout flag, [2 + b] block b solved (zeroed before the launch)
  int poll_limit;  // polls of one flag before the wait gives up
  int skip_flag;   // a block that never raises its flag (test hook only; -1 otherwise)
};
constexpr int kTrsvPollLimit = 1 << 22;  // with the 64 ns back-off: seconds, far above any block's solve

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// lower = 1: x <- L^-1 x (unit diagonal, blocks top-down); lower = 0:
// x <- U^-1 x (bottom-up; a zero U_ii is reported in info, as
// solve_upper_triangular_mut returns false, src/linalg/solve.rs:137-182).
// CTAs take row blocks in ticket order, so a CTA only ever waits for blocks
// whose CTAs have started: for each solved block it prefetches its tile of the
// triangle into registers, waits for the block's flag (bounded), and applies
// it; then it solves its diagonal block in shared memory, stores it and raises
// its own flag.  Every wait gives up after a fixed number of polls, sets the
// timeout flag and info = kTrsvInfoTimeout, and the CTA returns.
template <typename T>
__global__ void __launch_bounds__(kTrsvThreads) trsv_kernel(TrsvArgs<T> g) {
  constexpr int BS = TrsvTile<T>::BS, NC = TrsvTile<T>::NC, CW = TrsvTile<T>::CW, LD = BS + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* Ts = reinterpret_cast<T*>(smem_raw);  // Ts[k * LD + i] = A[r0 + i][r0 + k]
  __shared__ T xs[BS];
  __shared__ T rd[BS];
  __shared__ T part[NC][BS];
  constexpr int kW = kTrsvThreads / 32, kPer = 32 / kW;  // row update: warps, terms per warp
  constexpr int kH = (BS - 32 + 31) / 32;                 // 32-row groups on the far side of a piece
  __shared__ T pp[kW * kH * 32];
  __shared__ int s_ticket, s_abort;
  const int tid = threadIdx.x, tr = tid % BS, tc = tid / BS;
  const int n = g.n, lower = g.lower;
  static_assert(kTrsvThreads % 32 == 0, "warps");
  const int nblk = (n + BS - 1) / BS;
  if (tid == 0) {
    s_ticket = atomicAdd(&g.sync[0], 1);
    s_abort = 0;
  }
  __syncthreads();
  const int t = s_ticket;
  if (t >= nblk) return;
  const int kb = lower ? t : nblk - 1 - t;
  const int r0 = kb * BS, bs = min(BS, n - r0);
  const T* A = g.A;
  const int64_t lda = g.lda;
  // U's columns are pre-scaled by 1 / U_kk, so the diagonal solve takes one
  // FMA per step on the unscaled values (scaled once when the block is
  // stored); L has a unit diagonal
  if (!lower) {
    for (int i = tid; i < bs; i += kTrsvThreads) {
      const T d = A[(size_t)(r0 + i) * lda + r0 + i];
      if (d == T(0)) atomicMin(g.info, r0 + i + 1);
      rd[i] = T(1) / d;
    }
    __syncthreads();
  }
  for (int e = tid; e < bs * bs; e += kTrsvThreads) {
    const int k = e / bs, i = e - k * bs;
    if (lower ? (i > k) : (i < k)) {
      const T v = A[(size_t)(r0 + k) * lda + r0 + i];
      Ts[k * LD + i] = lower ? v : v * rd[k];
    }
  }
  T acc = (tc == 0 && tr < bs) ? g.x[r0 + tr] : T(0);
  for (int q = 0; q < t; ++q) {
    const int jb = lower ? q : nblk - 1 - q;
    const int c0 = jb * BS, cs = min(BS, n - c0);
    T a[CW];
#pragma unroll
    for (int u = 0; u < CW; ++u) {
      const int col = tc * CW + u;
      a[u] = (tr < bs && col < cs) ? A[(size_t)(c0 + col) * lda + r0 + tr] : T(0);
    }
    if (tid == 0) {
      int polls = 0;
      while (ld_acquire(&g.sync[2 + jb]) == 0) {
        if (++polls > g.poll_limit) {
          s_abort = 1;
          atomicExch(&g.sync[1], 1);
          atomicMin(g.info, kTrsvInfoTimeout);
          break;
        }
        __nanosleep(64);
      }
    }
    __syncthreads();
    if (s_abort) return;
    // all of xs: past cs it meets zero tile entries, and shared memory may
    // still hold an earlier kernel's inf or NaN there (NaN * 0)
    if (tid < BS) xs[tid] = tid < cs ? __ldcg(&g.x[c0 + tid]) : T(0);
    __syncthreads();
#pragma unroll
    for (int u = 0; u < CW; ++u) acc = axpy1<false>(acc, -xs[tc * CW + u], a[u]);
    __syncthreads();
  }
  part[tc][tr] = acc;
  __syncthreads();
  if (tid < bs) {
    T y = part[0][tid];
#pragma unroll
    for (int c = 1; c < NC; ++c) y += part[c][tid];
    xs[tid] = y;
  }
  __syncthreads();
  // the diagonal block, 32 rows at a time: one warp solves the 32 x 32
  // diagonal piece with shuffles, then all threads apply it to the block's
  // remaining rows
  const int warp = tid >> 5, lane = tid & 31;
  const int nsub = (bs + 31) / 32;
  for (int q = 0; q < nsub; ++q) {
    const int sb = lower ? q * 32 : (nsub - 1 - q) * 32;
    const int sw = min(32, bs - sb);
    if (warp == 0) {
      T v = lane < sw ? xs[sb + lane] : T(0);
      if (lower) {
#pragma unroll
        for (int kk = 0; kk < 32; ++kk) {
          const T xk = __shfl_sync(0xffffffffu, v, kk);
          if (lane > kk && lane < sw) v = axpy1<false>(v, -Ts[(sb + kk) * LD + sb + lane], xk);
        }
      } else {
#pragma unroll
        for (int kk = 31; kk >= 0; --kk) {
          const T xk = __shfl_sync(0xffffffffu, v, kk);
          if (lane < kk && kk < sw) v = axpy1<false>(v, -Ts[(sb + kk) * LD + sb + lane], xk);
        }
      }
      if (lane < sw) xs[sb + lane] = v;  // U: unscaled
    }
    __syncthreads();
    // the block's rows on the far side of the piece (at most BS - 32) take its
    // contribution: warp w sums its share of the piece's terms for row i0 +
    // lane (+ 32h), then one thread per row adds the partial sums (a short
    // chain instead of sw dependent FMAs on one warp)
    const int i0 = lower ? sb + sw : 0, i1 = lower ? bs : sb;
    if (i1 > i0) {
#pragma unroll
      for (int h = 0; h < kH; ++h) {
        const int i = i0 + lane + 32 * h;
        T acc = T(0);
        if (i < i1)
#pragma unroll
          for (int u = 0; u < kPer; ++u) {
            const int k = kPer * warp + u;
            if (k < sw) acc = axpy1<false>(acc, -Ts[(sb + k) * LD + i], xs[sb + k]);
          }
        pp[(warp * kH + h) * 32 + lane] = acc;
      }
      __syncthreads();
      for (int r = tid; r < i1 - i0; r += kTrsvThreads) {
        T y = xs[i0 + r];
#pragma unroll
        for (int w = 0; w < kW; ++w) y += pp[(w * kH + (r >> 5)) * 32 + (r & 31)];
        xs[i0 + r] = y;
      }
    }
    __syncthreads();
  }
  if (tid < bs) g.x[r0 + tid] = lower ? xs[tid] : xs[tid] * rd[tid];
  // the barrier orders the block's stores before thread 0's release, which is
  // cumulative over them: a CTA that acquires the flag sees x (no fence needed)
  __syncthreads();
  if (tid == 0 && kb != g.skip_flag) st_release(&g.sync[2 + kb], 1);
}

// info holds a large sentinel until some pivot fails; 0 afterwards means "ok".
__global__ void info_init_kernel(int32_t* info) { *info = 0x7fffffff; }
__global__ void info_finalize_kernel(int32_t* info) {
  if (*info == 0x7fffffff) *info = 0;
}

// x <- P x: nalgebra's row swaps in order (PermutationSequence::permute_rows,
// src/linalg/permutation_sequence.rs), one thread, the vector and the swap
// list staged in shared memory when they fit.
template <typename T>
__global__ void apply_pivots_kernel(int n, const int32_t* __restrict__ ipiv, T* x, int staged) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* xs = reinterpret_cast<T*>(smem_raw);
  int32_t* ps = reinterpret_cast<int32_t*>(xs + (staged ? n : 0));
  if (!staged) {
    if (threadIdx.x == 0)
      for (int i = 0; i < n; ++i) {
        const int p = ipiv[i];
        if (p != i) {
          const T t = x[i];
          x[i] = x[p];
          x[p] = t;
        }
      }
    return;
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    xs[i] = x[i];
    ps[i] = ipiv[i];
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 0; i < n; ++i) {
      const int p = ps[i];
      if (p != i) {
        const T t = xs[i];
        xs[i] = xs[p];
        xs[p] = t;
      }
    }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = xs[i];
}

// perm[i] = the source row of row i after the swaps (gathers replace them).
__global__ void pivots_to_perm_kernel(int n, const int32_t* __restrict__ ipiv, int32_t* perm, int staged) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int32_t* pm = staged ? reinterpret_cast<int32_t*>(smem_raw) : perm;
  int32_t* ps = staged ? pm + n : nullptr;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    pm[i] = i;
    if (staged) ps[i] = ipiv[i];
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 0; i < n; ++i) {
      const int p = staged ? ps[i] : ipiv[i];
      if (p != i) {
        const int32_t t = pm[i];
        pm[i] = pm[p];
        pm[p] = t;
      }
    }
  __syncthreads();
  if (staged)
    for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = pm[i];
}

// ---------------------------------------------------------------------------
// host drivers
// ---------------------------------------------------------------------------
int coop_grid(const void* kern, int threads, size_t smem) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
  if (per_sm < 1) per_sm = 1;
  return sm_count() * per_sm;
}

// The panel's exchange area (sized for FP64 and the widest panel).
size_t getrf_ws_bytes() { return (sizeof(PanelPub<double>) + 255) & ~(size_t)255; }

// slot 0: the next panel's columns (on the panel stream), slot 1: the rest of
// the trailing update (on the update stream, concurrently)
typedef int (*UpdateFn)(int m, int n, int k, const void* L21, const void* U12, void* A22, int64_t lda, void* ctx,
                        int slot, cudaStream_t s);

// Internal streams of the look-ahead schedule (per device, created on first
// use): the panel chain runs at the highest stream priority, the bulk of each
// trailing update at the lowest, so the next panel's CTAs are dispatched as
// soon as SMs free up.
struct LookaheadStreams {
  cudaStream_t panel = nullptr, rest = nullptr;
  cudaEvent_t fork = nullptr, trsm_done = nullptr, rest_done = nullptr, join = nullptr;
  bool ready = false;
};
LookaheadStreams g_lookahead[64];

int lookahead_streams(LookaheadStreams** out, const char* name) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  if (dev < 0 || dev >= 64) return record_arg_error(-99, "getrf: device index >= 64");
  LookaheadStreams& L = g_lookahead[dev];
  if (!L.ready) {
    int least = 0, greatest = 0;
    e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&L.panel, cudaStreamNonBlocking, greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&L.rest, cudaStreamNonBlocking, least);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L.fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L.trsm_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L.rest_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L.join, cudaEventDisableTiming);
    if (e != cudaSuccess) return record_cuda_error(e, name);
    L.ready = true;
  }
  *out = &L;
  return NACU_SUCCESS;
}

// CTAs per cluster for the cluster-form panel (16, else 8, else 0 = grid
// form only), from the occupancy API with the largest panel's shared memory;
// queried once per scalar type.
template <typename T>
int panel_cluster_ctas() {
  static int ctas = -1;
  if (ctas >= 0) return ctas;
  ctas = 0;
  auto kern = lu_panel_cluster_kernel<T>;
  if (ensure_dynamic_smem(kern, kPanelMaxSmem) != cudaSuccess ||
      cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
    cudaGetLastError();
    return ctas;
  }
  for (int c = kClusterMaxCtas; c >= 8; c /= 2) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(c);
    cfg.blockDim = dim3(kPanelThreads);
    cfg.dynamicSmemBytes = kPanelMaxSmem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = c;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) == cudaSuccess && nclusters >= 1) {
      ctas = c;
      break;
    }
    cudaGetLastError();
  }
  return ctas;
}

// Blocked LU with look-ahead: step k's panel chain (panel, row swaps, TRSM,
// and the update of the next panel's columns) runs on the panel stream; the
// rest of step k's trailing update runs on the update stream while panel k+1
// is factored.  Step k+1's row swaps wait for that update.  Forks from and
// joins to the caller's stream.
template <typename T>
int getrf_blocked(int n, T* A, int64_t lda, int32_t* ipiv, int32_t* info, void* ws, int nb, UpdateFn update,
                  void* ctx, cudaStream_t s, const char* name) {
  cudaError_t e;
  if (nb > kPanelMaxNb) nb = kPanelMaxNb;
  const void* pk = reinterpret_cast<const void*>(lu_panel_grid_kernel<T>);
  e = ensure_dynamic_smem(pk, kPanelMaxSmem);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  const int cluster = panel_cluster_ctas<T>();
  const int gmax = std::min(kPanelMaxG, sm_count());
  LookaheadStreams* la = nullptr;
  int rc = lookahead_streams(&la, name);
  if (rc != NACU_SUCCESS) return rc;
  const cudaStream_t sp = la->panel, su = la->rest;
  e = cudaEventRecord(la->fork, s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(sp, la->fork, 0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(su, la->fork, 0);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  info_init_kernel<<<1, 1, 0, sp>>>(info);
  bool rest_pending = false;
  for (int j0 = 0; j0 < n; j0 += nb) {
    const int jb = std::min(nb, n - j0);
    const int rows = n - j0;
    PanelArgs<T> pa{n, A, lda, j0, jb, 0, ipiv, info, reinterpret_cast<PanelPub<T>*>(ws)};
    const int cchunk = cluster ? (rows + cluster - 1) / cluster : 0;
    const size_t csmem = cluster_pub_bytes<T>(jb) + (size_t)(cchunk | 1) * jb * sizeof(T);
    if (cluster && csmem <= kPanelMaxSmem) {
      pa.chunk = cchunk;
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(cluster);
      cfg.blockDim = dim3(kPanelThreads);
      cfg.dynamicSmemBytes = csmem;
      cfg.stream = sp;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = cluster;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      e = cudaLaunchKernelEx(&cfg, lu_panel_cluster_kernel<T>, pa);
      if (e != cudaSuccess) return record_cuda_error(e, name);
    } else {
      const int max_rows = (int)(kPanelMaxSmem / ((size_t)jb * sizeof(T))) - 1;  // leading dimension chunk | 1
      int G = std::max((rows + kPanelRowsPerCta - 1) / kPanelRowsPerCta, (rows + max_rows - 1) / max_rows);
      G = std::max(1, std::min(G, gmax));
      const int chunk = (rows + G - 1) / G;
      if (chunk > max_rows) return record_arg_error(-1, "getrf: n too large for the shared-memory panel");
      pa.chunk = chunk;
      void* args[] = {&pa};
      e = cudaLaunchCooperativeKernel(pk, G, kPanelThreads, args, (size_t)(chunk | 1) * jb * sizeof(T), sp);
      if (e != cudaSuccess) return record_cuda_error(e, name);
    }
    if (rest_pending) {  // the swaps below touch the columns the previous update is still writing
      e = cudaStreamWaitEvent(sp, la->rest_done, 0);
      if (e != cudaSuccess) return record_cuda_error(e, name);
      rest_pending = false;
    }
    if (n > jb) lu_swap_kernel<T><<<(n - jb + 7) / 8, 256, 0, sp>>>(n, A, lda, pa.pub, j0, jb);
    const int rest = n - j0 - jb;
    if (rest > 0) {
      e = launch_trsm<T>(n, A, lda, j0, jb, rest, sp);
      if (e != cudaSuccess) return record_cuda_error(e, name);
      const T* L21 = A + (size_t)j0 * lda + j0 + jb;
      const T* U12 = A + (size_t)(j0 + jb) * lda + j0;
      T* A22 = A + (size_t)(j0 + jb) * lda + j0 + jb;
      const int nn = std::min(nb, rest);  // the next panel's columns
      rc = update(rest, nn, jb, L21, U12, A22, lda, ctx, 0, sp);
      if (rc != NACU_SUCCESS) return rc;
      if (rest > nn) {
        e = cudaEventRecord(la->trsm_done, sp);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(su, la->trsm_done, 0);
        if (e != cudaSuccess) return record_cuda_error(e, name);
        rc = update(rest, rest - nn, jb, L21, U12 + (size_t)nn * lda, A22 + (size_t)nn * lda, lda, ctx, 1, su);
        if (rc != NACU_SUCCESS) return rc;
        e = cudaEventRecord(la->rest_done, su);
        if (e != cudaSuccess) return record_cuda_error(e, name);
        rest_pending = true;
      }
    }
    rc = check_launch(name);
    if (rc != NACU_SUCCESS) return rc;
  }
  if (rest_pending) {
    e = cudaStreamWaitEvent(sp, la->rest_done, 0);
    if (e != cudaSuccess) return record_cuda_error(e, name);
  }
  info_finalize_kernel<<<1, 1, 0, sp>>>(info);
  e = cudaEventRecord(la->join, sp);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, la->join, 0);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  return check_launch(name);
}

// x <- U^-1 L^-1 x (the permutation already applied); sync: 2 + n/64 + 1 ints.
size_t trsv_sync_bytes(int n) { return ((size_t)n / 64 + 4) * sizeof(int); }

template <typename T>
int trsv_pair(int n, const T* LU, int64_t lda, T* x, int32_t* info, int* sync, cudaStream_t s, const char* name,
              int poll_limit = kTrsvPollLimit, int skip_lower_flag = -1) {
  const void* tk = reinterpret_cast<const void*>(trsv_kernel<T>);
  constexpr int BS = TrsvTile<T>::BS;
  const size_t smem = (size_t)BS * (BS + 1) * sizeof(T);
  cudaError_t e = ensure_dynamic_smem(tk, smem);
  if (e != cudaSuccess) return record_cuda_error(e, name);
  const int nblk = (n + BS - 1) / BS;
  for (int lower = 1; lower >= 0; --lower) {
    e = cudaMemsetAsync(sync, 0, (size_t)(nblk + 2) * sizeof(int), s);
    if (e != cudaSuccess) return record_cuda_error(e, name);
    TrsvArgs<T> ta{n, LU, lda, x, lower, info, sync, poll_limit, lower ? skip_lower_flag : -1};
    trsv_kernel<T><<<nblk, kTrsvThreads, smem, s>>>(ta);
  }
  return check_launch(name);
}

constexpr size_t kStageLimit = 160 * 1024;

template <typename T>
int getrs_one(int n, const T* LU, int64_t lda, const int32_t* ipiv, T* x, int32_t* info, int* sync, cudaStream_t s,
              const char* name, int poll_limit = kTrsvPollLimit, int skip_lower_flag = -1) {
  info_init_kernel<<<1, 1, 0, s>>>(info);
  const size_t stage = (size_t)n * (sizeof(T) + sizeof(int32_t));
  const int staged = stage <= kStageLimit;
  if (staged && stage > 48 * 1024) {
    cudaError_t e = ensure_dynamic_smem(apply_pivots_kernel<T>, kStageLimit);
    if (e != cudaSuccess) return record_cuda_error(e, name);
  }
  apply_pivots_kernel<T><<<1, 256, staged ? stage : 0, s>>>(n, ipiv, x, staged);
  int rc = trsv_pair<T>(n, LU, lda, x, info, sync, s, name, poll_limit, skip_lower_flag);
  if (rc != NACU_SUCCESS) return rc;
  info_finalize_kernel<<<1, 1, 0, s>>>(info);
  return check_launch(name);
}

int update_fp64(int m, int n, int k, const void* L21, const void* U12, void* A22, int64_t lda, void*, int,
                cudaStream_t s) {
  return nacu_dgemm(m, n, k, -1.0, static_cast<const double*>(L21), lda, static_cast<const double*>(U12), lda, 1.0,
                    static_cast<double*>(A22), lda, s);
}

// ---------------------------------------------------------------------------
// mixed precision: FP32 factor (tensor-core trailing updates), FP64 refinement
// ---------------------------------------------------------------------------
struct Update32Ctx {
  void* ws[2];  // one split-GEMM workspace per concurrent update (slot)
  size_t ws_bytes[2];
};

int update_fp32_split(int m, int n, int k, const void* L21, const void* U12, void* A22, int64_t lda, void* ctx,
                      int slot, cudaStream_t s) {
  const Update32Ctx* c = static_cast<const Update32Ctx*>(ctx);
  return split_gemm_run<float, float>(m, n, k, -1.0, static_cast<const float*>(L21), lda,
                                      static_cast<const float*>(U12), lda, 1.0, static_cast<float*>(A22), lda, 3,
                                      c->ws[slot], c->ws_bytes[slot], s);
}

__global__ void to_fp32_kernel(int n, const double* __restrict__ A, int64_t lda, float* __restrict__ A32) {
  const int64_t total = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = e / n, r = e - c * n;
    A32[e] = (float)A[c * lda + r];
  }
}

__device__ __forceinline__ unsigned long long dabs_bits(double x) { return abs_bits_f64(x); }

// part[cb * n + i] = sum over the column chunk cb of A[i][j] * x[j] (or |A[i][j]| when abs_mode).
constexpr int kGemvChunks = 16;
__global__ void gemv_partial_kernel(int n, const double* __restrict__ A, int64_t lda, const double* __restrict__ x,
                                    double* __restrict__ part, int abs_mode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int chunk = (n + kGemvChunks - 1) / kGemvChunks;
  const int j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
  double acc = 0.0;
  int j = j0;
  for (; j + 4 <= j1; j += 4) {
    const double a0 = A[(size_t)j * lda + i], a1 = A[(size_t)(j + 1) * lda + i];
    const double a2 = A[(size_t)(j + 2) * lda + i], a3 = A[(size_t)(j + 3) * lda + i];
    if (abs_mode) acc += fabs(a0) + fabs(a1) + fabs(a2) + fabs(a3);
    else acc = fma(a3, x[j + 3], fma(a2, x[j + 2], fma(a1, x[j + 1], fma(a0, x[j], acc))));
  }
  for (; j < j1; ++j) acc = abs_mode ? acc + fabs(A[(size_t)j * lda + i]) : fma(A[(size_t)j * lda + i], x[j], acc);
  part[(size_t)blockIdx.y * n + i] = acc;
}

// r = b - sum(part) (or the row sums when abs_mode); norms (max |.|, as bits) of
// r, x and b into nrm[0..2] (atomicMax on non-negative doubles' bit images).
__global__ void residual_finish_kernel(int n, const double* __restrict__ b, const double* __restrict__ x,
                                       const double* __restrict__ part, double* __restrict__ r,
                                       unsigned long long* nrm, int abs_mode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long rn = 0, xn = 0, bn = 0;
  if (i < n) {
    double s = 0.0;
    for (int cb = 0; cb < kGemvChunks; ++cb) s += part[(size_t)cb * n + i];
    const double v = abs_mode ? s : b[i] - s;
    if (!abs_mode) r[i] = v;
    rn = dabs_bits(v);
    xn = dabs_bits(x[i]);
    bn = dabs_bits(b[i]);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    rn = max(rn, __shfl_xor_sync(0xffffffffu, rn, off));
    xn = max(xn, __shfl_xor_sync(0xffffffffu, xn, off));
    bn = max(bn, __shfl_xor_sync(0xffffffffu, bn, off));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&nrm[0], rn);
    atomicMax(&nrm[1], xn);
    atomicMax(&nrm[2], bn);
  }
}

// d32 = (float)(P src * 2^-e): the row permutation of the factor fused as a gather
__global__ void scale_to_fp32_kernel(int n, const double* __restrict__ src, const int32_t* __restrict__ perm, int e,
                                     float* __restrict__ d32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d32[i] = (float)(src[perm[i]] * __longlong_as_double((long long)(1023 - e) << 52));
}
// x += (double)d32 * 2^e; max |d| into nrm[3]
__global__ void accumulate_kernel(int n, const float* __restrict__ d32, int e, double* __restrict__ x,
                                  unsigned long long* nrm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long dn = 0;
  if (i < n) {
    const double d = (double)d32[i] * __longlong_as_double((long long)(1023 + e) << 52);
    x[i] += d;
    dn = dabs_bits(d);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) dn = max(dn, __shfl_xor_sync(0xffffffffu, dn, off));
  if ((threadIdx.x & 31) == 0) atomicMax(&nrm[3], dn);
}

// ---- GMRES refinement (Carson & Higham 2018, "Accelerating the solution of
// linear systems by iterative refinement in three precisions", GMRES-IR) ----
// When u32 * cond(A) approaches 1 the FP32 correction (LU)^-1 r no longer
// contracts and classical refinement stalls.  GMRES-IR keeps the FP32 factors
// as a preconditioner instead: each outer step solves the correction equation
// M^-1 A d = M^-1 r (M = P^T L U, FP32) by restarted GMRES with FP64 vectors --
// the product A v in FP64, the preconditioner applied with the FP32 triangular
// solves (the vector scaled by a power of two into FP32 and back) -- and then
// forms the new FP64 residual.  The preconditioner is applied in FP64 with the
// FP32 factors promoted exactly to FP64 (applying it in FP32 inflated the
// first correction's error by the FP32 solve's own rounding, ~1e5x at cond
// 1e8 in a CPU study).  The Krylov basis is orthogonalised by
// classical Gram-Schmidt applied twice (one multi-dot and one update kernel
// per pass), the small Hessenberg least-squares problem is solved on the host
// with Givens rotations.
// When classical refinement diverges outright (the correction grows by more
// than kGmresMaxRho per step, u32 * cond well above 1), the FP32 preconditioner
// is too weak for GMRES to pay: measured at n = 4096, 100 GMRES iterations
// reduced the preconditioned residual only to 6e-2 at cond 1e8 (ratio 68)
// and 3e7 (ratio 15), against 29 iterations at cond 1e7 (ratio 1.4).  Those
// systems go to the FP64 refactorization at once, and so does a GMRES cycle
// that ends above kGmresGiveUp.
constexpr int kGmresM = 64;           // restart length (basis vectors)
constexpr double kGmresTol = 1e-6;    // relative reduction of the preconditioned residual per outer step
constexpr int kGmresOuter = 8;        // outer steps (FP64 residuals) before the FP64 fallback
constexpr double kGmresMaxRho = 2.5;  // correction growth per classical step above which GMRES is skipped
constexpr double kGmresGiveUp = 1e-2; // relative residual after a full cycle above which GMRES is abandoned

// y = sum of the GEMV partials; max |y| (bits) into *nrm
__global__ void gemv_finish_kernel(int n, const double* __restrict__ part, double* __restrict__ y,
                                   unsigned long long* nrm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long yn = 0;
  if (i < n) {
    double acc = 0.0;
    for (int cb = 0; cb < kGemvChunks; ++cb) acc += part[(size_t)cb * n + i];
    y[i] = acc;
    yn = abs_bits_f64(acc);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) yn = max(yn, __shfl_xor_sync(0xffffffffu, yn, off));
  if ((threadIdx.x & 31) == 0) atomicMax(nrm, yn);
}
// out[c] = V[:, c] . w for c < cols (one block per column, fixed reduction order)
__global__ void __launch_bounds__(256) block_dots_kernel(int n, const double* __restrict__ V, int64_t ldv,
                                                         const double* __restrict__ w, double* __restrict__ out) {
  __shared__ double red[8];
  const double* v = V + (size_t)blockIdx.x * ldv;
  double acc = 0.0;
  for (int t = threadIdx.x; t < n; t += 256) acc = fma(v[t], w[t], acc);
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int k = 0; k < 8; ++k) sum += red[k];
    out[blockIdx.x] = sum;
  }
}
// w += sign * V[:, 0..cols) h
__global__ void combo_kernel(int n, const double* __restrict__ V, int64_t ldv, int cols, const double* __restrict__ h,
                             double sign, double* __restrict__ w) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  double acc = 0.0;
  for (int c = 0; c < cols; ++c) acc = fma(V[(size_t)c * ldv + t], h[c], acc);
  w[t] = fma(sign, acc, w[t]);
}
// dst = P src (the factors' row permutation as a gather)
__global__ void permute_kernel(int n, const double* __restrict__ src, const int32_t* __restrict__ perm,
                               double* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[perm[i]];
}
// A64 = (double)A32, exact
__global__ void to_fp64_kernel(int64_t total, const float* __restrict__ A32, double* __restrict__ A64) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    A64[e] = (double)A32[e];
}
// v = w * s
__global__ void scale_kernel(int n, const double* __restrict__ w, double s, double* __restrict__ v) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) v[t] = w[t] * s;
}

struct MixedLuLayout {
  size_t a32, ipiv, perm, info, cand, split, split2, r, d32, part, nrm, a64, vk, wv, yv, hv, total;
};
inline size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }
MixedLuLayout mixed_lu_layout(int n, int nb) {
  MixedLuLayout L;
  size_t o = 0;
  L.a32 = o;   o = up256(o + (size_t)n * n * 4);
  L.ipiv = o;  o = up256(o + (size_t)n * 4);
  L.perm = o;  o = up256(o + (size_t)n * 4);
  L.info = o;  o = up256(o + 16);
  L.cand = o;  o = up256(o + getrf_ws_bytes());
  o = (o + 1023) & ~(size_t)1023;
  L.split = o; o = up256(o + nacu_gemm_split_workspace_bytes(n, n, nb));
  o = (o + 1023) & ~(size_t)1023;
  L.split2 = o; o = up256(o + nacu_gemm_split_workspace_bytes(n, nb, nb));
  L.r = o;     o = up256(o + (size_t)n * 8);
  L.d32 = o;   o = up256(o + (size_t)n * 4);
  L.part = o;  o = up256(o + (size_t)kGemvChunks * n * 8);
  L.nrm = o;   o = up256(o + 8 * 8);
  L.a64 = o;   o = up256(o + (size_t)n * n * 8);
  L.vk = o;    o = up256(o + (size_t)n * (kGmresM + 1) * 8);  // GMRES basis
  L.wv = o;    o = up256(o + (size_t)n * 8);
  L.yv = o;    o = up256(o + (size_t)n * 8);
  L.hv = o;    o = up256(o + (size_t)(2 * kGmresM + 4) * 8);  // two Gram-Schmidt passes' coefficients
  L.total = o + 1024;  // the caller's base may need aligning to 1024
  return L;
}

int exp_of_bits(unsigned long long b) {
  const int ex = (int)((b >> 52) & 0x7ff);
  if (ex == 0 || ex == 0x7ff) return 0;
  const int e = ex - 1023;
  return e < -1000 ? -1000 : (e > 1000 ? 1000 : e);
}

// The buffers of one GMRES correction solve.
struct GmresBufs {
  int n;
  const double* A;
  int64_t lda;
  const double* LU;       // the FP32 LU factors promoted to FP64 (packed, lda = n)
  const int32_t* perm;    // row permutation of the factors as a gather
  int32_t* info;          // trsv info slot
  void* trsv_sync;
  double* part;
  unsigned long long* nrm;  // [4]: max |y| of the last product
  double *V, *w, *y, *h;
};

// z = M^-1 src (M = P^T L U, the FP32 factors applied in FP64).
int gmres_precond(const GmresBufs& g, const double* src, double* z, cudaStream_t s) {
  const int nblk = (g.n + 255) / 256;
  permute_kernel<<<nblk, 256, 0, s>>>(g.n, src, g.perm, z);
  int rc = trsv_pair<double>(g.n, g.LU, g.n, z, g.info, static_cast<int*>(g.trsv_sync), s,
                             "nacu_dgesv_mixed_ir: gmres");
  if (rc != NACU_SUCCESS) return rc;
  return check_launch("nacu_dgesv_mixed_ir: gmres");
}

// d = approximate solution of M^-1 A d = M^-1 r by GMRES(kGmresM) from d = 0,
// the preconditioned residual reduced by kGmresTol (or the basis exhausted);
// d is added to x.  *inner counts the basis vectors used.
int gmres_correction(const GmresBufs& g, const double* r, double* x, int* inner, double* rel, cudaStream_t s) {
  const int n = g.n, nblk = (n + 255) / 256;
  double* V = g.V;
  // v0 = M^-1 r / ||M^-1 r||
  int rc = gmres_precond(g, r, g.w, s);
  if (rc != NACU_SUCCESS) return rc;
  block_dots_kernel<<<1, 256, 0, s>>>(n, g.w, n, g.w, g.h);
  double hb[kGmresM + 2];
  cudaMemcpyAsync(hb, g.h, 8, cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgesv_mixed_ir: gmres");
  const double beta = std::sqrt(hb[0]);
  *inner = 0;
  *rel = 0.0;
  if (!(beta > 0.0) || !std::isfinite(beta)) return NACU_SUCCESS;
  scale_kernel<<<nblk, 256, 0, s>>>(n, g.w, 1.0 / beta, V);
  static thread_local double H[kGmresM + 1][kGmresM];  // column j: H[0..j+1][j]
  double cs[kGmresM], sn[kGmresM], gv[kGmresM + 1];
  for (int i = 0; i <= kGmresM; ++i) gv[i] = 0.0;
  gv[0] = beta;
  int k = 0;
  for (int j = 0; j < kGmresM; ++j) {
    // w = M^-1 A v_j
    cudaMemsetAsync(g.nrm + 4, 0, 8, s);
    gemv_partial_kernel<<<dim3(nblk, kGemvChunks), 256, 0, s>>>(n, g.A, g.lda, V + (size_t)j * n, g.part, 0);
    gemv_finish_kernel<<<nblk, 256, 0, s>>>(n, g.part, g.y, g.nrm + 4);
    rc = gmres_precond(g, g.y, g.w, s);
    if (rc != NACU_SUCCESS) return rc;
    // classical Gram-Schmidt, twice: h = V^T w, w -= V h
    block_dots_kernel<<<j + 1, 256, 0, s>>>(n, V, n, g.w, g.h);
    combo_kernel<<<nblk, 256, 0, s>>>(n, V, n, j + 1, g.h, -1.0, g.w);
    double* h2d = g.h + kGmresM + 2;
    block_dots_kernel<<<j + 1, 256, 0, s>>>(n, V, n, g.w, h2d);
    combo_kernel<<<nblk, 256, 0, s>>>(n, V, n, j + 1, h2d, -1.0, g.w);
    block_dots_kernel<<<1, 256, 0, s>>>(n, g.w, n, g.w, g.y);  // ||w||^2 (y is free here)
    double h1[kGmresM + 1], h2[kGmresM + 1], hn2 = 0.0;
    cudaMemcpyAsync(h1, g.h, (size_t)(j + 1) * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(h2, h2d, (size_t)(j + 1) * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&hn2, g.y, 8, cudaMemcpyDeviceToHost, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgesv_mixed_ir: gmres");
    const double hn = std::sqrt(hn2);
    for (int i = 0; i <= j; ++i) H[i][j] = h1[i] + h2[i];
    H[j + 1][j] = hn;
    // previous rotations, then the one that zeroes H[j+1][j]
    for (int i = 0; i < j; ++i) {
      const double t = cs[i] * H[i][j] + sn[i] * H[i + 1][j];
      H[i + 1][j] = -sn[i] * H[i][j] + cs[i] * H[i + 1][j];
      H[i][j] = t;
    }
    const double den = std::hypot(H[j][j], H[j + 1][j]);
    cs[j] = den > 0.0 ? H[j][j] / den : 1.0;
    sn[j] = den > 0.0 ? H[j + 1][j] / den : 0.0;
    H[j][j] = den;
    H[j + 1][j] = 0.0;
    gv[j + 1] = -sn[j] * gv[j];
    gv[j] = cs[j] * gv[j];
    k = j + 1;
    if (!std::isfinite(gv[j + 1]) || std::fabs(gv[j + 1]) <= kGmresTol * beta || !(hn > 0.0)) break;
    if (j + 1 < kGmresM) scale_kernel<<<nblk, 256, 0, s>>>(n, g.w, 1.0 / hn, V + (size_t)(j + 1) * n);
  }
  // y = H^-1 g (upper triangular k x k), then x += V y
  double yk[kGmresM];
  for (int i = k - 1; i >= 0; --i) {
    double acc = gv[i];
    for (int c = i + 1; c < k; ++c) acc -= H[i][c] * yk[c];
    yk[i] = (H[i][i] != 0.0) ? acc / H[i][i] : 0.0;
  }
  cudaMemcpyAsync(g.h, yk, (size_t)k * 8, cudaMemcpyHostToDevice, s);
  combo_kernel<<<nblk, 256, 0, s>>>(n, V, n, k, g.h, 1.0, x);
  e = cudaStreamSynchronize(s);  // yk lives on the host stack
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgesv_mixed_ir: gmres");
  *inner = k;
  *rel = (k > 0) ? std::fabs(gv[k]) / beta : 1.0;
  return check_launch("nacu_dgesv_mixed_ir: gmres");
}

}  // namespace nacu

extern "C" {

size_t nacu_gesv_mixed_workspace_bytes(int n) { return nacu::mixed_lu_layout(n, 128).total; }

int nacu_dgesv_mixed_ir(int n, const double* A, int64_t lda, const double* b, double* x, double tol_units,
                        int max_iter, int* iters_out, double* berr_out, int* fallback_out, void* workspace,
                        size_t workspace_bytes, nacu_stream_t stream) {
  using namespace nacu;
  if (n < 0) return record_arg_error(-1, "dgesv_mixed_ir: n < 0");
  if (n == 0) return NACU_SUCCESS;
  if (!A || lda < n) return record_arg_error(-2, "dgesv_mixed_ir: bad A / lda");
  if (!b || !x) return record_arg_error(-4, "dgesv_mixed_ir: null b or x");
  const int nb = 128;
  MixedLuLayout L = mixed_lu_layout(n, nb);
  if (!workspace || workspace_bytes < L.total) return record_arg_error(-11, "dgesv_mixed_ir: workspace too small");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)workspace + 1023) & ~(uintptr_t)1023);
  float* A32 = reinterpret_cast<float*>(base + L.a32);
  int32_t* ipiv = reinterpret_cast<int32_t*>(base + L.ipiv);
  int32_t* perm = reinterpret_cast<int32_t*>(base + L.perm);
  int32_t* info = reinterpret_cast<int32_t*>(base + L.info);
  void* cand = base + L.cand;
  void* split_ws = base + L.split;
  double* r = reinterpret_cast<double*>(base + L.r);
  float* d32 = reinterpret_cast<float*>(base + L.d32);
  double* part = reinterpret_cast<double*>(base + L.part);
  unsigned long long* nrm = reinterpret_cast<unsigned long long*>(base + L.nrm);
  double* A64 = reinterpret_cast<double*>(base + L.a64);
  const double tol = (tol_units > 0 ? tol_units : 1.0) * n * 2.220446049250313e-16;
  if (max_iter <= 0) max_iter = 30;
  const int nblk = (n + 255) / 256;
  int iters = 0, fallback = 0;
  double berr = INFINITY;
  unsigned long long h[4];
  // ||A||_inf (FP64 row sums of |A|)
  cudaMemsetAsync(nrm, 0, 64, s);
  gemv_partial_kernel<<<dim3(nblk, kGemvChunks), 256, 0, s>>>(n, A, lda, x, part, 1);
  residual_finish_kernel<<<nblk, 256, 0, s>>>(n, b, b, part, r, nrm, 1);
  cudaMemcpyAsync(h, nrm, 32, cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgesv_mixed_ir");
  const double anorm = __builtin_bit_cast(double, h[0]);
  const double bnorm = __builtin_bit_cast(double, h[2]);
  // FP32 factor
  to_fp32_kernel<<<sm_count() * 8, 256, 0, s>>>(n, A, lda, A32);
  Update32Ctx uctx{{base + L.split2, split_ws},
                   {nacu_gemm_split_workspace_bytes(n, nb, nb), nacu_gemm_split_workspace_bytes(n, n, nb)}};
  int rc = getrf_blocked<float>(n, A32, n, ipiv, info, cand, nb, update_fp32_split, &uctx, s, "nacu_dgesv_mixed_ir");
  if (rc != NACU_SUCCESS) return rc;
  int32_t hinfo = 0;
  cudaMemcpyAsync(&hinfo, info, 4, cudaMemcpyDeviceToHost, s);
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgesv_mixed_ir");
  bool converged = false;
  double last_rho = INFINITY;  // growth of the correction over the last classical step
  if (hinfo == 0) {
    const int staged = (size_t)n * 8 <= kStageLimit;
    if (staged && (size_t)n * 8 > 48 * 1024) {
      e = ensure_dynamic_smem(pivots_to_perm_kernel, kStageLimit);
      if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgesv_mixed_ir");
    }
    pivots_to_perm_kernel<<<1, 256, staged ? (size_t)n * 8 : 0, s>>>(n, ipiv, perm, staged);
    // refinement: x0 = 0, r0 = b
    cudaMemsetAsync(x, 0, (size_t)n * 8, s);
    cudaMemcpyAsync(r, b, (size_t)n * 8, cudaMemcpyDeviceToDevice, s);
    double rnorm = bnorm, dprev = 0.0;
    last_rho = 0.0;
    for (int it = 0; it < max_iter; ++it) {
      // d = (LU)^-1 P r in FP32, scaled by the exponent of ||r||
      int er = 0;
      {
        const double m = rnorm;
        er = (m > 0.0 && std::isfinite(m)) ? exp_of_bits(__builtin_bit_cast(unsigned long long, m)) : 0;
      }
      scale_to_fp32_kernel<<<nblk, 256, 0, s>>>(n, r, perm, er, d32);
      rc = trsv_pair<float>(n, A32, n, d32, info + 1, reinterpret_cast<int*>(cand), s, "nacu_dgesv_mixed_ir");
      if (rc != NACU_SUCCESS) return rc;
      cudaMemsetAsync(nrm, 0, 64, s);
      accumulate_kernel<<<nblk, 256, 0, s>>>(n, d32, er, x, nrm);
      gemv_partial_kernel<<<dim3(nblk, kGemvChunks), 256, 0, s>>>(n, A, lda, x, part, 0);
      residual_finish_kernel<<<nblk, 256, 0, s>>>(n, b, x, part, r, nrm, 0);
      cudaMemcpyAsync(h, nrm, 32, cudaMemcpyDeviceToHost, s);
      e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgesv_mixed_ir");
      ++iters;
      rnorm = __builtin_bit_cast(double, h[0]);
      const double xnorm = __builtin_bit_cast(double, h[1]);
      const double dnorm = __builtin_bit_cast(double, h[3]);
      berr = rnorm / (anorm * xnorm + bnorm);
      if (berr <= tol) {
        converged = true;
        break;
      }
      if (it >= 1 && dprev > 0.0) last_rho = dnorm / dprev;
      if (!std::isfinite(berr)) last_rho = INFINITY;
      if (!std::isfinite(berr) || (it >= 1 && dprev > 0.0 && dnorm > 0.5 * dprev)) break;  // stagnation
      dprev = dnorm;
    }
  }
  if (!converged && hinfo == 0 && last_rho <= kGmresMaxRho) {
    // GMRES-IR with the FP32 factors as the preconditioner, from x = 0
    to_fp64_kernel<<<sm_count() * 8, 256, 0, s>>>((int64_t)n * n, A32, A64);
    GmresBufs gb{n, A, lda, A64, perm, info + 1, cand, part, nrm,
                 reinterpret_cast<double*>(base + L.vk), reinterpret_cast<double*>(base + L.wv),
                 reinterpret_cast<double*>(base + L.yv), reinterpret_cast<double*>(base + L.hv)};
    cudaMemsetAsync(x, 0, (size_t)n * 8, s);
    cudaMemcpyAsync(r, b, (size_t)n * 8, cudaMemcpyDeviceToDevice, s);
    double best = INFINITY;
    for (int outer = 0; outer < kGmresOuter; ++outer) {
      int inner = 0;
      double rel = 1.0;
      rc = gmres_correction(gb, r, x, &inner, &rel, s);
      if (rc != NACU_SUCCESS) return rc;
      if (!(rel <= kGmresGiveUp)) break;  // the preconditioner is too weak: FP64
      cudaMemsetAsync(nrm, 0, 64, s);
      gemv_partial_kernel<<<dim3(nblk, kGemvChunks), 256, 0, s>>>(n, A, lda, x, part, 0);
      residual_finish_kernel<<<nblk, 256, 0, s>>>(n, b, x, part, r, nrm, 0);
      cudaMemcpyAsync(h, nrm, 32, cudaMemcpyDeviceToHost, s);
      e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgesv_mixed_ir");
      ++iters;
      berr = __builtin_bit_cast(double, h[0]) / (anorm * __builtin_bit_cast(double, h[1]) + bnorm);
      if (berr <= tol) {
        converged = true;
        fallback = 2;
        break;
      }
      if (!std::isfinite(berr) || !(berr < 0.5 * best) || inner == 0) break;  // no progress: FP64 fallback
      best = berr;
    }
  }
  if (!converged) {
    // FP64 fallback on a copy of A
    fallback = 1;
    cudaMemcpy2DAsync(A64, (size_t)n * 8, A, (size_t)lda * 8, (size_t)n * 8, n, cudaMemcpyDeviceToDevice, s);
    rc = nacu_dgetrf(n, A64, n, ipiv, info, cand, getrf_ws_bytes(), stream);
    if (rc != NACU_SUCCESS) return rc;
    cudaMemcpyAsync(x, b, (size_t)n * 8, cudaMemcpyDeviceToDevice, s);
    rc = nacu_dgetrs(n, A64, n, ipiv, x, info + 1, cand, getrf_ws_bytes(), stream);
    if (rc != NACU_SUCCESS) return rc;
    cudaMemsetAsync(nrm, 0, 64, s);
    gemv_partial_kernel<<<dim3(nblk, kGemvChunks), 256, 0, s>>>(n, A, lda, x, part, 0);
    residual_finish_kernel<<<nblk, 256, 0, s>>>(n, b, x, part, r, nrm, 0);
    cudaMemcpyAsync(h, nrm, 32, cudaMemcpyDeviceToHost, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return record_cuda_error(e, "nacu_dgesv_mixed_ir");
    berr = __builtin_bit_cast(double, h[0]) / (anorm * __builtin_bit_cast(double, h[1]) + bnorm);
  }
  if (iters_out) *iters_out = iters;
  if (berr_out) *berr_out = berr;
  if (fallback_out) *fallback_out = fallback;
  return check_launch("nacu_dgesv_mixed_ir");
}

size_t nacu_getrf_workspace_bytes(int n) {
  return std::max(nacu::getrf_ws_bytes(), nacu::trsv_sync_bytes(n < 0 ? 0 : n));
}

int nacu_dgetrf(int n, double* A, int64_t lda, int32_t* ipiv, int32_t* info, void* workspace, size_t workspace_bytes,
                nacu_stream_t stream) {
  using namespace nacu;
  if (n < 0) return record_arg_error(-1, "dgetrf: n < 0");
  if (n == 0) return NACU_SUCCESS;
  if (!A) return record_arg_error(-2, "dgetrf: null A");
  if (lda < n) return record_arg_error(-3, "dgetrf: lda < n");
  if (!ipiv || !info) return record_arg_error(-4, "dgetrf: null ipiv or info");
  if (!workspace || workspace_bytes < nacu_getrf_workspace_bytes(n))
    return record_arg_error(-6, "dgetrf: workspace too small");
  return getrf_blocked<double>(n, A, lda, ipiv, info, workspace, 64, update_fp64, nullptr, (cudaStream_t)stream,
                               "nacu_dgetrf");
}

int nacu_dgetrs(int n, const double* LU, int64_t lda, const int32_t* ipiv, double* b, int32_t* info, void* workspace,
                size_t workspace_bytes, nacu_stream_t stream) {
  using namespace nacu;
  if (n < 0) return record_arg_error(-1, "dgetrs: n < 0");
  if (n == 0) return NACU_SUCCESS;
  if (!LU || !ipiv || !b || !info) return record_arg_error(-2, "dgetrs: null argument");
  if (lda < n) return record_arg_error(-3, "dgetrs: lda < n");
  if (!workspace || workspace_bytes < nacu::trsv_sync_bytes(n))
    return record_arg_error(-7, "dgetrs: workspace too small");
  return getrs_one<double>(n, LU, lda, ipiv, b, info, static_cast<int*>(workspace), (cudaStream_t)stream,
                           "nacu_dgetrs");
}

int nacu_test_dgetrs_flag_timeout(int n, const double* LU, int64_t lda, const int32_t* ipiv, double* b,
                                  int32_t* info, int skip_block, int poll_limit, void* workspace,
                                  size_t workspace_bytes, nacu_stream_t stream) {
  using namespace nacu;
  if (n <= 0) return record_arg_error(-1, "test_dgetrs_flag_timeout: n <= 0");
  if (!LU || !ipiv || !b || !info) return record_arg_error(-2, "test_dgetrs_flag_timeout: null argument");
  if (lda < n) return record_arg_error(-3, "test_dgetrs_flag_timeout: lda < n");
  const int nblk = (n + TrsvTile<double>::BS - 1) / TrsvTile<double>::BS;
  if (skip_block < 0 || skip_block >= nblk)
    return record_arg_error(-7, "test_dgetrs_flag_timeout: skip_block outside the row blocks");
  if (poll_limit < 1 || poll_limit > kTrsvPollLimit)
    return record_arg_error(-8, "test_dgetrs_flag_timeout: poll_limit outside [1, 2^22]");
  if (!workspace || workspace_bytes < nacu::trsv_sync_bytes(n))
    return record_arg_error(-10, "test_dgetrs_flag_timeout: workspace too small");
  return getrs_one<double>(n, LU, lda, ipiv, b, info, static_cast<int*>(workspace), (cudaStream_t)stream,
                           "nacu_test_dgetrs_flag_timeout", poll_limit, skip_block);
}

}  // extern "C"
