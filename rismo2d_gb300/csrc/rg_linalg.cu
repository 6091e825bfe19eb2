// Sparse linear algebra of the Newton step: L2 scaling, SpMV, ILU(0)
// factorisation, ILU(0) triangular solves and right-preconditioned BiCGStab.
//
// Restates CRSMAT::ScaleL2Norm (CRSMat.cpp:319-346), CRSMAT::MulVec
// (CRSMat.cpp:466-496), PRECO_ILU0::Factor (Preco_ilu0.cpp:64-189),
// PRECO_ILU0::Solve (Preco_ilu0.cpp:497-530, 964-980) and BICGSTAB::Iterate
// (Bicgstab.cpp:66-375).
//
// The ILU(0) factorisation and both triangular solves follow the reference's
// equation order exactly, so they inherit its dependency chains.  They run as
// persistent, co-resident ("cooperative") grids in which warp w owns rows
// w, w+W, w+2W, ... and each row waits only for the rows it reads:
//   * the factorisation publishes a per-row epoch flag with release
//     semantics; readers acquire it (bounded spin, error word on timeout);
//   * the triangular solves need no flags: the solution vector is pre-filled
//     with a signalling-NaN sentinel and each entry is written once with a
//     single 64/32-bit store, so the value itself is the "ready" signal.
// Row ownership in increasing order makes the schedule deadlock-free when all
// warps are resident; every wait is bounded and reports RG_ERR_DEVICE_WAIT
// instead of hanging.

#include "rg_internal.cuh"

#include <algorithm>
#include <cstdio>

#include <cooperative_groups.h>

namespace {

constexpr long long kSpinLimit = 1ll << 20;   // ~0.5 s of polling at L2 latency
constexpr int kDevErrWait = 1;
constexpr int kDevErrPivot = 2;
constexpr int kDevErrWidth = 4;

// ---- sentinels: signalling NaNs never produced by arithmetic ---------------
__device__ __forceinline__ unsigned long long sent64() { return 0x7FF4DEADBEEF0001ull; }
__device__ __forceinline__ unsigned int sent32() { return 0x7FA0BEEFu; }

__device__ __forceinline__ double ld_relaxed(const double* p) {
  double v;
  asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ float ld_relaxed(const float* p) {
  float v;
  asm volatile("ld.relaxed.gpu.global.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(double* p, double v) {
  asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(float* p, float v) {
  asm volatile("st.relaxed.gpu.global.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ bool is_sent(double v) { return __double_as_longlong(v) == (long long)sent64(); }
__device__ __forceinline__ bool is_sent(float v) { return __float_as_uint(v) == sent32(); }
template <class T> __device__ __forceinline__ T sentinel();
template <> __device__ __forceinline__ double sentinel<double>() { return __longlong_as_double((long long)sent64()); }
template <> __device__ __forceinline__ float sentinel<float>() { return __uint_as_float(sent32()); }

__device__ __forceinline__ int ld_relaxed_i(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// err[0] error bits (any bit set aborts every waiting warp), err[1] kernel
// tag, err[2] row that gave up, err[3] the dependency it waited for
__device__ void record_wait_failure(int* err, int tag, int row, int dep) {
  if (atomicCAS(&err[1], 0, tag) == 0) {
    err[2] = row;
    err[3] = dep;
  }
  atomicOr(&err[0], kDevErrWait);
}

// the polling limit of the bounded waits: err[4..5] holds the context's limit
// (rg_set_wait_limit; 0 = kSpinLimit)
__device__ __forceinline__ long long spin_limit(const int* err) {
  const long long v = *reinterpret_cast<const volatile long long*>(err + 4);
  return v > 0 ? v : kSpinLimit;
}

template <class T>
__device__ __forceinline__ T wait_value(const T* p, int* err, int tag, int row, int dep) {
  T v = ld_relaxed(p);
  if (!is_sent(v)) return v;
  const long long limit = spin_limit(err);
  long long it = 0;
  while (is_sent(v)) {
    ++it;
    if ((it & 1023) == 0 && ld_relaxed_i(err) != 0) return (T)0;   // another warp gave up
    if (it > limit) {
      record_wait_failure(err, tag, row, dep);
      return (T)0;
    }
    v = ld_relaxed(p);
  }
  return v;
}

__device__ __forceinline__ bool wait_flag(const int* flag, int epoch, int* err, int tag, int row, int dep) {
  if (ld_acquire(flag) == epoch) return true;
  const long long limit = spin_limit(err);
  long long it = 0;
  while (ld_acquire(flag) != epoch) {
    ++it;
    if ((it & 1023) == 0 && ld_relaxed_i(err) != 0) return false;
    if (it > limit) {
      record_wait_failure(err, tag, row, dep);
      return false;
    }
  }
  return true;
}

// round-to-nearest products/sums without contraction (keeps the reference's
// separately rounded multiply-then-add of Preco_ilu0.cpp:181)
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <class T>
__global__ void k_fill(T* p, int64_t n, T v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}
template <class T>
__global__ void k_fill_sentinel(T* p, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = sentinel<T>();
}

// ---- reductions: block partials, then one block sums them in fixed order ----
template <int NV>
__device__ __forceinline__ void block_partials(double (&v)[NV], double* partial) {
  __shared__ double sh[NV][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; k++) {
    double s = warp_sum(v[k]);
    if (lane == 0) sh[k][wid] = s;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) {
      double s = (lane < nw) ? sh[k][lane] : 0.0;
      s = warp_sum(s);
      if (lane == 0) partial[(size_t)k * gridDim.x + blockIdx.x] = s;
    }
  }
}

__device__ double block_sum_fixed(const double* p, int n) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += p[i];
  s = warp_sum(s);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = s;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;   // valid in thread 0
}

// ---- CRSMAT::ScaleL2Norm ----------------------------------------------------
template <class VT>
__global__ void k_sumsq(const VT* b, int n, double* partial) {
  double v[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[0] += (double)b[i] * b[i];
  block_partials<1>(v, partial);
}
__global__ void k_scale_fin(const double* partial, int nparts, KrylovScalars* ks) {
  double s = block_sum_fixed(partial, nparts);
  if (threadIdx.x == 0) ks->t1 = sqrt(s);
}
template <class MT>
__global__ void k_scale_apply(MT* A, int64_t nnz, double* B, int n, const KrylovScalars* ks) {
  const double s = ks->t1;
  if (!(fabs(s) > 1.0e-40)) return;
  const MT sm = (MT)s;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x)
    A[i] = A[i] / sm;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) B[i] = B[i] / s;
}

// ---- CRSMAT::MulVec: 16 lanes per row, optional fused dot products ---------
// r = A x; if d1: partial dot (r, d1); if d2 == r: partial (r, r)
template <class VT, class MT, class AT, int ND>
__global__ void k_spmv(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                       const MT* __restrict__ A, const VT* __restrict__ x, VT* __restrict__ r,
                       const VT* __restrict__ d1, double* partial, const KrylovScalars* ks) {
  if (ks && ks->conv != 0) return;
  constexpr int NDX = (ND > 0) ? ND : 1;
  const int sub = threadIdx.x & 15;
  const int half = (threadIdx.x >> 4) & 1;
  double dv[NDX];
#pragma unroll
  for (int k = 0; k < NDX; k++) dv[k] = 0.0;
  // two rows per warp; the trip count is uniform across the warp so the
  // full-mask shuffles below always see all 32 lanes
  const int warps_per_block = blockDim.x >> 5;
  const int gwarp = blockIdx.x * warps_per_block + (threadIdx.x >> 5);
  const int nwarp = gridDim.x * warps_per_block;
  for (int r0 = 2 * gwarp; r0 < n; r0 += 2 * nwarp) {
    const int row = r0 + half;
    const bool valid = row < n;
    AT acc = 0;
    if (valid) {
      const int b = rowptr[row], e = rowptr[row + 1];
      for (int q = b + sub; q < e; q += 16) acc += (AT)A[q] * (AT)x[col[q]];
    }
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (valid && sub == 0) {
      VT rv = (VT)acc;
      r[row] = rv;
      if (ND >= 1) dv[0] += (double)rv * (double)d1[row];
      if (ND >= 2) dv[1] += (double)rv * (double)rv;
    }
  }
  if (ND > 0) block_partials<NDX>(dv, partial);
}

// ---- ILU(0) factorisation (sync-free, warp per row, epoch flags) ----------
template <class MT>
struct RowBuf {
  int col[RG_MAXW];
  MT val[RG_MAXW];
};

// replay the eliminations of pivots k < upto on a copy of row c (the state row
// c has in the reference's right-looking loop when pivot `upto` is reached)
template <class MT>
__device__ void partial_row(int c, int upto, const int* rowptr, const int* col, const MT* LU,
                            const int* lsort_ptr, const int* lsort_pos, int* fflag, int epoch,
                            RowBuf<MT>& rb, int* err, int lane) {
  const int b = rowptr[c], w = rowptr[c + 1] - b;
  for (int j = lane; j < w; j += 32) {
    rb.col[j] = col[b + j];
    rb.val[j] = __ldcg(&LU[b + j]);   // row c itself is not final: it is re-derived from A below
  }
  __syncwarp();
  for (int q = lsort_ptr[c]; q < lsort_ptr[c + 1]; q++) {
    const int p = lsort_pos[q];
    const int k = rb.col[p];
    if (k >= upto) break;   // sorted by column
    if (lane == 0) wait_flag(&fflag[k], epoch, err, 2, c, k);
    __syncwarp();
    const MT piv = __ldcg(&LU[rowptr[k]]);
    const MT factor = -rb.val[p] / piv;
    __syncwarp();
    if (lane == 0) rb.val[p] = factor;
    for (int q2 = rowptr[k] + 1 + lane; q2 < rowptr[k + 1]; q2 += 32) {
      const int cc = col[q2];
      if (cc <= k) continue;
      for (int l = 0; l < w; l++)
        if (rb.col[l] == cc) {
          rb.val[l] = add_rn(rb.val[l], mul_rn(factor, __ldcg(&LU[q2])));
          break;
        }
    }
    __syncwarp();
  }
}

template <class MT, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_factor(int n, const int* __restrict__ rowptr,
                                                       const int* __restrict__ col, const MT* __restrict__ A,
                                                       MT* LU, const int* __restrict__ lsort_ptr,
                                                       const int* __restrict__ lsort_pos, int* fflag, int epoch,
                                                       int* err) {
  __shared__ RowBuf<MT> rows[WARPS];
  __shared__ RowBuf<MT> cand[WARPS];
  __shared__ RowBuf<MT> best[WARPS];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int gw = blockIdx.x * WARPS + wib, nw = gridDim.x * WARPS;
  RowBuf<MT>& s = rows[wib];
  for (int i = gw; i < n; i += nw) {
    const int b = rowptr[i], w = rowptr[i + 1] - b;
    if (w > RG_MAXW) {
      if (lane == 0) {
        atomicOr(&err[0], kDevErrWidth);
        st_release(&fflag[i], epoch);
      }
      continue;
    }
    for (int j = lane; j < w; j += 32) {
      s.col[j] = col[b + j];
      s.val[j] = A[b + j];
    }
    __syncwarp();
    // eliminations by the pivots k < i of row i, in increasing k
    for (int q = lsort_ptr[i]; q < lsort_ptr[i + 1]; q++) {
      const int p = lsort_pos[q];
      const int k = s.col[p];
      if (lane == 0) wait_flag(&fflag[k], epoch, err, 1, i, k);
      __syncwarp();
      const MT piv = __ldcg(&LU[rowptr[k]]);
      const MT factor = -s.val[p] / piv;
      __syncwarp();
      if (lane == 0) s.val[p] = factor;
      for (int q2 = rowptr[k] + 1 + lane; q2 < rowptr[k + 1]; q2 += 32) {
        const int cc = col[q2];
        if (cc <= k) continue;
        for (int l = 0; l < w; l++)
          if (s.col[l] == cc) {
            s.val[l] = add_rn(s.val[l], mul_rn(factor, __ldcg(&LU[q2])));
            break;
          }
      }
      __syncwarp();
    }
    // zero-pivot repair (Preco_ilu0.cpp:95-138): add the partially eliminated
    // row with the largest entry in column i
    if (fabs((double)s.val[0]) < 1.0e-20) {
      int piv = -1;
      double mx = 0.0;
      for (int j = 1; j < w; j++) {
        const int c = s.col[j];
        if (c <= i) continue;
        // restore row c from A, then replay its pivots < i
        const int bc = rowptr[c], wc = rowptr[c + 1] - bc;
        for (int jj = lane; jj < wc; jj += 32) {
          cand[wib].col[jj] = col[bc + jj];
        }
        __syncwarp();
        // partial_row reads row c's current LU, which (row c > i) has not been
        // written yet in this epoch: LU still holds A copied in by the host
        partial_row<MT>(c, i, rowptr, col, LU, lsort_ptr, lsort_pos, fflag, epoch, cand[wib], err, lane);
        double p = 0.0;
        for (int jj = 0; jj < wc; jj++)
          if (cand[wib].col[jj] == i) p = fabs((double)cand[wib].val[jj]);
        if (p > mx) {
          mx = p;
          piv = c;
          for (int jj = lane; jj < wc; jj += 32) {
            best[wib].col[jj] = cand[wib].col[jj];
            best[wib].val[jj] = cand[wib].val[jj];
          }
        }
        __syncwarp();
      }
      if (piv > 0) {
        const int wp = rowptr[piv + 1] - rowptr[piv];
        for (int j = lane; j < w; j += 32)
          for (int k = 0; k < wp; k++)
            if (s.col[j] == best[wib].col[k]) s.val[j] = s.val[j] + best[wib].val[k];
      } else if (lane == 0) {
        atomicOr(&err[0], kDevErrPivot);
      }
      __syncwarp();
    }
    for (int j = lane; j < w; j += 32) __stcg(&LU[b + j], s.val[j]);
    __threadfence();
    __syncwarp();
    if (lane == 0) st_release(&fflag[i], epoch);
  }
}

// level-scheduled ILU(0): the rows of one dependency level are eliminated in
// parallel (warp per row, same arithmetic as k_factor), levels separated by a
// grid-wide barrier.  A pivot below the repair threshold stops the kernel with
// a flag; the host then reruns the dependency-driven kernel, which repairs.
template <class MT, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_factor_level(int nlev, const int* __restrict__ lev_ptr,
                                                             const int* __restrict__ lev_rows,
                                                             const int* __restrict__ rowptr,
                                                             const int* __restrict__ col, const MT* __restrict__ A,
                                                             MT* LU, const int* __restrict__ lsort_ptr,
                                                             const int* __restrict__ lsort_pos, int* err) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  __shared__ RowBuf<MT> rows[WARPS];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int gw = blockIdx.x * WARPS + wib, nw = gridDim.x * WARPS;
  RowBuf<MT>& s = rows[wib];
  for (int l = 0; l < nlev; l++) {
    const int b0 = lev_ptr[l], b1 = lev_ptr[l + 1];
    for (int idx = b0 + gw; idx < b1; idx += nw) {
      const int i = lev_rows[idx];
      const int b = rowptr[i], w = rowptr[i + 1] - b;
      for (int j = lane; j < w; j += 32) {
        s.col[j] = col[b + j];
        s.val[j] = A[b + j];
      }
      __syncwarp();
      for (int q = lsort_ptr[i]; q < lsort_ptr[i + 1]; q++) {
        const int p = lsort_pos[q];
        const int k = s.col[p];
        const MT piv = __ldcg(&LU[rowptr[k]]);
        const MT factor = -s.val[p] / piv;
        __syncwarp();
        if (lane == 0) s.val[p] = factor;
        for (int q2 = rowptr[k] + 1 + lane; q2 < rowptr[k + 1]; q2 += 32) {
          const int cc = col[q2];
          if (cc <= k) continue;
          for (int ll = 0; ll < w; ll++)
            if (s.col[ll] == cc) {
              s.val[ll] = add_rn(s.val[ll], mul_rn(factor, __ldcg(&LU[q2])));
              break;
            }
        }
        __syncwarp();
      }
      if (fabs((double)s.val[0]) < 1.0e-20 && lane == 0) atomicOr(&err[0], 16);   // needs the repair path
      for (int j = lane; j < w; j += 32) __stcg(&LU[b + j], s.val[j]);
      __syncwarp();
    }
    grid.sync();
  }
}

// fill map of the level-scheduled factorisation: for every L entry p of row i
// (sorted by column k) and every entry t >= 1 of row k, the position of that
// column in row i, or -1 (the linear searches of Preco_ilu0.cpp:177-184, done
// once per pattern)
__global__ void k_build_fmap(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                             const int* __restrict__ lsort_ptr, const int* __restrict__ lsort_pos,
                             const long long* __restrict__ fmap_off, short* __restrict__ fmap) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = gw; i < n; i += nw) {
    const int b = rowptr[i], w = rowptr[i + 1] - b;
    for (int q = lsort_ptr[i]; q < lsort_ptr[i + 1]; q++) {
      const int k = col[b + lsort_pos[q]];
      const int bk = rowptr[k], wk = rowptr[k + 1] - bk;
      for (int t = 1 + lane; t < wk; t += 32) {
        const int cc = col[bk + t];
        short pos = -1;
        if (cc > k)
          for (int l = 0; l < w; l++)
            if (col[b + l] == cc) {
              pos = (short)l;
              break;
            }
        fmap[fmap_off[q] + (t - 1)] = pos;
      }
    }
  }
}

// level-scheduled ILU(0) with the fill map: per row, the pivots and pivot rows
// of all its L entries are fetched in one parallel batch into shared memory,
// then the eliminations run in column order from shared memory
//
// Rows flagged in fp64row (FP32 factors only: the rows of near-dry nodes in the
// mixed precision path) are eliminated in FP64 -- the row, its multipliers and its
// pivot in double, from the FP32 pivot rows -- and stored in FP32 like the others.
template <class MT, int WARPS, int STAGE>
__global__ void __launch_bounds__(WARPS * 32) k_factor_level2(int nlev, const int* __restrict__ lev_ptr,
                                                              const int* __restrict__ lev_rows,
                                                              const int* __restrict__ rowptr,
                                                              const int* __restrict__ col,
                                                              const MT* __restrict__ A, MT* LU,
                                                              const int* __restrict__ lsort_ptr,
                                                              const int* __restrict__ lsort_pos,
                                                              const int* __restrict__ lsort_col,
                                                              const long long* __restrict__ fmap_off,
                                                              const short* __restrict__ fmap, int* err,
                                                              const unsigned char* __restrict__ fp64row) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  __shared__ MT sval[WARPS][RG_MAXW];
  __shared__ MT spiv[WARPS][RG_MAXW];
  __shared__ int sbeg[WARPS][RG_MAXW + 1];     // start of each pivot row in the stage
  __shared__ int spos[WARPS][RG_MAXW];         // position of the L entry in the row
  __shared__ int srow[WARPS][RG_MAXW];         // first U-side entry of the pivot row
  __shared__ MT stage[WARPS][STAGE];
  __shared__ short smap[WARPS][STAGE];
  __shared__ double svd[sizeof(MT) == 4 ? WARPS : 1][RG_MAXW];   // FP64 working row of a flagged row
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int gw = blockIdx.x * WARPS + wib, nw = gridDim.x * WARPS;
  for (int l = 0; l < nlev; l++) {
    const int b0 = lev_ptr[l], b1 = lev_ptr[l + 1];
    for (int idx = b0 + gw; idx < b1; idx += nw) {
      const int i = lev_rows[idx];
      const int b = rowptr[i], w = rowptr[i + 1] - b;
      const int q0 = lsort_ptr[i], nl = lsort_ptr[i + 1] - q0;
      for (int j = lane; j < w; j += 32) sval[wib][j] = A[b + j];
      // pivot rows of all L entries in one parallel batch; stage offsets by a warp scan
      int run = 0;
      for (int p0 = 0; p0 < nl; p0 += 32) {
        const int p = p0 + lane;
        int cnt = 0;
        if (p < nl) {
          const int k = lsort_col[q0 + p];
          const int rb = rowptr[k];
          cnt = rowptr[k + 1] - rb - 1;
          spiv[wib][p] = __ldcg(&LU[rb]);
          spos[wib][p] = lsort_pos[q0 + p];
          srow[wib][p] = rb + 1;
        }
        int v = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, v, o);
          if (lane >= o) v += t;
        }
        if (p < nl) sbeg[wib][p] = run + v - cnt;
        run += __shfl_sync(0xffffffffu, v, 31);
      }
      if (lane == 0) sbeg[wib][nl] = run;
      __syncwarp();
      const bool staged = run <= STAGE;
      if (staged) {
        for (int p = 0; p < nl; p++) {
          const int bk = srow[wib][p], dst = sbeg[wib][p], cnt = sbeg[wib][p + 1] - dst;
          const long long mo = fmap_off[q0 + p];
          for (int t = lane; t < cnt; t += 32) {
            stage[wib][dst + t] = __ldcg(&LU[bk + t]);
            smap[wib][dst + t] = fmap[mo + t];
          }
        }
      }
      __syncwarp();
      if (sizeof(MT) == 4 && fp64row && fp64row[i]) {
        // near-dry row: the elimination in FP64 (same order, same fill map)
        double* rw = svd[sizeof(MT) == 4 ? wib : 0];
        for (int j = lane; j < w; j += 32) rw[j] = (double)sval[wib][j];
        __syncwarp();
        for (int p = 0; p < nl; p++) {
          const int pp = spos[wib][p];
          const double factor = -rw[pp] / (double)spiv[wib][p];
          __syncwarp();
          if (lane == 0) rw[pp] = factor;
          const int dst = sbeg[wib][p], cnt = sbeg[wib][p + 1] - dst;
          const int bk = srow[wib][p];
          const long long mo = fmap_off[q0 + p];
          for (int t = lane; t < cnt; t += 32) {
            const int pos = staged ? smap[wib][dst + t] : fmap[mo + t];
            const double u = staged ? (double)stage[wib][dst + t] : (double)__ldcg(&LU[bk + t]);
            if (pos >= 0) rw[pos] = __dadd_rn(rw[pos], __dmul_rn(factor, u));
          }
          __syncwarp();
        }
        if (lane == 0 && fabs(rw[0]) < 1.0e-20) atomicOr(&err[0], 16);   // needs the repair path
        for (int j = lane; j < w; j += 32) __stcg(&LU[b + j], (MT)rw[j]);
        __syncwarp();
        continue;
      }
      for (int p = 0; p < nl; p++) {
        const int pp = spos[wib][p];
        const MT factor = -sval[wib][pp] / spiv[wib][p];
        __syncwarp();
        if (lane == 0) sval[wib][pp] = factor;
        const int dst = sbeg[wib][p], cnt = sbeg[wib][p + 1] - dst;
        if (staged) {
          for (int t = lane; t < cnt; t += 32) {
            const int pos = smap[wib][dst + t];
            if (pos >= 0) sval[wib][pos] = add_rn(sval[wib][pos], mul_rn(factor, stage[wib][dst + t]));
          }
        } else {
          const int bk = srow[wib][p];
          const long long mo = fmap_off[q0 + p];
          for (int t = lane; t < cnt; t += 32) {
            const int pos = fmap[mo + t];
            if (pos >= 0) sval[wib][pos] = add_rn(sval[wib][pos], mul_rn(factor, __ldcg(&LU[bk + t])));
          }
        }
        __syncwarp();
      }
      if (lane == 0 && fabs((double)sval[wib][0]) < 1.0e-20) atomicOr(&err[0], 16);   // needs the repair path
      for (int j = lane; j < w; j += 32) __stcg(&LU[b + j], sval[wib][j]);
      __syncwarp();
    }
    grid.sync();
  }
}

// gather the split triangular operands from the factors
template <class MT>
__global__ void k_split(int n, const int* rowptr, const MT* LU, int nl, const int* Lsrc, MT* Lv, int nu,
                        const int* Usrc, MT* Uv, MT* Dv) {
  int t = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  for (int q = t; q < nl; q += stride) Lv[q] = LU[Lsrc[q]];
  for (int q = t; q < nu; q += stride) Uv[q] = LU[Usrc[q]];
  for (int i = t; i < n; i += stride) Dv[i] = LU[rowptr[i]];
}

// ---- triangular solves (sync-free; the value is the ready flag) ------------
// LOWER: x_i = b_i + sum_{j<i} L_ij x_j      (Preco_ilu0.cpp:517-530)
// UPPER: x_i = (b_i - sum_{j>i} U_ij x_j) / D_i  (Preco_ilu0.cpp:964-980)
template <class VT, class MT, bool LOWER, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_trsv(int n, const int* __restrict__ ptr,
                                                     const int* __restrict__ col, const MT* __restrict__ val,
                                                     const MT* __restrict__ diag, const VT* b, VT* x, int* err,
                                                     const KrylovScalars* ks) {
  if (ks && ks->conv != 0) return;
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * WARPS + (threadIdx.x >> 5), nw = gridDim.x * WARPS;
  for (int t = gw; t < n; t += nw) {
    const int row = LOWER ? t : n - 1 - t;
    const int beg = ptr[row], end = ptr[row + 1];
    VT acc = 0;
    for (int q = beg + lane; q < end; q += 32) {
      const int c = col[q];
      const VT xv = wait_value<VT>(&x[c], err, LOWER ? 3 : 4, row, c);
      acc += (VT)val[q] * xv;
    }
    acc = warp_sum(acc);
    if (lane == 0) {
      VT v;
      if (LOWER)
        v = b[row] + acc;
      else
        v = (b[row] - acc) / (VT)diag[row];
      st_relaxed(&x[row], v);
    }
  }
}

// ---- BiCGStab vector steps (Bicgstab.cpp:158-347) ---------------------------
// restart test and beta (Bicgstab.cpp:164-203); ks->t1 holds (r0, ri)
__global__ void k_bicg_beta(KrylovScalars* ks) {
  ks->it += 1;
  const double temp1 = ks->t1;
  ks->beta = temp1 / ks->rho * ks->alfa / ks->omega;
  ks->rho = temp1;
}
// p = r + beta (p - omega v); also arms the preconditioner outputs
template <class VT>
__global__ void k_bicg_p(int n, VT* p, const VT* r, const VT* v, const KrylovScalars* ks, VT* s1, VT* s2) {
  const double beta = ks->beta, omega = ks->omega;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    p[i] = (VT)(r[i] + beta * (p[i] - omega * v[i]));
    s1[i] = sentinel<VT>();
    s2[i] = sentinel<VT>();
  }
}
__global__ void k_bicg_alfa(const double* partial, int nparts, KrylovScalars* ks) {
  double s = block_sum_fixed(partial, nparts);
  if (threadIdx.x == 0) {
    ks->t1 = s;
    ks->alfa = ks->rho / s;
  }
}
// r -= alfa v; partial ||r||^2
template <class VT>
__global__ void k_bicg_r1(int n, VT* r, const VT* v, const KrylovScalars* ks, double* partial) {
  const double alfa = ks->alfa;
  double acc[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    VT ri = (VT)(r[i] - alfa * v[i]);
    r[i] = ri;
    acc[0] += (double)ri * ri;
  }
  block_partials<1>(acc, partial);
}
// diff = ||r|| / ||r0||; best-iterate bookkeeping (Bicgstab.cpp:253-301)
__global__ void k_bicg_diff(const double* partial, int nparts, KrylovScalars* ks, double maxDiff, int maxIter) {
  double s = block_sum_fixed(partial, nparts);
  if (threadIdx.x == 0) {
    double diff = sqrt(s) / ks->l2r0;
    ks->diff = diff;
    int improved = diff < ks->accuracy;
    if (improved) ks->accuracy = diff;
    if (diff < maxDiff)
      ks->conv = 1;
    else if (ks->it >= maxIter)
      ks->conv = -1;
    else
      ks->conv = 0;
    ks->t2 = improved ? 1.0 : 0.0;
  }
}
// xm = x + alfa y when improved; x += alfa y when converged
template <class VT>
__global__ void k_bicg_xm(int n, const VT* x, const VT* y, VT* xm, VT* xfin, const KrylovScalars* ks) {
  const double alfa = ks->alfa;
  const bool improved = ks->t2 != 0.0;
  const int conv = ks->conv;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (improved) xm[i] = (VT)(x[i] + alfa * y[i]);
    if (conv == 1) xfin[i] = (VT)(x[i] + alfa * y[i]);
  }
}
__global__ void k_bicg_omega(const double* partial, int nparts, KrylovScalars* ks) {
  if (ks->conv != 0) return;
  double t1 = block_sum_fixed(partial, nparts);
  double t2 = block_sum_fixed(partial + nparts, nparts);
  if (threadIdx.x == 0) {
    ks->t1 = t1;
    ks->t2 = t2;
    ks->omega = t1 / t2;
  }
}
// x += alfa y + omega z; r -= omega t; partial (r0, r) for the next iteration
template <class VT>
__global__ void k_bicg_x(int n, VT* x, const VT* y, const VT* z, VT* r, const VT* t, const VT* r0,
                         const KrylovScalars* ks, double* partial) {
  if (ks->conv != 0) return;
  const double alfa = ks->alfa, omega = ks->omega;
  double acc[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] = (VT)(x[i] + (alfa * y[i] + omega * z[i]));
    VT ri = (VT)(r[i] - omega * t[i]);
    r[i] = ri;
    acc[0] += (double)r0[i] * ri;
  }
  block_partials<1>(acc, partial);
}
__global__ void k_fin_t1(const double* partial, int nparts, KrylovScalars* ks) {
  if (ks->conv != 0) return;
  double s = block_sum_fixed(partial, nparts);
  if (threadIdx.x == 0) ks->t1 = s;
}
// start: r0 = r = b - A x (x = 0 here, so r0 = r = b); ||r0||; (r0, r)
template <class VT>
__global__ void k_bicg_start(int n, const VT* b, const VT* t_, VT* r0, VT* r, VT* p, VT* v, double* partial) {
  double acc[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    VT ri = b[i] - t_[i];
    r0[i] = ri;
    r[i] = ri;
    p[i] = 0;
    v[i] = 0;
    acc[0] += (double)ri * ri;
  }
  block_partials<1>(acc, partial);
}
__global__ void k_bicg_init(const double* partial, int nparts, KrylovScalars* ks) {
  double s = block_sum_fixed(partial, nparts);
  if (threadIdx.x == 0) {
    ks->l2r0 = sqrt(s);
    ks->t1 = s;   // (r0, r) = ||r0||^2 for the first iteration
    ks->alfa = 1.0;
    ks->rho = 1.0;
    ks->omega = 1.0;
    ks->accuracy = 1.0;
    ks->it = 0;
    ks->conv = 0;
    ks->restarts = 0;
  }
}

template <class VT>
__global__ void k_fill_sentinel_if(VT* a, VT* b, int n, const KrylovScalars* ks) {
  if (ks->conv != 0) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    a[i] = sentinel<VT>();
    b[i] = sentinel<VT>();
  }
}
// restart (Bicgstab.cpp:176-198): t_ = A x already in t_
template <class VT>
__global__ void k_bicg_restart(int n, const VT* b, const VT* t_, VT* r0, VT* r, VT* p, VT* v, double* partial) {
  double acc[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    VT ri = b[i] - t_[i];
    r0[i] = ri;
    r[i] = ri;
    p[i] = 0;
    v[i] = 0;
    acc[0] += (double)ri * ri;
  }
  block_partials<1>(acc, partial);
}
__global__ void k_bicg_restart_fin(const double* partial, int nparts, KrylovScalars* ks) {
  double s = block_sum_fixed(partial, nparts);
  if (threadIdx.x == 0) {
    ks->t1 = s;
    ks->alfa = 1.0;
    ks->rho = 1.0;
    ks->omega = 1.0;
    ks->restarts += 1;
  }
}
// FP64 residual of the refinement loop: r = B - t; r32 = (float) r; partial ||r||^2
// t == nullptr: X = 0, the residual is B itself
__global__ void k_resid(int n, const double* B, const double* t, float* r32, double* partial) {
  double acc[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double r = t ? B[i] - t[i] : B[i];
    r32[i] = (float)r;
    acc[0] += r * r;
  }
  block_partials<1>(acc, partial);
}
__global__ void k_fin_to(const double* partial, int nparts, double* dst) {
  double s = block_sum_fixed(partial, nparts);
  if (threadIdx.x == 0) *dst = s;
}
__global__ void k_add_f(int n, const float* d, double* X) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) X[i] += (double)d[i];
}

}  // namespace

// =============================================================================
// host launchers

static int grid_for(rg_ctx* c, int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  int64_t cap = (int64_t)c->num_sms * 8;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

cudaError_t launch_scale(rg_ctx* c, double* scale_host) {
  const int nb = grid_for(c, c->neq, 256);
  k_sumsq<double><<<nb, 256, 0, rg_counted(c)>>>(c->B.p, c->neq, c->partial.p);
  k_scale_fin<<<1, 256, 0, rg_counted(c)>>>(c->partial.p, nb, c->ks.p);
  if (c->prec == RG_PREC_FP64)
    k_scale_apply<double><<<grid_for(c, c->nnz, 256), 256, 0, rg_counted(c)>>>(c->A64.p, c->nnz, c->B.p, c->neq, c->ks.p);
  else
    k_scale_apply<float><<<grid_for(c, c->nnz, 256), 256, 0, rg_counted(c)>>>(c->A32.p, c->nnz, c->B.p, c->neq, c->ks.p);
  c->d2h_bytes += sizeof(KrylovScalars);
  cudaError_t e = cudaMemcpyAsync(c->ks_host, c->ks.p, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, c->st);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) return e;
  *scale_host = c->ks_host->t1;
  return cudaGetLastError();
}

template <class MT, int WARPS>
static cudaError_t launch_factor_t(rg_ctx* c, const MT* A, MT* LU) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_factor<MT, WARPS>, WARPS * 32, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorLaunchOutOfResources;
  int blocks = per_sm * c->num_sms;
  int nrows_blocks = (c->neq + WARPS - 1) / WARPS;
  if (blocks > nrows_blocks) blocks = nrows_blocks;
  c->fepoch += 1;
  int n = c->neq;
  const int* rp = c->rowptr.p;
  const int* cl = c->col.p;
  const int* lp = c->lsort_ptr.p;
  const int* lpos = c->lsort_pos.p;
  int* ff = c->fflag.p;
  int ep = c->fepoch;
  int* err = c->dev_err.p;
  // LU starts as a copy of A: the zero-pivot repair re-derives later rows from it
  e = cudaMemcpyAsync(LU, A, c->nnz * sizeof(MT), cudaMemcpyDeviceToDevice, c->st);
  if (e != cudaSuccess) return e;
  void* args[] = {&n, &rp, &cl, &A, &LU, &lp, &lpos, &ff, &ep, &err};
  return cudaLaunchCooperativeKernel((void*)k_factor<MT, WARPS>, blocks, WARPS * 32, args, 0, rg_counted(c));
}

template <class MT, int WARPS>
static cudaError_t launch_factor_level_t(rg_ctx* c, const MT* A, MT* LU) {
  static int per_sm_dev[kMaxDevices] = {0};
  if (!device_slot_ok(c)) return cudaErrorInvalidDevice;
  int& per_sm = per_sm_dev[c->device];
  cudaError_t e;
  if (per_sm == 0) {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_factor_level<MT, WARPS>, WARPS * 32, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorLaunchOutOfResources;
    if (per_sm > 4) per_sm = 4;   // enough warps for a level; fewer blocks make the grid barrier cheaper
  }
  int blocks = per_sm * c->num_sms;
  int nlev = (int)c->waveL.lev_ptr.size() - 1;
  const int* lp = c->flev_ptr.p;
  const int* lr = c->flev_rows.p;
  const int* rp = c->rowptr.p;
  const int* cl = c->col.p;
  const int* lsp = c->lsort_ptr.p;
  const int* lspos = c->lsort_pos.p;
  int* err = c->dev_err.p;
  void* args[] = {&nlev, &lp, &lr, &rp, &cl, &A, &LU, &lsp, &lspos, &err};
  return cudaLaunchCooperativeKernel((void*)k_factor_level<MT, WARPS>, blocks, WARPS * 32, args, 0, rg_counted(c));
}

cudaError_t launch_factor(rg_ctx* c) {
  if (c->prec == RG_PREC_FP64) return launch_factor_t<double, 4>(c, c->A64.p, c->LU64.p);
  return launch_factor_t<float, 4>(c, c->A32.p, c->LU32.p);
}

template <class MT, int WARPS, int STAGE>
static cudaError_t launch_factor_level2_t(rg_ctx* c, const MT* A, MT* LU) {
  static int per_sm_dev[kMaxDevices] = {0};
  if (!device_slot_ok(c)) return cudaErrorInvalidDevice;
  int& per_sm = per_sm_dev[c->device];
  cudaError_t e;
  if (per_sm == 0) {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_factor_level2<MT, WARPS, STAGE>, WARPS * 32, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorLaunchOutOfResources;
  }
  const std::vector<int>& lp_h = c->waveL.lev_ptr;
  int maxw = 1;
  for (size_t l = 0; l + 1 < lp_h.size(); l++) maxw = std::max(maxw, lp_h[l + 1] - lp_h[l]);
  // enough warps for a typical level, few enough blocks for a cheap grid barrier
  int blocks = std::min(std::min(per_sm * c->num_sms, c->num_sms), (maxw + WARPS - 1) / WARPS);
  int nlev = (int)lp_h.size() - 1;
  const int* lp = c->flev_ptr.p;
  const int* lr = c->flev_rows.p;
  const int* rp = c->rowptr.p;
  const int* cl = c->col.p;
  const int* lsp = c->lsort_ptr.p;
  const int* lspos = c->lsort_pos.p;
  const int* lscol = c->lsort_col.p;
  const long long* fo = c->fmap_off.p;
  const short* fm = c->fmap.p;
  int* err = c->dev_err.p;
  const unsigned char* f64 = nullptr;
  if (sizeof(MT) == 4 && c->prec == RG_PREC_MIXED && c->fp64_pivot_depth > 0.0 && c->S.p && c->z.p) {
    cudaError_t e2 = launch_near_dry_rows(c);
    if (e2 != cudaSuccess) return e2;
    f64 = c->fp64row.p;
  }
  void* args[] = {&nlev, &lp, &lr, &rp, &cl, &A, &LU, &lsp, &lspos, &lscol, &fo, &fm, &err, &f64};
  return cudaLaunchCooperativeKernel((void*)k_factor_level2<MT, WARPS, STAGE>, blocks, WARPS * 32, args, 0, rg_counted(c));
}

// rows of the nodes shallower than the context's FP64-pivot depth (rg_set_fp64_pivots)
__global__ void k_near_dry_rows(int np, const double* __restrict__ S, const double* __restrict__ z,
                                const int* __restrict__ eqno, double depth, unsigned char* __restrict__ flag, int n) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < np; k += gridDim.x * blockDim.x) {
    const bool shallow = S[k] - z[k] < depth;
    for (int j = 0; j < 3; j++) {
      const int e = eqno[3 * k + j];
      if (e >= 0 && e < n) flag[e] = shallow ? 1 : 0;
    }
  }
}

cudaError_t launch_near_dry_rows(rg_ctx* c) {
  cudaError_t e = c->fp64row.alloc((size_t)c->neq);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(c->fp64row.p, 0, (size_t)c->neq, c->st);
  if (e != cudaSuccess) return e;
  k_near_dry_rows<<<grid_for(c, c->np, 256), 256, 0, rg_counted(c)>>>(c->np, c->S.p, c->z.p, c->eqno.p,
                                                                      c->fp64_pivot_depth, c->fp64row.p, c->neq);
  return cudaGetLastError();
}

cudaError_t launch_build_fmap(rg_ctx* c) {
  k_build_fmap<<<c->num_sms * 4, 256, 0, rg_counted(c)>>>(c->neq, c->rowptr.p, c->col.p, c->lsort_ptr.p, c->lsort_pos.p,
                                                   c->fmap_off.p, c->fmap.p);
  return cudaGetLastError();
}

// level-scheduled factorisation; returns cudaSuccess with err bit 16 set in the
// device error word when a pivot needs the repair path
cudaError_t launch_factor_level(rg_ctx* c) {
  if (c->fmap.p) {
    if (c->prec == RG_PREC_FP64) return launch_factor_level2_t<double, 4, 640>(c, c->A64.p, c->LU64.p);
    return launch_factor_level2_t<float, 4, 1280>(c, c->A32.p, c->LU32.p);
  }
  if (c->prec == RG_PREC_FP64) return launch_factor_level_t<double, 8>(c, c->A64.p, c->LU64.p);
  return launch_factor_level_t<float, 8>(c, c->A32.p, c->LU32.p);
}

cudaError_t launch_split(rg_ctx* c) {
  int nl = (int)c->Lcol.n, nu = (int)c->Ucol.n;
  int g = grid_for(c, c->nnz, 256);
  if (c->prec == RG_PREC_FP64)
    k_split<double><<<g, 256, 0, rg_counted(c)>>>(c->neq, c->rowptr.p, c->LU64.p, nl, c->Lsrc.p, c->Lv64.p, nu, c->Usrc.p,
                                          c->Uv64.p, c->Dv64.p);
  else
    k_split<float><<<g, 256, 0, rg_counted(c)>>>(c->neq, c->rowptr.p, c->LU32.p, nl, c->Lsrc.p, c->Lv32.p, nu, c->Usrc.p,
                                         c->Uv32.p, c->Dv32.p);
  return cudaGetLastError();
}

template <class VT, class MT, bool LOWER>
static cudaError_t launch_trsv_t(rg_ctx* c, const MT* val, const MT* diag, const VT* b, VT* x,
                                 const KrylovScalars* ks) {
  constexpr int W = 8;
  static int per_sm_dev[kMaxDevices] = {0};
  if (!device_slot_ok(c)) return cudaErrorInvalidDevice;
  int& per_sm = per_sm_dev[c->device];   // one cache per template instantiation and device
  cudaError_t e;
  if (per_sm == 0) {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trsv<VT, MT, LOWER, W>, W * 32, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorLaunchOutOfResources;
  }
  int blocks = per_sm * c->num_sms;
  int nrows_blocks = (c->neq + W - 1) / W;
  if (blocks > nrows_blocks) blocks = nrows_blocks;
  int n = c->neq;
  const int* ptr = LOWER ? c->Lptr.p : c->Uptr.p;
  const int* cl = LOWER ? c->Lcol.p : c->Ucol.p;
  int* err = c->dev_err.p;
  void* args[] = {&n, &ptr, &cl, &val, &diag, &b, &x, &err, &ks};
  return cudaLaunchCooperativeKernel((void*)k_trsv<VT, MT, LOWER, W>, blocks, W * 32, args, 0, rg_counted(c));
}

// y = M^-1 b with w as the intermediate; w and y must hold sentinels on entry
template <class VT, class MT>
static cudaError_t ilu_apply_t(rg_ctx* c, const MT* Lv, const MT* Uv, const MT* Dv, const VT* b, VT* w, VT* y,
                               const KrylovScalars* ks) {
  cudaError_t e = launch_trsv_t<VT, MT, true>(c, Lv, Dv, b, w, ks);
  if (e != cudaSuccess) return e;
  return launch_trsv_t<VT, MT, false>(c, Uv, Dv, w, y, ks);
}

template <class VT, class MT, class AT, int ND>
static void spmv_t(rg_ctx* c, const MT* A, const VT* x, VT* r, const VT* d1, int nb, const KrylovScalars* ks) {
  prof_begin(c, RG_PROF_SPMV);
  k_spmv<VT, MT, AT, ND><<<nb, 256, 0, rg_counted(c)>>>(c->neq, c->rowptr.p, c->col.p, A, x, r, d1, c->partial.p, ks);
  prof_end(c);
}

cudaError_t launch_spmv_d(rg_ctx* c, const double* x, double* r) {
  int nb = grid_for(c, c->neq * 16ll, 256);
  if (c->prec == RG_PREC_FP64)
    spmv_t<double, double, double, 0>(c, c->A64.p, x, r, nullptr, nb, nullptr);
  else
    spmv_t<double, float, double, 0>(c, c->A32.p, x, r, nullptr, nb, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_ilu_apply_d(rg_ctx* c, const double* b, double* x) {
  if (c->use_wave && c->prec != RG_PREC_MIXED) return launch_wave_solve(c, true, b, c->tmp.p, x, nullptr);
  int nb = grid_for(c, c->neq, 256);
  k_fill_sentinel<double><<<nb, 256, 0, rg_counted(c)>>>(c->tmp.p, c->neq);
  k_fill_sentinel<double><<<nb, 256, 0, rg_counted(c)>>>(x, c->neq);
  if (c->prec == RG_PREC_FP64)
    return ilu_apply_t<double, double>(c, c->Lv64.p, c->Uv64.p, c->Dv64.p, b, c->tmp.p, x, nullptr);
  return ilu_apply_t<double, float>(c, c->Lv32.p, c->Uv32.p, c->Dv32.p, b, c->tmp.p, x, nullptr);
}

// ---- BiCGStab ---------------------------------------------------------------
// One Krylov solve A x = b, x = 0 start, in vector type VT with matrix MT.
// The second half of every iteration is predicated on the device flag
// ks->conv == 0, so the host synchronises once per iteration.
template <class VT, class MT, class AT>
static rg_status bicgstab_t(rg_ctx* c, const MT* A, const MT* Lv, const MT* Uv, const MT* Dv, const VT* b, VT* x,
                            VT* r0, VT* ri, VT* vi, VT* pi, VT* yi, VT* zi, VT* ti, VT* xm, VT* w,
                            int maxIter, double maxDiff, int* iters, double* acc) {
  const int n = c->neq;
  const int nb = grid_for(c, n, 256);
  const int nbs = grid_for(c, n * 16ll, 256);
  KrylovScalars* ks = c->ks.p;
  double* part = c->partial.p;
  cudaError_t e;
#define CK(x)                                        \
  do {                                               \
    e = (x);                                         \
    if (e != cudaSuccess) return rg_cuda(c, e, #x);  \
  } while (0)
  k_fill<VT><<<nb, 256, 0, rg_counted(c)>>>(x, n, (VT)0);
  k_fill<VT><<<nb, 256, 0, rg_counted(c)>>>(xm, n, (VT)0);
  k_fill<VT><<<nb, 256, 0, rg_counted(c)>>>(ti, n, (VT)0);   // t_ = A x = 0 for x = 0
  k_bicg_start<VT><<<nb, 256, 0, rg_counted(c)>>>(n, b, ti, r0, ri, pi, vi, part);
  k_bicg_init<<<1, 256, 0, rg_counted(c)>>>(part, nb, ks);
  CK(cudaGetLastError());
  int it = 0;
  rg_status st = RG_OK;
  for (;;) {
    k_bicg_beta<<<1, 1, 0, rg_counted(c)>>>(ks);
    k_bicg_p<VT><<<nb, 256, 0, rg_counted(c)>>>(n, pi, ri, vi, ks, w, yi);
    if (c->use_wave)
      CK(launch_wave_solve(c, sizeof(VT) == 8, pi, w, yi, nullptr));
    else
      CK((ilu_apply_t<VT, MT>(c, Lv, Uv, Dv, pi, w, yi, nullptr)));
    spmv_t<VT, MT, AT, 1>(c, A, yi, vi, r0, nbs, nullptr);
    k_bicg_alfa<<<1, 256, 0, rg_counted(c)>>>(part, nbs, ks);
    k_bicg_r1<VT><<<nb, 256, 0, rg_counted(c)>>>(n, ri, vi, ks, part);
    k_bicg_diff<<<1, 256, 0, rg_counted(c)>>>(part, nb, ks, maxDiff, maxIter);
    k_bicg_xm<VT><<<nb, 256, 0, rg_counted(c)>>>(n, x, yi, xm, x, ks);
    // second half, skipped on the device once converged or out of iterations
    k_fill_sentinel_if<VT><<<nb, 256, 0, rg_counted(c)>>>(w, zi, n, ks);
    if (c->use_wave)
      CK(launch_wave_solve(c, sizeof(VT) == 8, ri, w, zi, ks));
    else
      CK((ilu_apply_t<VT, MT>(c, Lv, Uv, Dv, ri, w, zi, ks)));
    spmv_t<VT, MT, AT, 2>(c, A, zi, ti, ri, nbs, ks);
    k_bicg_omega<<<1, 256, 0, rg_counted(c)>>>(part, nbs, ks);
    k_bicg_x<VT><<<nb, 256, 0, rg_counted(c)>>>(n, x, yi, zi, ri, ti, r0, ks, part);
    k_fin_t1<<<1, 256, 0, rg_counted(c)>>>(part, nb, ks);
    c->d2h_bytes += sizeof(KrylovScalars);
    CK(cudaMemcpyAsync(c->ks_host, ks, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    it = c->ks_host->it;
    if (c->trace >= 3) {
      int eh[4];
      CK(cudaMemcpy(eh, c->dev_err.p, sizeof(eh), cudaMemcpyDeviceToHost));
      fprintf(stderr, "[rg]     bicg it=%d diff=%.3e t1=%.3e rho=%.3e alfa=%.3e omega=%.3e conv=%d err=%d/%d/%d/%d\n",
              it, c->ks_host->diff, c->ks_host->t1, c->ks_host->rho, c->ks_host->alfa, c->ks_host->omega,
              c->ks_host->conv, eh[0], eh[1], eh[2], eh[3]);
    }
    if (c->ks_host->conv == 1) break;
    if (c->ks_host->conv == -1) {
      CK(cudaMemcpyAsync(x, xm, n * sizeof(VT), cudaMemcpyDeviceToDevice, c->st));
      st = RG_NOT_CONVERGED;
      break;
    }
    if (!(c->ks_host->diff == c->ks_host->diff) || !(c->ks_host->t1 == c->ks_host->t1)) {
      st = RG_ERR_NONFINITE;
      break;
    }
    if (fabs(c->ks_host->t1) < 1.0e-30) {
      // restart (Bicgstab.cpp:174-199): r = r0 = b - A x, p = v = 0, scalars reset
      spmv_t<VT, MT, AT, 0>(c, A, x, ti, nullptr, nbs, nullptr);
      k_bicg_restart<VT><<<nb, 256, 0, rg_counted(c)>>>(n, b, ti, r0, ri, pi, vi, part);
      k_bicg_restart_fin<<<1, 256, 0, rg_counted(c)>>>(part, nb, ks);
      CK(cudaGetLastError());
    }
  }
#undef CK
  if (iters) *iters = it;
  if (acc) *acc = c->ks_host->accuracy;
  return st;
}

rg_status run_bicgstab(rg_ctx* c, int maxIter, double maxDiff, int* iters, double* acc) {
  if (c->prec == RG_PREC_FP64)
    return bicgstab_t<double, double, double>(c, c->A64.p, c->Lv64.p, c->Uv64.p, c->Dv64.p, c->B.p, c->X.p, c->r0.p,
                                              c->ri.p, c->vi.p, c->pi.p, c->yi.p, c->zi.p, c->ti.p, c->xm.p, c->tmp.p,
                                              maxIter, maxDiff, iters, acc);
  if (c->prec == RG_PREC_REF32)
    return bicgstab_t<double, float, double>(c, c->A32.p, c->Lv32.p, c->Uv32.p, c->Dv32.p, c->B.p, c->X.p, c->r0.p,
                                             c->ri.p, c->vi.p, c->pi.p, c->yi.p, c->zi.p, c->ti.p, c->xm.p, c->tmp.p,
                                             maxIter, maxDiff, iters, acc);
  // mixed: FP32 BiCGStab on the correction equation inside FP64 iterative
  // refinement -- the residual r = B - A X is formed with FP64 accumulation
  const int n = c->neq;
  const int nb = grid_for(c, n, 256);
  const int nbs = grid_for(c, n * 16ll, 256);
  cudaError_t e;
  k_fill<double><<<nb, 256, 0, rg_counted(c)>>>(c->X.p, n, 0.0);
  double bnorm = -1.0, last = 1.0;
  int total = 0;
  rg_status st = RG_NOT_CONVERGED;
  for (int refine = 0; refine < 12; refine++) {
    if (refine > 0) spmv_t<double, float, double, 0>(c, c->A32.p, c->X.p, c->tt.p, nullptr, nbs, nullptr);
    k_resid<<<nb, 256, 0, rg_counted(c)>>>(n, c->B.p, refine > 0 ? c->tt.p : nullptr, c->f_b.p, c->partial.p);
    k_fin_to<<<1, 256, 0, rg_counted(c)>>>(c->partial.p, nb, &c->ks.p->t2);
    c->d2h_bytes += sizeof(KrylovScalars);
    e = cudaMemcpyAsync(c->ks_host, c->ks.p, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) return rg_cuda(c, e, "mixed residual");
    const double rn = sqrt(c->ks_host->t2);
    if (!(rn == rn)) return RG_ERR_NONFINITE;
    if (bnorm < 0) bnorm = rn;
    last = (bnorm > 0) ? rn / bnorm : 0.0;
    if (rn <= maxDiff * bnorm || bnorm == 0.0) {
      st = RG_OK;
      break;
    }
    if (total >= maxIter) break;
    // inner tolerance: what FP32 can deliver, never tighter than what is missing
    double inner = 1.0e-5, need = maxDiff * bnorm / rn;
    if (need > inner) inner = need;
    int its = 0;
    double a2 = 0;
    rg_status s2 = bicgstab_t<float, float, float>(c, c->A32.p, c->Lv32.p, c->Uv32.p, c->Dv32.p, c->f_b.p, c->f_x.p,
                                                   c->f_r0.p, c->f_ri.p, c->f_vi.p, c->f_pi.p, c->f_yi.p, c->f_zi.p,
                                                   c->f_ti.p, c->f_xm.p, c->f_w.p, maxIter - total, inner, &its,
                                                   &a2);
    total += its;
    if (s2 != RG_OK && s2 != RG_NOT_CONVERGED) return s2;
    k_add_f<<<nb, 256, 0, rg_counted(c)>>>(n, c->f_x.p, c->X.p);
    e = cudaGetLastError();
    if (e != cudaSuccess) return rg_cuda(c, e, "mixed update");
  }
  if (iters) *iters = total;
  if (acc) *acc = last;
  return st;
}

// y = M^-1 b on float vectors with the FP32 factors of a mixed-precision context: the
// inner solve of the mixed BiCGStab (wavefront kernels, or the dependency-driven ones)
cudaError_t launch_ilu_apply_f(rg_ctx* c, const float* b, float* w, float* y) {
  if (c->use_wave) return launch_wave_solve(c, false, b, w, y, nullptr);
  int nb = grid_for(c, c->neq, 256);
  k_fill_sentinel<float><<<nb, 256, 0, rg_counted(c)>>>(w, c->neq);
  k_fill_sentinel<float><<<nb, 256, 0, rg_counted(c)>>>(y, c->neq);
  return ilu_apply_t<float, float>(c, c->Lv32.p, c->Uv32.p, c->Dv32.p, b, w, y, nullptr);
}

// y = M^-1 b on double vectors with a caller-chosen intermediate w (n values):
// the same kernels as launch_ilu_apply_d, which uses the context's own vector
cudaError_t launch_ilu_apply_w(rg_ctx* c, const double* b, double* w, double* x) {
  if (c->use_wave && c->prec != RG_PREC_MIXED) return launch_wave_solve(c, true, b, w, x, nullptr);
  int nb = grid_for(c, c->neq, 256);
  k_fill_sentinel<double><<<nb, 256, 0, rg_counted(c)>>>(w, c->neq);
  k_fill_sentinel<double><<<nb, 256, 0, rg_counted(c)>>>(x, c->neq);
  if (c->prec == RG_PREC_FP64)
    return ilu_apply_t<double, double>(c, c->Lv64.p, c->Uv64.p, c->Dv64.p, b, w, x, nullptr);
  return ilu_apply_t<double, float>(c, c->Lv32.p, c->Uv32.p, c->Dv32.p, b, w, x, nullptr);
}
