// Wavefront ILU(0) triangular solves: one CTA walks the dependency levels of
// PRECO_ILU0::Solve (Preco_ilu0.cpp:517-530 forward, 964-980 backward) in the
// reference's equation order.
//
// The solves are latency-bound chains (a level holds a few hundred rows, the
// depth is hundreds to thousands of levels), so the kernel keeps the whole
// chain on one SM and takes global-memory latency off the critical path:
//   * the rows of every level are packed host-side into a contiguous image per
//     chunk (row meta, right-hand side, diagonal, warp slices of entries);
//   * one producer thread streams the images of the next chunks into NST
//     shared-memory stages with cp.async.bulk (TMA bulk copies) completing on
//     mbarriers; the next chunk descriptor is loaded while it waits;
//   * solution values live in a shared-memory ring indexed by level-order
//     position, plus pinned slots for the most-read far sources; the host
//     decides per entry where its source is (else it is read from global memory);
//   * one consumer thread per row; chunks are separated by a named barrier.
// Levels too large for a stage are split into consecutive chunks (rows of one
// level do not depend on each other).
//
// Solves whose summation order is free (FP32 and FP64) use split layouts: entries whose
// source lies outside the ring and the pinned slots -- about a fifth of them
// on the 4M-triangle river -- are not in the images.  The same cooperative
// launch then holds helper blocks: a helper takes a future chunk once the
// wavefront block has published (progress word) that the chunk's far sources
// are solved, sums the chunk's far contributions into its right-hand side in
// the image and flags the chunk; the producer stages a chunk only after its
// flag.  Far sources lie at least the ring's reach (~31 chunks) behind, so the
// helpers work ahead of the wavefront and the far reads leave its critical
// path.  The progress word is published by a warp of its own (its GPU-scope
// release stays off the consumers' path), the producer reads the helpers'
// flags in batches, and split images hold 16-bit source slots (every source
// is a ring or pinned slot).  All waits are bounded.

#include "rg_internal.cuh"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>

namespace {

constexpr int kThreads = kWaveThreads;
constexpr int kConsumers = kWaveRows;   // warps 0-15; warp 16 produces, warp 17 publishes
// a chunk's far sources lie at least the ring's reach (kWaveRing - kWaveRows
// positions, so more than kWaveMaxStages chunks) before it: the wavefront block
// has finished them before its producer stages the chunk, so a helper can always
// complete a chunk the producer waits for
static_assert(kWaveRing - kWaveRows >= kWaveMaxStages * kWaveRows, "ring too small for the helper blocks");
static_assert(kWaveRing64 - kWaveRows >= kWaveMaxStages * kWaveRows, "ring too small for the helper blocks");
static_assert(kWaveStages32 <= kWaveMaxStages && kWaveStages64 <= kWaveMaxStages, "stage table");
constexpr long long kMbarSpin = 1ll << 26;
constexpr long long kFlagSpin = 1ll << 24;   // polls of a global flag (~10 s at L2 latency)
constexpr long long kDrainSpin = 1ll << 16;
// launch options of the wavefront solve, packed in one int: bits 0-7 the chunk
// images prefetched into L2 ahead of the stages, bit 8 progress published by the
// publisher warp (split layouts), bits 9-13 the chunk flags the producer reads
// ahead in one batch (split layouts; 0 = one acquire per chunk), bits 14-15 the bulk
// copies per chunk image minus one, bits 16-23 how many chunks ahead of the wavefront
// the helper blocks prefetch images into L2 (split layouts; 0 = none, else at least
// the stage count), bit 31 stage waits that poll mbarrier.test_wait instead of
// suspending in try_wait
constexpr int kWavePrefetch = 0, kWavePublish = 1, kWaveScan = 16, kWavePieces = 1, kWaveL2Ahead = 0,
              kWaveSpin = 0;
static_assert(kWaveScan < 32, "scan width field");

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// non-blocking test of an mbarrier phase (no suspension: the caller spins)
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// global -> shared bulk copy completing on an mbarrier (16-byte aligned, size % 16 == 0);
// the image is read once per solve, so its lines are marked first to leave L2 and the
// solution vector (read back for far sources) stays resident
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar, uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(pol)
      : "memory");
}

// global -> L2 prefetch of a chunk image (16-byte aligned, size % 16 == 0)
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, int bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

}  // namespace

namespace {

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// bounded wait on an mbarrier phase; false when the bound ran out.  spin: poll with
// test_wait instead of the suspending try_wait (the waiting thread notices the phase
// change sooner)
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, long long limit = kMbarSpin,
                                                  bool spin = false) {
  long long it = 0;
  while (!(spin ? mbar_test_wait(bar, parity) : mbar_try_wait(bar, parity))) {
    if (++it > limit) return false;
  }
  return true;
}

// a stage wait that ran out: error bit 8, and (first failure only) the kernel tag and the
// chunk, read by the host's device-error check
__device__ __forceinline__ void wave_wait_failed(int* err, int tag, int chunk) {
  if (atomicCAS(&err[1], 0, tag) == 0) {
    err[2] = chunk;
    err[3] = -1;
  }
  atomicOr(err, 8);
}

// bounded wait that also gives up when the producer has aborted (checked every 1024 polls)
__device__ __forceinline__ bool mbar_wait_abortable(uint64_t* bar, unsigned parity, volatile int* abort_flag,
                                                    bool spin = false) {
  long long it = 0;
  while (!(spin ? mbar_test_wait(bar, parity) : mbar_try_wait(bar, parity))) {
    if (++it > kMbarSpin) return false;
    if ((it & 1023) == 0 && *abort_flag) return false;
  }
  return true;
}

__device__ __forceinline__ void consumers_sync() {
  asm volatile("bar.sync 1, %0;" ::"r"(kConsumers) : "memory");
}

// Warp-specialised wavefront solve: warp 16 (one elected lane) is the producer
// that streams chunk images into NST shared-memory stages with cp.async.bulk;
// warps 0..15 consume the stages in order, one dependency-level chunk at a
// time, one row per thread, synchronising on a named barrier between chunks;
// with split layouts one lane of warp 17 publishes the consumers' progress to
// the helper blocks.
//
// Row r of a chunk is solved by consumer thread r: its entries sit in its warp
// slice column by column, so the 32 lanes of a warp read consecutive words.
// The sum runs over the row's entries in the factor's order with separately
// rounded products and sums, as PRECO_ILU0::Solve does (Preco_ilu0.cpp:520-528
// forward from b, 964-977 backward, then the division by the diagonal).
template <class VT>
__device__ __forceinline__ VT fmul(VT a, VT b);
template <>
__device__ __forceinline__ float fmul<float>(float a, float b) { return __fmul_rn(a, b); }
template <>
__device__ __forceinline__ double fmul<double>(double a, double b) { return __dmul_rn(a, b); }
template <class VT>
__device__ __forceinline__ VT fadd(VT a, VT b);
template <>
__device__ __forceinline__ float fadd<float>(float a, float b) { return __fadd_rn(a, b); }
template <>
__device__ __forceinline__ double fadd<double>(double a, double b) { return __dadd_rn(a, b); }

// one entry of a row sum: acc + v*x (ADD) or acc - v*x, with separately rounded
// product and sum as the reference does, or (FUSED) one fused multiply-add -- the
// FP64 split solves, whose order already differs from the reference's and whose
// rate on this GPU is bound by the FP64 pipe
template <class VT, bool ADD, bool FUSED>
__device__ __forceinline__ VT row_term(VT acc, VT v, VT x) {
  if (FUSED) return ADD ? fma(v, x, acc) : fma(-v, x, acc);
  return ADD ? fadd(acc, fmul(v, x)) : fadd(acc, -fmul(v, x));
}

// the solution value at source slot s: ring or pinned slot, or (FAR layouts
// only) -(row + 1) for a row read back from global memory
template <class VT, bool FAR>
__device__ __forceinline__ VT source_value(const VT* vals, const VT* x, int s) {
  if (FAR) return s >= 0 ? vals[s] : __ldcg(&x[-s - 1]);
  return vals[s];
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_relaxed_s32(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
// with the relaxed loads before it, an acquire of what they observed
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ int ld_acquire_s32(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_release_s32(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_release_cta_shared(int* p, int v) {
  asm volatile("st.release.cta.shared::cta.s32 [%0], %1;" ::"r"(smem_addr(p)), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_acquire_cta_shared(const int* p) {
  int v;
  asm volatile("ld.acquire.cta.shared::cta.s32 %0, [%1];" : "=r"(v) : "r"(smem_addr(p)) : "memory");
  return v;
}
// generic-proxy writes to global memory before async-proxy (TMA) reads of it
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

// Helper block of a split solve: for its chunks k = h, h + H, ... (h = block - 1,
// H = helpers) with far entries, wait until the wavefront block has solved the
// chunk's far sources, add the far contributions of every row (one thread per
// row) to the row's right-hand side in the image, and flag the chunk.
template <class VT, bool LOWER>
__device__ void wave_helper(int nchunks, const WaveChunk* __restrict__ chunks, unsigned char* img,
                            const VT* __restrict__ x, int* err, const long long* __restrict__ far_ptr,
                            const int* __restrict__ far_src, const VT* __restrict__ far_val,
                            const int* __restrict__ bidx, int* chunk_ready, const unsigned long long* progress,
                            unsigned epoch, int l2_ahead) {
  __shared__ int s_go;
  const int H = gridDim.x - 1;
  VT* bimg = reinterpret_cast<VT*>(img);
  for (int k = blockIdx.x - 1; k < nchunks; k += H) {
    const WaveChunk ch = chunks[k];
    // wait for the chunk's far sources, and (l2_ahead > 0) until the wavefront is
    // l2_ahead chunks short of the chunk: then its image goes into L2 from this SM,
    // so that the wavefront block's copy reads it from L2 rather than DRAM
    long long dep = ch.far_dep + 1;
    if (l2_ahead > 0) dep = std::max(dep, (long long)k - l2_ahead);
    if (dep <= 0 && ch.far_dep < 0) {   // nothing to wait for or add: flagged at once
      if (threadIdx.x == 0) st_release_s32(&chunk_ready[k], (int)epoch);
      continue;
    }
    if (threadIdx.x == 0) {
      const unsigned long long need = ((unsigned long long)epoch << 32) | (unsigned long long)std::max(dep, 0ll);
      long long it = 0;
      int go = 1;
      while (ld_acquire_u64(progress) < need) {
        if ((++it & 1023) == 0 && *reinterpret_cast<volatile int*>(err) != 0) {
          go = 0;
          break;
        }
        if (it > kFlagSpin) {
          wave_wait_failed(err, LOWER ? 32 : 33, k);
          go = 0;
          break;
        }
      }
      s_go = go;
      if (go && l2_ahead > 0) bulk_prefetch_l2(img + ch.img_off, ch.img_bytes);
    }
    __syncthreads();
    if (!s_go) return;
    if (ch.far_dep < 0) {
      if (threadIdx.x == 0) st_release_s32(&chunk_ready[k], (int)epoch);
      continue;
    }
    for (int r = threadIdx.x; r < ch.nrows; r += blockDim.x) {
      const int p = ch.pos0 + r;
      const long long e0 = far_ptr[p], e1 = far_ptr[p + 1];
      if (e0 == e1) continue;
      VT sum = 0;
      for (long long e = e0; e < e1; e++) sum += far_val[e] * __ldcg(&x[far_src[e]]);
      const int bi = bidx[p];
      bimg[bi] = LOWER ? bimg[bi] + sum : bimg[bi] - sum;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      fence_proxy_async_global();
      st_release_s32(&chunk_ready[k], (int)epoch);
    }
  }
}

template <class VT, bool LOWER, int G, bool FAR, bool SPLIT>
__global__ void __launch_bounds__(kThreads, 1)
    k_trsv_wave(int nchunks, const WaveChunk* __restrict__ chunks, unsigned char* img, VT* __restrict__ x,
                int stage_bytes, int* err, const KrylovScalars* ks, const long long* __restrict__ far_ptr,
                const int* __restrict__ far_src, const VT* __restrict__ far_val, const int* __restrict__ bidx,
                int* chunk_ready, unsigned long long* progress, unsigned epoch, int tune) {
  if (ks && ks->conv != 0) return;
  if (SPLIT && blockIdx.x > 0) {
    wave_helper<VT, LOWER>(nchunks, chunks, img, x, err, far_ptr, far_src, far_val, bidx, chunk_ready, progress,
                           epoch, (tune >> 16) & 0xff);
    return;
  }
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int RING = wave_ring(sizeof(VT)), PIN = wave_pin(sizeof(VT)), nst = wave_stages(sizeof(VT));
  constexpr bool kFused = SPLIT && sizeof(VT) == 8;
  using SlotT = typename std::conditional<SPLIT, unsigned short, int>::type;   // 16-bit slots in split layouts
  constexpr int kSlot = (int)sizeof(SlotT);
  constexpr int kStride = kWaveSlice * (kSlot + (int)sizeof(VT));   // bytes per entry column of a slice
  static_assert((RING & (RING - 1)) == 0, "ring size must be a power of two");
  static_assert(G == 1 || G == 2 || G == 4, "threads per row");
  // solution values: ring slots [0, RING), pinned long-range slots [RING, RING + PIN)
  VT* vals = reinterpret_cast<VT*>(smem);
  unsigned char* stage0 = smem + (RING + PIN) * sizeof(VT);
  __shared__ __align__(8) uint64_t full[kWaveMaxStages];
  __shared__ __align__(8) uint64_t empty[kWaveMaxStages];
  __shared__ WaveChunk sdesc[kWaveMaxStages];
  __shared__ int s_issued;   // copies the producer has started
  __shared__ int s_abort;    // set by a consumer whose wait ran out (read after a barrier)
  __shared__ int s_done;     // chunks the consumers have completed (publisher mode)
  const int tid = threadIdx.x;
  const int prefetch = tune & 255;
  const bool publish = SPLIT && ((tune >> 8) & 1) != 0;
  const int scan = (tune >> 9) & 31;
  const int pieces = 1 + ((tune >> 14) & 3);   // 1..4 bulk copies per chunk image
  const bool spin = ((tune >> 31) & 1) != 0;    // stage waits poll test_wait
  if (tid == 0) {
    for (int s = 0; s < nst; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    s_issued = 0;
    s_abort = 0;
    s_done = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  volatile int* v_issued = &s_issued;
  volatile int* v_abort = &s_abort;

  if (tid >= kConsumers) {
    // ---- producer ------------------------------------------------------------
    if (tid == kConsumers && nchunks > 0) {
      const uint64_t pol = policy_evict_first();
      int ready_hi = -1;   // split layouts: chunks up to this one are known to be flagged
      WaveChunk next = chunks[0];
      // the images of the first chunks into L2 ahead of their stages
      for (int q = 1; q < prefetch && q < nchunks; q++) bulk_prefetch_l2(img + chunks[q].img_off, chunks[q].img_bytes);
      for (int k = 0; k < nchunks; k++) {
        const int s = k % nst;
        const WaveChunk ch = next;
        if (k + 1 < nchunks) next = chunks[k + 1];   // descriptor load overlaps the wait below
        if (prefetch > 0 && k + prefetch < nchunks) {
          const WaveChunk ahead = chunks[k + prefetch];
          bulk_prefetch_l2(img + ahead.img_off, ahead.img_bytes);
        }
        if (k >= nst && !mbar_wait_bounded(&empty[s], (unsigned)(((k / nst) - 1) & 1), kMbarSpin, spin)) {
          wave_wait_failed(err, LOWER ? 30 : 31, k);
          *v_abort = 1;
          break;
        }
        if (*v_abort) break;
        if (SPLIT && scan > 0 && k > ready_hi) {
          // the helpers' far sums must be in the images before they are staged: wait for
          // chunk k's flag, then read the flags of the next chunks in one batch of
          // independent loads; one fence makes them all acquires
          long long it = 0;
          bool ok = true;
          while (ld_relaxed_s32(&chunk_ready[k]) != (int)epoch) {
            if ((++it & 1023) == 0 && (*reinterpret_cast<volatile int*>(err) != 0 || *v_abort)) {
              ok = false;
              break;
            }
            if (it > kFlagSpin) {
              wave_wait_failed(err, LOWER ? 34 : 35, k);
              ok = false;
              break;
            }
          }
          if (!ok) {
            *v_abort = 1;
            break;
          }
          int f[31];
#pragma unroll
          for (int q = 0; q < 31; q++)
            if (q < scan - 1 && k + 1 + q < nchunks) f[q] = ld_relaxed_s32(&chunk_ready[k + 1 + q]);
          int hi = k;
#pragma unroll
          for (int q = 0; q < 31; q++)
            if (q < scan - 1 && k + 1 + q < nchunks && hi == k + q && f[q] == (int)epoch) hi = k + 1 + q;
          fence_acq_rel_gpu();
          fence_proxy_async_global();
          ready_hi = hi;
        } else if (SPLIT && scan == 0 && ch.far_dep >= 0) {
          // the helper's far sums must be in the image before it is staged
          long long it = 0;
          bool ok = true;
          while (ld_acquire_s32(&chunk_ready[k]) != (int)epoch) {
            if ((++it & 1023) == 0 && (*reinterpret_cast<volatile int*>(err) != 0 || *v_abort)) {
              ok = false;
              break;
            }
            if (it > kFlagSpin) {
              wave_wait_failed(err, LOWER ? 34 : 35, k);
              ok = false;
              break;
            }
          }
          if (!ok) {
            *v_abort = 1;
            break;
          }
          fence_proxy_async_global();
        }
        sdesc[s] = ch;
        *v_issued = k + 1;
        fence_proxy_async();   // earlier generic reads of the stage precede the async refill
        mbar_expect_tx(&full[s], (unsigned)ch.img_bytes);
        // the image in `pieces` bulk copies of 16-byte multiples, all completing on the stage's barrier
        const unsigned piece = ((unsigned)((ch.img_bytes + pieces - 1) / pieces) + 15u) & ~15u;
        for (unsigned off = 0; off < (unsigned)ch.img_bytes; off += piece)
          bulk_g2s(stage0 + s * (size_t)stage_bytes + off, img + ch.img_off + off,
                   min(piece, (unsigned)ch.img_bytes - off), &full[s], pol);
      }
    } else if (publish && tid == kConsumers + 32) {
      // ---- publisher: the consumers' chunk count to the helper blocks -----------
      // The consumers' x stores precede their barrier and thread 0's CTA-scope
      // release of s_done; this thread's acquire of it and its GPU-scope release of
      // the progress word carry them to the helpers (the fence stays off the
      // consumers' path).  Bounded: ends at the last chunk, on an abort or an error.
      int seen = 0;
      long long it = 0;
      while (seen < nchunks) {
        const int d = ld_acquire_cta_shared(&s_done);
        if (d > seen) {
          seen = d;
          st_release_u64(progress, ((unsigned long long)epoch << 32) | (unsigned long long)d);
          it = 0;
        } else if ((++it & 1023) == 0 && (*v_abort || *reinterpret_cast<volatile int*>(err) != 0 || it > kMbarSpin)) {
          break;
        }
      }
    }
    return;
  }

  // ---- consumers -------------------------------------------------------------
  const int lane = tid & 31;
  for (int k = 0; k < nchunks; k++) {
    const int s = k % nst;
    const bool got = mbar_wait_abortable(&full[s], (unsigned)((k / nst) & 1), v_abort, spin);
    if (!__all_sync(0xffffffffu, got)) {   // warp-uniform: the row sums below shuffle across lanes
      if (lane == 0) wave_wait_failed(err, LOWER ? 30 : 31, k);
      *v_abort = 1;
    } else {
      const WaveChunk ch = sdesc[s];
      const unsigned char* st = stage0 + s * (size_t)stage_bytes;
      const int r = tid / G, g = tid & (G - 1);
      const bool valid = r < ch.nrows;
      int4 mt = make_int4(0, 0, 0, -1);   // row, entries, slice offset, pinned slot
      VT acc = 0;
      if (valid) {
        mt = reinterpret_cast<const int4*>(st)[r];
        if (G == 1) acc = reinterpret_cast<const VT*>(st + ch.b_off)[r];
        const unsigned char* col = st + mt.z;
        const SlotT* src = reinterpret_cast<const SlotT*>(col) + lane;
        const VT* val = reinterpret_cast<const VT*>(col + kSlot * kWaveSlice) + lane;
        constexpr int kS = kStride / kSlot;             // column stride in slots
        constexpr int kV = kStride / (int)sizeof(VT);   // column stride in values
        const int cnt = mt.y > g ? (mt.y - g + G - 1) / G : 0;   // this lane's entries g, g+G, ...
        int t = 0;
        // batches of 8: all sources and values first, then the gathers, then the sums in order
        for (; t + 8 <= cnt; t += 8) {
          int sq[8];
          VT vq[8], xq[8];
#pragma unroll
          for (int q = 0; q < 8; q++) {
            sq[q] = src[(t + q) * kS];
            vq[q] = val[(t + q) * kV];
          }
#pragma unroll
          for (int q = 0; q < 8; q++) xq[q] = source_value<VT, FAR>(vals, x, sq[q]);
#pragma unroll
          for (int q = 0; q < 8; q++) acc = row_term<VT, (LOWER || G > 1), kFused>(acc, vq[q], xq[q]);
        }
        if (t + 4 <= cnt) {
          int sq[4];
          VT vq[4], xq[4];
#pragma unroll
          for (int q = 0; q < 4; q++) {
            sq[q] = src[(t + q) * kS];
            vq[q] = val[(t + q) * kV];
          }
#pragma unroll
          for (int q = 0; q < 4; q++) xq[q] = source_value<VT, FAR>(vals, x, sq[q]);
#pragma unroll
          for (int q = 0; q < 4; q++) acc = row_term<VT, (LOWER || G > 1), kFused>(acc, vq[q], xq[q]);
          t += 4;
        }
        for (; t < cnt; t++) {
          const int s0 = src[t * kS];
          const VT v0 = val[t * kV];
          const VT x0 = source_value<VT, FAR>(vals, x, s0);
          acc = row_term<VT, (LOWER || G > 1), kFused>(acc, v0, x0);
        }
      }
      if (G > 1) {
        // G lanes per row: tree sum of the partial sums, then b +/- sum
#pragma unroll
        for (int o = 1; o < G; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (valid) {
          const VT b = reinterpret_cast<const VT*>(st + ch.b_off)[r];
          acc = LOWER ? b + acc : b - acc;
        }
      }
      if (valid && g == 0) {
        if (!LOWER) acc = acc / reinterpret_cast<const VT*>(st + ch.diag_off)[r];
        vals[(ch.pos0 + r) & (RING - 1)] = acc;
        if (mt.w >= 0) vals[mt.w] = acc;
        x[mt.x] = acc;
      }
    }
    consumers_sync();                 // chunk k complete: its values are visible, its stage is free
    // publish the progress for the helper blocks (x stores of the chunk precede it)
    if (SPLIT && tid == 0) {
      if (publish) {
        st_release_cta_shared(&s_done, k + 1);
      } else {
        __threadfence();
        st_release_u64(progress, ((unsigned long long)epoch << 32) | (unsigned long long)(k + 1));
      }
    }
    if (*v_abort) {
      // a copy never completed: stop, after giving the copies already started a bounded time to land
      if (tid == 0)
        for (int q = k; q < *v_issued; q++) mbar_wait_bounded(&full[q % nst], (unsigned)((q / nst) & 1), kDrainSpin);
      return;
    }
    if (tid == 0) mbar_arrive(&empty[s]);
  }
}

// right-hand side into the chunk images (level order)
template <class VT>
__global__ void k_gather_lev(int n, const int* __restrict__ order, const int* __restrict__ bidx,
                             const VT* __restrict__ b, VT* __restrict__ img, const KrylovScalars* ks) {
  if (ks && ks->conv != 0) return;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) img[bidx[p]] = b[order[p]];
}

// factor values into the chunk images (entries and, for U, the diagonal)
template <class MT, class VT>
__global__ void k_pack_wave(int nent, const long long* __restrict__ ent_dst, const int* __restrict__ ent_src,
                            int ndiag, const long long* __restrict__ diag_dst, const int* __restrict__ diag_src,
                            const MT* __restrict__ LU, unsigned char* img) {
  int t = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  for (int q = t; q < nent; q += stride) *reinterpret_cast<VT*>(img + ent_dst[q]) = (VT)LU[ent_src[q]];
  for (int q = t; q < ndiag; q += stride) *reinterpret_cast<VT*>(img + diag_dst[q]) = (VT)LU[diag_src[q]];
}

// factor values of the far entries (split layouts)
template <class MT, class VT>
__global__ void k_pack_far(long long nfar, const int* __restrict__ far_vsrc, const MT* __restrict__ LU,
                           VT* __restrict__ far_val) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nfar; q += (long long)gridDim.x * blockDim.x)
    far_val[q] = (VT)LU[far_vsrc[q]];
}

}  // namespace

// ---- host side ----------------------------------------------------------------

template <class VT, bool LOWER, int G, bool FAR, bool SPLIT>
static cudaError_t launch_wave_k(rg_ctx* c, WaveDev& wd, VT* x, const KrylovScalars* ks, size_t smem) {
  static int attr_done[kMaxDevices] = {0};   // per device: the attribute is a device property
  static int blocks_dev[kMaxDevices] = {0};  // co-resident blocks of the split launch
  if (!device_slot_ok(c)) return cudaErrorInvalidDevice;
  auto kern = k_trsv_wave<VT, LOWER, G, FAR, SPLIT>;
  if (attr_done[c->device] < (int)smem) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_done[c->device] = (int)smem;
    blocks_dev[c->device] = 0;
  }
  int nchunks = (int)wd.nchunks;
  const WaveChunk* chunks = wd.chunks.p;
  unsigned char* img = wd.img.p;
  int stage_bytes = wd.stage_bytes;
  int* err = c->dev_err.p;
  const long long* fptr = wd.far_ptr.p;
  const int* fsrc = wd.far_src.p;
  const VT* fval = reinterpret_cast<const VT*>(wd.far_val.p);
  const int* bidx = wd.bidx.p;
  int* ready = wd.chunk_ready.p;
  unsigned long long* prog = wd.progress.p;
  unsigned epoch = 0;
  // launch options (tuning overrides: RG_WAVE_PREFETCH chunks, 0 = none;
  // RG_WAVE_PUBLISH 0/1; RG_WAVE_SCAN flags per batch, 0 = one acquire per chunk;
  // RG_WAVE_PIECES 1-4 bulk copies per chunk; RG_WAVE_L2AHEAD chunks; RG_WAVE_SPIN 0/1)
  static int tune = -1;
  if (tune < 0) {
    const char* e = getenv("RG_WAVE_PREFETCH");
    const int pf = e ? std::max(0, std::min(64, atoi(e))) : kWavePrefetch;
    e = getenv("RG_WAVE_PUBLISH");
    const int pub = e ? (atoi(e) != 0) : kWavePublish;
    e = getenv("RG_WAVE_SCAN");
    const int sc = e ? std::max(0, std::min(31, atoi(e))) : kWaveScan;
    e = getenv("RG_WAVE_PIECES");
    const int pc = e ? std::max(1, std::min(4, atoi(e))) : kWavePieces;
    e = getenv("RG_WAVE_L2AHEAD");
    int bo = e ? std::max(0, std::min(255, atoi(e))) : kWaveL2Ahead;
    if (bo > 0) bo = std::max(bo, kWaveMaxStages);   // the producer's flag wait must not wait on itself
    e = getenv("RG_WAVE_SPIN");
    const unsigned sp = e ? (atoi(e) != 0) : kWaveSpin;
    tune = (int)((unsigned)(pf | (pub << 8) | (sc << 9) | ((pc - 1) << 14) | (bo << 16)) | (sp << 31));
  }
  if (!SPLIT) {
    kern<<<1, kThreads, smem, rg_counted(c)>>>(nchunks, chunks, img, x, stage_bytes, err, ks, fptr, fsrc, fval, bidx,
                                               ready, prog, epoch, tune);
    return cudaGetLastError();
  }
  // one wavefront block and a helper block on every other SM, all co-resident
  if (blocks_dev[c->device] == 0) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorLaunchOutOfResources;
    blocks_dev[c->device] = per_sm * c->num_sms;
  }
  int blocks = std::max(2, std::min(blocks_dev[c->device], c->num_sms));
  epoch = ++wd.epoch;
  void* args[] = {&nchunks, &chunks, &img, &x, &stage_bytes, &err, &ks, &fptr, &fsrc, &fval, &bidx, &ready, &prog,
                  &epoch, &tune};
  return cudaLaunchCooperativeKernel((void*)kern, blocks, kThreads, args, smem, rg_counted(c));
}

template <class VT, bool LOWER>
static cudaError_t launch_wave_t(rg_ctx* c, WaveDev& wd, const VT* b, VT* x, const KrylovScalars* ks) {
  const int n = c->neq;
  int nb = (n + 255) / 256;
  if (nb > c->num_sms * 4) nb = c->num_sms * 4;
  k_gather_lev<VT><<<nb, 256, 0, rg_counted(c)>>>(n, wd.order.p, wd.bidx.p, b, reinterpret_cast<VT*>(wd.img.p), ks);
  const int nst = wave_stages(sizeof(VT));
  const size_t smem = (size_t)(wave_ring(sizeof(VT)) + wave_pin(sizeof(VT))) * sizeof(VT) + (size_t)nst * (size_t)wd.stage_bytes;
  if (wd.split) {
    if (wd.lanes != 1) return cudaErrorInvalidValue;   // split layouts: one lane per row
    return launch_wave_k<VT, LOWER, 1, false, true>(c, wd, x, ks, smem);
  }
  const bool far = wd.ring_misses > 0;
  if (sizeof(VT) == 8 || wd.lanes == 1)
    return far ? launch_wave_k<VT, LOWER, 1, true, false>(c, wd, x, ks, smem)
               : launch_wave_k<VT, LOWER, 1, false, false>(c, wd, x, ks, smem);
  if (wd.lanes == 2)
    return far ? launch_wave_k<VT, LOWER, 2, true, false>(c, wd, x, ks, smem)
               : launch_wave_k<VT, LOWER, 2, false, false>(c, wd, x, ks, smem);
  return far ? launch_wave_k<VT, LOWER, 4, true, false>(c, wd, x, ks, smem)
             : launch_wave_k<VT, LOWER, 4, false, false>(c, wd, x, ks, smem);
}

cudaError_t launch_wave_solve(rg_ctx* c, bool dbl, const void* b, void* w, void* y, const KrylovScalars* ks) {
  cudaError_t e = prof_begin(c, RG_PROF_TRSV);
  if (e != cudaSuccess) return e;
  if (dbl)
    e = launch_wave_t<double, true>(c, c->waveL, (const double*)b, (double*)w, ks);
  else
    e = launch_wave_t<float, true>(c, c->waveL, (const float*)b, (float*)w, ks);
  if (e != cudaSuccess) return e;
  e = prof_end(c);
  if (e == cudaSuccess) e = prof_begin(c, RG_PROF_TRSV);
  if (e != cudaSuccess) return e;
  if (dbl)
    e = launch_wave_t<double, false>(c, c->waveU, (const double*)w, (double*)y, ks);
  else
    e = launch_wave_t<float, false>(c, c->waveU, (const float*)w, (float*)y, ks);
  if (e != cudaSuccess) return e;
  return prof_end(c);
}

// pack the current factors into both images (and the far values of split layouts)
cudaError_t launch_wave_pack(rg_ctx* c) {
  for (WaveDev* wd : {&c->waveL, &c->waveU}) {
    if (wd->split && wd->nfar > 0) {
      const int nbf = (int)std::min<long long>((wd->nfar + 255) / 256, (long long)c->num_sms * 8);
      if (c->prec == RG_PREC_FP64)
        k_pack_far<double, double><<<nbf, 256, 0, rg_counted(c)>>>(wd->nfar, wd->far_vsrc.p, c->LU64.p,
                                                                     reinterpret_cast<double*>(wd->far_val.p));
      else
        k_pack_far<float, float><<<nbf, 256, 0, rg_counted(c)>>>(wd->nfar, wd->far_vsrc.p, c->LU32.p,
                                                                   reinterpret_cast<float*>(wd->far_val.p));
    }
    int nb = (int)std::min<long long>((wd->nent + 255) / 256 + 1, (long long)c->num_sms * 8);
    if (c->prec == RG_PREC_FP64)
      k_pack_wave<double, double><<<nb, 256, 0, rg_counted(c)>>>((int)wd->nent, wd->ent_dst.p, wd->ent_src.p,
                                                         (int)wd->ndiag, wd->diag_dst.p, wd->diag_src.p,
                                                         c->LU64.p, wd->img.p);
    else if (c->prec == RG_PREC_REF32)
      k_pack_wave<float, double><<<nb, 256, 0, rg_counted(c)>>>((int)wd->nent, wd->ent_dst.p, wd->ent_src.p,
                                                        (int)wd->ndiag, wd->diag_dst.p, wd->diag_src.p, c->LU32.p,
                                                        wd->img.p);
    else
      k_pack_wave<float, float><<<nb, 256, 0, rg_counted(c)>>>((int)wd->nent, wd->ent_dst.p, wd->ent_src.p,
                                                       (int)wd->ndiag, wd->diag_dst.p, wd->diag_src.p, c->LU32.p,
                                                       wd->img.p);
  }
  return cudaGetLastError();
}
