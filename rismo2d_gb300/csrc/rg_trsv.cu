// Wavefront ILU(0) triangular solves: one CTA walks the dependency levels of
// PRECO_ILU0::Solve (Preco_ilu0.cpp:517-530 forward, 964-980 backward) in the
// reference's equation order.
//
// The solves are latency-bound chains (a level holds a few hundred rows, the
// depth is hundreds to thousands of levels), so the kernel keeps the whole
// chain on one SM and takes global-memory latency off the critical path:
//   * the rows of every level are packed host-side into a contiguous image
//     {row meta, diagonal, (value, source) entries} padded to 16 bytes;
//   * thread 0 streams the images of the next levels into a 3-stage shared
//     memory buffer with cp.async.bulk (TMA bulk copies) completing on
//     mbarriers, together with the right-hand side gathered into level order;
//   * solution values live in a shared-memory ring indexed by level-order
//     position; the host decides per entry whether its source is still in the
//     ring (else it is read back from global memory);
//   * levels are separated by __syncthreads.
// Levels too large for a stage are split into consecutive chunks (rows of one
// level do not depend on each other).  All waits are bounded.

#include "rg_internal.cuh"

#include <algorithm>
#include <cstring>

namespace {

constexpr int kThreads = 1024;
constexpr int kGroup = 4;                 // threads per row
constexpr long long kMbarSpin = 1ll << 26;

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

// global -> shared bulk copy completing on an mbarrier (16-byte aligned, size % 16 == 0)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

}  // namespace

namespace {

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// bounded wait on an mbarrier phase; false when the bound ran out
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
  long long it = 0;
  while (!mbar_try_wait(bar, parity)) {
    if (++it > kMbarSpin) return false;
  }
  return true;
}

__device__ __forceinline__ void consumers_sync() {
  asm volatile("bar.sync 1, %0;" ::"r"(kThreads - 32) : "memory");
}

// Warp-specialised wavefront solve: warp 31 (one elected lane) is the producer
// that streams chunk images and right-hand sides into NST stages with
// cp.async.bulk; warps 0..30 consume the stages in order, one dependency level
// chunk at a time, synchronising on a named barrier between chunks.
template <class VT, bool LOWER, int RING, int PIN>
__global__ void __launch_bounds__(kThreads, 1)
    k_trsv_wave(int nchunks, const WaveChunk* __restrict__ chunks, const unsigned char* __restrict__ img,
                const VT* __restrict__ blev, VT* __restrict__ x, int stage_bytes, int bstage_bytes, int* err,
                const KrylovScalars* ks) {
  if (ks && ks->conv != 0) return;
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int NST = 3;
  constexpr int kConsumers = kThreads - 32;
  // solution values: ring slots [0, RING), pinned long-range slots [RING, RING + PIN)
  VT* vals = reinterpret_cast<VT*>(smem);
  unsigned char* stage0 = smem + (RING + PIN) * sizeof(VT);
  unsigned char* bstage0 = stage0 + NST * (size_t)stage_bytes;
  __shared__ __align__(8) uint64_t full[NST];
  __shared__ __align__(8) uint64_t empty[NST];
  __shared__ WaveChunk sdesc[NST];
  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int s = 0; s < NST; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  if (tid >= kConsumers) {
    // ---- producer ------------------------------------------------------------
    if (tid == kConsumers) {
      for (int k = 0; k < nchunks; k++) {
        const int s = k % NST;
        if (k >= NST && !mbar_wait_bounded(&empty[s], (unsigned)(((k / NST) - 1) & 1))) {
          atomicOr(err, 8);
          break;
        }
        const WaveChunk ch = chunks[k];
        sdesc[s] = ch;
        fence_proxy_async();   // earlier generic reads of the stage precede the async refill
        mbar_expect_tx(&full[s], (unsigned)(ch.img_bytes + ch.b_bytes));
        bulk_g2s(stage0 + s * (size_t)stage_bytes, img + ch.img_off, (unsigned)ch.img_bytes, &full[s]);
        bulk_g2s(bstage0 + s * (size_t)bstage_bytes, blev + ch.b_off, (unsigned)ch.b_bytes, &full[s]);
      }
    }
    return;
  }

  // ---- consumers -------------------------------------------------------------
  const int g = tid & (kGroup - 1);
  const int rows_per_pass = kConsumers / kGroup;
  for (int k = 0; k < nchunks; k++) {
    const int s = k % NST;
    if (!mbar_wait_bounded(&full[s], (unsigned)((k / NST) & 1))) {
      if (tid == 0) atomicOr(err, 8);
    }
    const WaveChunk ch = sdesc[s];
    const unsigned char* st = stage0 + s * (size_t)stage_bytes;
    const int4* meta = reinterpret_cast<const int4*>(st);
    const VT* diag = reinterpret_cast<const VT*>(st + ch.diag_off);
    const VT* ev = reinterpret_cast<const VT*>(st + ch.val_off);
    const int* es = reinterpret_cast<const int*>(st + ch.src_off);
    const VT* bv = reinterpret_cast<const VT*>(bstage0 + s * (size_t)bstage_bytes);
    const int m = ch.nrows;
    for (int base = 0; base < m; base += rows_per_pass) {   // uniform trip count
      const int r = base + tid / kGroup;
      const bool valid = r < m;
      VT acc = 0;
      int4 mt = make_int4(0, 0, 0, -1);
      if (valid) {
        mt = meta[r];
        for (int e = mt.y + g; e < mt.y + mt.z; e += kGroup) {
          const int src = es[e];
          const VT xv = (src >= 0) ? vals[src] : x[-src - 1];
          acc += ev[e] * xv;
        }
      }
      acc += __shfl_xor_sync(0xffffffffu, acc, 1);
      acc += __shfl_xor_sync(0xffffffffu, acc, 2);
      if (valid && g == 0) {
        VT xi;
        if (LOWER)
          xi = bv[r] + acc;
        else
          xi = (bv[r] - acc) / diag[r];
        vals[(ch.pos0 + r) % RING] = xi;
        if (mt.w >= 0) vals[mt.w] = xi;
        x[mt.x] = xi;
      }
    }
    consumers_sync();                 // chunk k complete: its values are visible, its stage is free
    if (tid == 0) mbar_arrive(&empty[s]);
  }
}

// right-hand side into padded level order
template <class VT>
__global__ void k_gather_lev(int n, const int* __restrict__ order, const int* __restrict__ bidx,
                             const VT* __restrict__ b, VT* __restrict__ blev, const KrylovScalars* ks) {
  if (ks && ks->conv != 0) return;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) blev[bidx[p]] = b[order[p]];
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

}  // namespace

// ---- host side ----------------------------------------------------------------

template <class VT, bool LOWER>
static cudaError_t launch_wave_t(rg_ctx* c, WaveDev& wd, const VT* b, VT* x, const KrylovScalars* ks) {
  constexpr int RING = kWaveRing;
  constexpr int PIN = kWavePin;
  const int n = c->neq;
  int nb = (n + 255) / 256;
  if (nb > c->num_sms * 4) nb = c->num_sms * 4;
  VT* blev = reinterpret_cast<VT*>(wd.blev.p);
  k_gather_lev<VT><<<nb, 256, 0, rg_counted(c)>>>(n, wd.order.p, wd.bidx.p, b, blev, ks);
  const size_t smem = (RING + PIN) * sizeof(VT) + 3 * (size_t)wd.stage_bytes + 3 * (size_t)wd.bstage_bytes;
  static bool attr_done[2][2] = {{false, false}, {false, false}};
  bool& done = attr_done[sizeof(VT) == 8][LOWER];
  cudaError_t e;
  if (!done) {
    e = cudaFuncSetAttribute(k_trsv_wave<VT, LOWER, RING, PIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    done = true;
  }
  k_trsv_wave<VT, LOWER, RING, PIN><<<1, kThreads, smem, rg_counted(c)>>>((int)wd.nchunks, wd.chunks.p, wd.img.p, blev, x,
                                                             wd.stage_bytes, wd.bstage_bytes, c->dev_err.p, ks);
  return cudaGetLastError();
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

// pack the current factors into both images
cudaError_t launch_wave_pack(rg_ctx* c) {
  for (WaveDev* wd : {&c->waveL, &c->waveU}) {
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
