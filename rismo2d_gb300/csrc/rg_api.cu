// C-ABI entry points of rg300 (include/rg300.h), the host-side preparation of
// the device data structures (CRS layout, element->CRS slot map, element
// colouring, ILU(0) schedule) and the Newton-correction kernels.

#include "rg_internal.cuh"

#include <algorithm>
#include <atomic>
#include <thread>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

rg_status rg_fail(rg_ctx* c, rg_status s, const char* msg) {
  if (c) c->err = msg ? msg : "";
  return s;
}

rg_status rg_cuda(rg_ctx* c, cudaError_t e, const char* where) {
  if (e == cudaSuccess) return RG_OK;
  if (c) {
    c->err = std::string(where) + ": " + cudaGetErrorString(e);
  }
  return RG_ERR_CUDA;
}

#define TRY(expr)                                        \
  do {                                                   \
    cudaError_t _e = (expr);                             \
    if (_e != cudaSuccess) return rg_cuda(c, _e, #expr); \
  } while (0)

// host <-> device copies on the context's stream, counted for rg_get_stats
static cudaError_t rg_copy(rg_ctx* c, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
  if (kind == cudaMemcpyHostToDevice) c->h2d_bytes += (long long)bytes;
  if (kind == cudaMemcpyDeviceToHost) c->d2h_bytes += (long long)bytes;
  return cudaMemcpyAsync(dst, src, bytes, kind, c->st);
}

static cudaError_t h2d(rg_ctx* c, void* d, const void* h, size_t bytes) {
  return rg_copy(c, d, h, bytes, cudaMemcpyHostToDevice);
}

static cudaError_t d2h(rg_ctx* c, void* h, const void* d, size_t bytes) {
  return rg_copy(c, h, d, bytes, cudaMemcpyDeviceToHost);
}

template <class T>
static cudaError_t upload(rg_ctx* c, DBuf<T>& d, const T* h, size_t n) {
  cudaError_t e = d.alloc(n);
  if (e != cudaSuccess || n == 0 || !h) return e;
  return h2d(c, d.p, h, n * sizeof(T));
}

template <class T>
static cudaError_t upload_if(rg_ctx* c, DBuf<T>& d, const T* h, size_t n) {
  if (!h) return cudaSuccess;
  if (d.n != n) {
    cudaError_t e = d.alloc(n);
    if (e != cudaSuccess) return e;
  }
  return h2d(c, d.p, h, n * sizeof(T));
}

// ---- per-kernel-class event accounting ---------------------------------------

cudaError_t prof_flush(rg_ctx* c) {
  if (c->prof_used == 0) return cudaSuccess;
  cudaError_t e = cudaEventSynchronize(c->prof_ev[2 * (c->prof_used - 1) + 1]);
  if (e != cudaSuccess) return e;
  for (int i = 0; i < c->prof_used; i++) {
    float ms = 0;
    e = cudaEventElapsedTime(&ms, c->prof_ev[2 * i], c->prof_ev[2 * i + 1]);
    if (e != cudaSuccess) return e;
    c->prof_ms[c->prof_cls[i]] += ms;
    c->prof_launches[c->prof_cls[i]]++;
  }
  c->prof_used = 0;
  return cudaSuccess;
}

cudaError_t prof_begin(rg_ctx* c, int cls) {
  if (!c->prof_on) return cudaSuccess;
  if (c->prof_used == rg_ctx::kProfPairs) {
    cudaError_t e = prof_flush(c);
    if (e != cudaSuccess) return e;
  }
  c->prof_cls[c->prof_used] = cls;
  return cudaEventRecord(c->prof_ev[2 * c->prof_used], c->st);
}

cudaError_t prof_end(rg_ctx* c) {
  if (!c->prof_on) return cudaSuccess;
  cudaError_t e = cudaEventRecord(c->prof_ev[2 * c->prof_used + 1], c->st);
  c->prof_used++;
  return e;
}

rg_status check_device_error(rg_ctx* c) {
  TRY(d2h(c, c->err_host, c->dev_err.p, 4 * sizeof(int)));
  TRY(cudaStreamSynchronize(c->st));
  int e = c->err_host[0];
  if (e == 0) return RG_OK;
  char msg[256];
  snprintf(msg, sizeof msg, "device wait gave up (kernel %d: row %d waited for %d)", c->err_host[1],
           c->err_host[2], c->err_host[3]);
  TRY(cudaMemsetAsync(c->dev_err.p, 0, 4 * sizeof(int), c->st));
  TRY(cudaStreamSynchronize(c->st));
  if (e & 2) return rg_fail(c, RG_ERR_ZERO_PIVOT, "ILU(0) zero pivot without a repair row");
  if (e & 4) return rg_fail(c, RG_ERR_ARG, "CRS row wider than the supported maximum");
  return rg_fail(c, RG_ERR_DEVICE_WAIT, msg);
}

// =============================================================================
// Newton correction kernels (EqsUVS2D.cpp:455-759, Update.cpp:42-187)

namespace {

__device__ __forceinline__ double atomic_max_pos(double* addr, double v) {
  // non-negative doubles order like their bit patterns
  return __longlong_as_double(atomicMax((long long*)addr, __double_as_longlong(v)));
}

// upd[0..2] max|X| per variable, [3] sum of squares, [4] max |dUs|, [5] max |dS|
__global__ void k_upd_reduce(int npm, const int* __restrict__ mnodes, const int* __restrict__ eqno,
                             const double* __restrict__ X, double* upd) {
  double m0 = 0, m1 = 0, m2 = 0, ss = 0, mus = 0, ms = 0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < npm; t += gridDim.x * blockDim.x) {
    const int n = mnodes[t];
    const int qU = eqno[3 * n], qV = eqno[3 * n + 1], qS = eqno[3 * n + 2];
    double dU = qU >= 0 ? fabs(X[qU]) : 0.0;
    double dV = qV >= 0 ? fabs(X[qV]) : 0.0;
    double dS = qS >= 0 ? fabs(X[qS]) : 0.0;
    m0 = fmax(m0, dU);
    m1 = fmax(m1, dV);
    m2 = fmax(m2, dS);
    ss += dU * dU + dV * dV + dS * dS;
    mus = fmax(mus, sqrt(dU * dU + dV * dV));
    ms = fmax(ms, dS);
  }
  for (int o = 16; o > 0; o >>= 1) {
    m0 = fmax(m0, __shfl_xor_sync(0xffffffffu, m0, o));
    m1 = fmax(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    m2 = fmax(m2, __shfl_xor_sync(0xffffffffu, m2, o));
    ss += __shfl_xor_sync(0xffffffffu, ss, o);
    mus = fmax(mus, __shfl_xor_sync(0xffffffffu, mus, o));
    ms = fmax(ms, __shfl_xor_sync(0xffffffffu, ms, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_max_pos(&upd[0], m0);
    atomic_max_pos(&upd[1], m1);
    atomic_max_pos(&upd[2], m2);
    atomicAdd(&upd[3], ss);   // reported only (relaxation "norm"); order-dependent in the last bits
    atomic_max_pos(&upd[4], mus);
    atomic_max_pos(&upd[5], ms);
  }
}

// relaxation factors (method 0 / 2, EqsUVS2D.cpp:461-544)
__global__ void k_upd_relax(double* upd, int method, double maxDeltaUV, double maxDeltaS) {
  double relaxUs = 1.0, relaxS = 1.0;
  if (method == 2) {
    relaxUs = maxDeltaUV / upd[4];
    relaxS = maxDeltaS / upd[5];
    if (relaxUs > 1.0) relaxUs = 1.0;
    if (relaxS > 1.0) relaxS = 1.0;
  }
  upd[6] = relaxUs;
  upd[7] = relaxS;
  upd[8] = sqrt(upd[3]);
}

__global__ void k_upd_apply(int npm, const int* __restrict__ mnodes, const int* __restrict__ eqno,
                            const int* __restrict__ nflag, const double* __restrict__ rot,
                            const double* __restrict__ X, const double* upd, double* U, double* V, double* S,
                            double* z, const double* __restrict__ zor, double maxUs, double dryLimit, int drymethod,
                            double hmin) {
  const double relaxUs = upd[6], relaxS = upd[7];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < npm; t += gridDim.x * blockDim.x) {
    const int n = mnodes[t];
    const int qU = eqno[3 * n], qV = eqno[3 * n + 1], qS = eqno[3 * n + 2];
    double dU = qU >= 0 ? X[qU] * relaxUs : 0.0;
    double dV = qV >= 0 ? X[qV] * relaxUs : 0.0;
    double dS = qS >= 0 ? X[qS] * relaxS : 0.0;
    double u = U[n], v = V[n];
    if (nflag[n] & RG_N_ROTAT) {
      const double* r = rot + 4 * n;
      u += r[0] * dU;
      v += r[2] * dU;
      u += r[1] * dV;
      v += r[3] * dV;
    } else {
      u += dU;
      v += dV;
    }
    const double Us = sqrt(u * u + v * v);
    if (Us > maxUs) {
      u = u * maxUs / Us;
      v = v * maxUs / Us;
    }
    U[n] = u;
    V[n] = v;
    if (qS >= 0) {
      double s = S[n] + dS;
      if (drymethod == 0 || drymethod == 2 || drymethod == 3) {
        const double H = s - zor[n];
        z[n] = (H < dryLimit) ? s - dryLimit : zor[n];
      } else {
        if (s - z[n] <= 0.0) s = z[n] + hmin;
      }
      S[n] = s;
    }
  }
}

// mid-side S and z as corner means over all region triangles (EqsUVS2D.cpp:735-759)
__global__ void k_upd_midside(int ner, const int* __restrict__ rnodes, double* S, double* z) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ner; e += gridDim.x * blockDim.x) {
    const int* nd = rnodes + 6 * e;
    if (nd[3] < 0) continue;
#pragma unroll
    for (int i = 3; i < 6; i++) {
      const int l = nd[i - 3], r = nd[(i - 2) % 3];
      S[nd[i]] = 0.5 * (S[l] + S[r]);
      z[nd[i]] = 0.5 * (z[l] + z[r]);
    }
  }
}

// EQS_UVS2D::Timegrad (EqsUVS2D.cpp:1183-1230)
__global__ void k_timegrad(int np, const int* __restrict__ nflag, const double* U, const double* V, const double* S,
                           const double* oU, const double* oV, const double* oS, const double* odU,
                           const double* odV, const double* odS, double* dU, double* dV, double* dS, double iTheta,
                           double thdt) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < np; n += gridDim.x * blockDim.x) {
    // kDry | kDryPrev | kMarsh | kMarshPrev
    if (nflag[n] & (64 | 128 | 256 | 512)) {
      dU[n] = dV[n] = dS[n] = 0.0;
    } else {
      dU[n] = iTheta * odU[n] + thdt * (U[n] - oU[n]);
      dV[n] = iTheta * odV[n] + thdt * (V[n] - oV[n]);
      dS[n] = iTheta * odS[n] + thdt * (S[n] - oS[n]);
    }
  }
}

__global__ void k_zero_uv(int n, const int* nodes, double* U, double* V) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    U[nodes[i]] = 0.0;
    V[nodes[i]] = 0.0;
  }
}

}  // namespace

cudaError_t launch_update(rg_ctx* c, const rg_update_opts* o, double* stats) {
  cudaError_t e = cudaMemsetAsync(c->upd.p, 0, 16 * sizeof(double), c->st);
  if (e != cudaSuccess) return e;
  int nb = (c->np_model + 255) / 256;
  if (nb > c->num_sms * 8) nb = c->num_sms * 8;
  if (nb < 1) nb = 1;
  k_upd_reduce<<<nb, 256, 0, rg_counted(c)>>>(c->np_model, c->model_nodes.p, c->eqno.p, c->X.p, c->upd.p);
  k_upd_relax<<<1, 1, 0, rg_counted(c)>>>(c->upd.p, o->relax_method, o->max_delta_uv, o->max_delta_s);
  k_upd_apply<<<nb, 256, 0, rg_counted(c)>>>(c->np_model, c->model_nodes.p, c->eqno.p, c->nflag.p, c->rot.p, c->X.p,
                                     c->upd.p, c->U.p, c->V.p, c->S.p, c->z.p, c->zor.p, o->max_us, o->dry_limit,
                                     o->dryrew_method, c->hmin);
  int nbe = (c->ne_region + 255) / 256;
  if (nbe < 1) nbe = 1;
  k_upd_midside<<<nbe, 256, 0, rg_counted(c)>>>(c->ne_region, c->region_nodes.p, c->S.p, c->z.p);
  double h[16];
  e = rg_copy(c, h, c->upd.p, 16 * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) return e;
  if (stats) {
    stats[0] = h[0];
    stats[1] = h[1];
    stats[2] = h[2];
    stats[3] = h[6];
    stats[4] = h[7];
    stats[5] = h[8];
  }
  return cudaGetLastError();
}

// =============================================================================
// C ABI

// Host loops of the pattern set-up run on plain threads in contiguous blocks
// (each block writes only its own outputs, so the results do not depend on the
// thread count).
template <class F>
static void par_blocks(long long n, F&& fn) {
  unsigned hw = std::thread::hardware_concurrency();
  int nt = (int)std::min<unsigned>(hw ? hw : 1, 16);
  if (const char* e = getenv("RG_HOST_THREADS")) nt = std::max(1, std::min(64, atoi(e)));
  if (nt <= 1 || n < 65536) {
    fn(0ll, n);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 1; t < nt; t++) th.emplace_back([&, t] { fn(n * t / nt, n * (t + 1) / nt); });
  fn(0ll, n / nt);
  for (std::thread& x : th) x.join();
}

extern "C" {

const char* rg_version(void) { return "rg300 0.1 (sm_103a)"; }

const char* rg_last_error(rg_ctx* c) { return c ? c->err.c_str() : "null context"; }

rg_status rg_create(const rg_mesh* m, int precision, int device, rg_ctx** out) {
  if (!m || !out || m->np <= 0 || m->ne < 0 || !m->x || !m->y || !m->elem_nodes || !m->elem_nnd ||
      !m->elem_flag || !m->elem_vt)
    return RG_ERR_ARG;
  if (precision < RG_PREC_FP64 || precision > RG_PREC_MIXED) return RG_ERR_ARG;
  for (int e = 0; e < m->ne; e++) {
    int nnd = m->elem_nnd[e];
    if (nnd != 6 && nnd != 3) return RG_ERR_ARG;
    for (int i = 0; i < nnd; i++) {
      int k = m->elem_nodes[6 * e + i];
      if (k < 0 || k >= m->np) return RG_ERR_ARG;
    }
  }
  rg_ctx* c = new rg_ctx();
  *out = c;
  c->prec = precision;
  if (const char* tr = getenv("RG_TRACE")) c->trace = atoi(tr);
  if (device < 0) {
    TRY(cudaGetDevice(&c->device));
  } else {
    c->device = device;
  }
  TRY(cudaSetDevice(c->device));
  TRY(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device));
  int coop = 0;
  TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, c->device));
  if (!coop) return rg_fail(c, RG_ERR_CUDA, "device does not support cooperative launches");
  TRY(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
  for (int i = 0; i < 16; i++) TRY(cudaEventCreate(&c->ev[i]));
  TRY(cudaMallocHost((void**)&c->ks_host, sizeof(KrylovScalars)));
  TRY(cudaMallocHost((void**)&c->err_host, 4 * sizeof(int)));
  c->np = m->np;
  c->ne = m->ne;
  c->g = m->g;
  c->hmin = m->hmin;
  if (precision == RG_PREC_MIXED) c->fp64_pivot_depth = 10.0 * m->hmin;   // near-dry rows factor in FP64
  c->vk = m->vk;
  TRY(upload(c, c->x, m->x, m->np));
  TRY(upload(c, c->y, m->y, m->np));
  TRY(upload(c, c->enodes, m->elem_nodes, 6 * (size_t)m->ne));
  TRY(upload(c, c->ennd, m->elem_nnd, m->ne));
  TRY(upload(c, c->eflag, m->elem_flag, m->ne));
  TRY(upload(c, c->evt, m->elem_vt, m->ne));
  // keep host copies needed by the pattern preparation
  c->h_enodes.assign(m->elem_nodes, m->elem_nodes + 6 * (size_t)m->ne);
  c->h_ennd.assign(m->elem_nnd, m->elem_nnd + m->ne);
  c->h_eflag.assign(m->elem_flag, m->elem_flag + m->ne);
  const size_t np = m->np;
  for (DBuf<double>* b : {&c->U, &c->V, &c->S, &c->dUdt, &c->dVdt, &c->dSdt, &c->z, &c->cf, &c->cfw, &c->niox,
                          &c->nioy, &c->bcU, &c->bcS}) {
    TRY(b->alloc(np));
    TRY(cudaMemsetAsync(b->p, 0, np * sizeof(double), c->st));
  }
  TRY(c->rot.alloc(4 * np));
  TRY(cudaMemsetAsync(c->rot.p, 0, 4 * np * sizeof(double), c->st));
  TRY(c->nflag.alloc(np));
  TRY(c->bckind.alloc(np));
  TRY(cudaMemsetAsync(c->nflag.p, 0, np * sizeof(int), c->st));
  TRY(cudaMemsetAsync(c->bckind.p, 0, np * sizeof(int), c->st));
  TRY(c->ks.alloc(1));
  TRY(cudaMemsetAsync(c->ks.p, 0, sizeof(KrylovScalars), c->st));
  // error word: [0] bits, [1] kernel tag, [2] row, [3] awaited row; [4..5] the polling
  // limit of the bounded waits (int64, 0 = the built-in limit)
  TRY(c->dev_err.alloc(6));
  TRY(cudaMemsetAsync(c->dev_err.p, 0, 6 * sizeof(int), c->st));
  TRY(c->upd.alloc(16));
  TRY(cudaStreamSynchronize(c->st));
  return RG_OK;
}

rg_status rg_destroy(rg_ctx* c) {
  if (!c) return RG_OK;
  cudaSetDevice(c->device);
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->ks_host) cudaFreeHost(c->ks_host);
  if (c->err_host) cudaFreeHost(c->err_host);
  for (int i = 0; i < 16; i++)
    if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  for (cudaEvent_t e : c->prof_ev) cudaEventDestroy(e);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
  return RG_OK;
}

static rg_status set_pattern_impl(rg_ctx* c, int neq, const int* width, const int* index, const int* eqno) {
  if (!c || neq <= 0 || !width || !index || !eqno) return rg_fail(c, RG_ERR_ARG, "rg_set_pattern: bad arguments");
  TRY(cudaSetDevice(c->device));
  // CRS layout
  std::vector<int> rowptr(neq + 1, 0);
  for (int i = 0; i < neq; i++) {
    if (width[i] < 1 || width[i] > RG_MAXW) return rg_fail(c, RG_ERR_ARG, "rg_set_pattern: row width out of range");
    rowptr[i + 1] = rowptr[i] + width[i];
  }
  const int nnz = rowptr[neq];
  {
    std::atomic<int> bad{0};
    par_blocks(neq, [&](long long b, long long e) {
      for (long long i = b; i < e; i++) {
        if (index[rowptr[i]] != i) bad = 1;
        for (int q = rowptr[i]; q < rowptr[i + 1]; q++)
          if (index[q] < 0 || index[q] >= neq) bad = 2;
      }
    });
    if (bad == 1) return rg_fail(c, RG_ERR_ARG, "rg_set_pattern: diagonal must come first");
    if (bad == 2) return rg_fail(c, RG_ERR_ARG, "rg_set_pattern: column out of range");
  }
  for (int k = 0; k < 3 * c->np; k++)
    if (eqno[k] < -1 || eqno[k] >= neq) return rg_fail(c, RG_ERR_ARG, "rg_set_pattern: bad equation number");
  c->neq = neq;
  c->nnz = nnz;
  c->h_rowptr = rowptr;
  c->h_col.assign(index, index + nnz);
  TRY(upload(c, c->rowptr, rowptr.data(), rowptr.size()));
  TRY(upload(c, c->col, index, (size_t)nnz));
  TRY(upload(c, c->eqno, eqno, 3 * (size_t)c->np));

  // element rows and slot map (the linear searches of Assemble.cpp:256-263,
  // done once per pattern instead of once per entry and iteration)
  const int ne = c->ne;
  std::vector<int> erow((size_t)ne * RG_EQ, -1), slot((size_t)ne * RG_EQ * RG_EQ, -1);
  par_blocks(ne, [&](long long e0, long long e1) {
  for (long long e = e0; e < e1; e++) {
    const int nnd = c->h_ennd[e];
    const int* nd = &c->h_enodes[6 * (size_t)e];
    int eq[RG_EQ];
    for (int r = 0; r < RG_EQ; r++) eq[r] = -1;
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < nnd; i++) {
        int r = i + j * nnd;
        if (r < RG_EQ) eq[r] = eqno[3 * nd[i] + j];
      }
    for (int r = 0; r < RG_EQ; r++) {
      erow[(size_t)e * RG_EQ + r] = eq[r];
      if (eq[r] < 0) continue;
      for (int cc = 0; cc < RG_EQ; cc++) {
        if (eq[cc] < 0) continue;
        for (int q = rowptr[eq[r]]; q < rowptr[eq[r] + 1]; q++)
          if (index[q] == eq[cc]) {
            slot[((size_t)e * RG_EQ + r) * RG_EQ + cc] = q;
            break;
          }
      }
    }
  }
  });
  TRY(upload(c, c->erow, erow.data(), erow.size()));
  TRY(upload(c, c->slot, slot.data(), slot.size()));

  // greedy colouring: no two elements of a colour share a node, so their
  // scatters touch disjoint CRS rows
  std::vector<unsigned long long> used(c->np, 0ull);
  std::vector<int> color(ne, -1);
  int ncol = 0;
  for (int e = 0; e < ne; e++) {
    if (c->h_eflag[e] & RG_E_DRY) continue;   // EQS_UVS2D::Coefs skips dry elements
    const int nnd = c->h_ennd[e];
    const int* nd = &c->h_enodes[6 * (size_t)e];
    unsigned long long forb = 0;
    for (int i = 0; i < nnd; i++) forb |= used[nd[i]];
    int k = 0;
    while (k < 64 && (forb >> k) & 1ull) k++;
    if (k >= 64) return rg_fail(c, RG_ERR_ARG, "rg_set_pattern: more than 64 element colours needed");
    color[e] = k;
    for (int i = 0; i < nnd; i++) used[nd[i]] |= 1ull << k;
    ncol = std::max(ncol, k + 1);
  }
  // per colour: its region elements, then its boundary lines, each in element order
  std::vector<int> celem;
  c->color_ptr.assign(3 * (size_t)ncol, 0);
  {
    std::vector<int> cnt(2 * (size_t)ncol + 1, 0);
    for (int e = 0; e < ne; e++)
      if (color[e] >= 0) cnt[2 * color[e] + ((c->h_eflag[e] & RG_E_BOUND) ? 1 : 0) + 1]++;
    for (int k = 0; k < 2 * ncol; k++) cnt[k + 1] += cnt[k];
    celem.resize(cnt[2 * ncol]);
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int e = 0; e < ne; e++)
      if (color[e] >= 0) celem[fill[2 * color[e] + ((c->h_eflag[e] & RG_E_BOUND) ? 1 : 0)]++] = e;
    for (int k = 0; k < ncol; k++) {
      c->color_ptr[3 * k] = cnt[2 * k];
      c->color_ptr[3 * k + 1] = cnt[2 * k + 1];
      c->color_ptr[3 * k + 2] = cnt[2 * k + 2];
    }
  }
  TRY(upload(c, c->color_elem, celem.data(), celem.size()));

  // two-phase assembly: element lists and, per CRS entry and per equation, its
  // contributions in assembly order -- the order the colour-by-colour scatter adds them
  {
    const long long nasm = (long long)celem.size();
    if (nasm * RG_EQ * RG_EQ > 2147483647ll) return rg_fail(c, RG_ERR_ARG, "rg_set_pattern: too many elements");
    std::vector<int> areg, abnd;
    for (int k = 0; k < ncol; k++) {
      for (int p = c->color_ptr[3 * k]; p < c->color_ptr[3 * k + 1]; p++) areg.push_back(p);
      for (int p = c->color_ptr[3 * k + 1]; p < c->color_ptr[3 * k + 2]; p++) abnd.push_back(p);
    }
    // per equation: its contributions (position * RG_EQ + local row) in assembly order
    std::vector<long long> gptr((size_t)nnz + 1, 0), rptr((size_t)neq + 1, 0);
    for (long long p = 0; p < nasm; p++) {
      const int e = celem[p];
      const int nr = (c->h_eflag[e] & RG_E_BOUND) ? 9 : RG_EQ;
      for (int r = 0; r < nr; r++) {
        const int row = erow[(size_t)e * RG_EQ + r];
        if (row >= 0) rptr[row + 1]++;
      }
    }
    for (int r = 0; r < neq; r++) rptr[r + 1] += rptr[r];
    std::vector<int> rsrc((size_t)rptr[neq]);
    {
      std::vector<long long> rfill(rptr.begin(), rptr.end() - 1);
      for (long long p = 0; p < nasm; p++) {
        const int e = celem[p];
        const int nr = (c->h_eflag[e] & RG_E_BOUND) ? 9 : RG_EQ;
        for (int r = 0; r < nr; r++) {
          const int row = erow[(size_t)e * RG_EQ + r];
          if (row >= 0) rsrc[rfill[row]++] = (int)(p * RG_EQ + r);
        }
      }
    }
    // per CRS entry: its contributions in assembly order.  Every entry of row r is fed
    // only by the contributions of row r, so rows are processed independently, each
    // walking its own contributions in assembly order.
    auto row_entries = [&](long long r, bool fill_pass, std::vector<int>* gsrc, long long* gfill) {
      for (long long t = rptr[r]; t < rptr[r + 1]; t++) {
        const long long p = rsrc[t] / RG_EQ;
        const int lr = (int)(rsrc[t] % RG_EQ);
        const int e = celem[p];
        const int nr = (c->h_eflag[e] & RG_E_BOUND) ? 9 : RG_EQ;
        const int* sl = &slot[((size_t)e * RG_EQ + lr) * RG_EQ];
        for (int cc = 0; cc < nr; cc++) {
          const int q = sl[cc];
          if (q < 0) continue;
          if (fill_pass)
            (*gsrc)[gfill[q]++] = (int)(p * RG_EQ * RG_EQ + lr * RG_EQ + cc);
          else
            gptr[q + 1]++;
        }
      }
    };
    par_blocks(neq, [&](long long b, long long e) {
      for (long long r = b; r < e; r++) row_entries(r, false, nullptr, nullptr);
    });
    for (size_t q = 0; q < (size_t)nnz; q++) gptr[q + 1] += gptr[q];
    std::vector<int> gsrc((size_t)gptr[nnz]);
    {
      std::vector<long long> gfill(gptr.begin(), gptr.end() - 1);
      par_blocks(neq, [&](long long b, long long e) {
        for (long long r = b; r < e; r++) row_entries(r, true, &gsrc, gfill.data());
      });
    }
    c->n_asm_reg = (int)areg.size();
    c->n_asm_bnd = (int)abnd.size();
    TRY(upload(c, c->asm_reg, areg.data(), std::max<size_t>(areg.size(), 1)));
    TRY(upload(c, c->asm_bnd, abnd.data(), std::max<size_t>(abnd.size(), 1)));
    TRY(upload(c, c->gat_ptr, gptr.data(), gptr.size()));
    TRY(upload(c, c->grow_ptr, rptr.data(), rptr.size()));
    TRY(upload(c, c->gat_src, gsrc.data(), std::max<size_t>(gsrc.size(), 1)));
    TRY(upload(c, c->grow_src, rsrc.data(), std::max<size_t>(rsrc.size(), 1)));
    const size_t nk = (size_t)std::max<long long>(nasm, 1) * RG_EQ * RG_EQ;
    if (c->prec == RG_PREC_MIXED) {
      TRY(c->EK32.alloc(nk));
    } else {
      TRY(c->EK64.alloc(nk));
    }
    TRY(c->EF.alloc((size_t)std::max<long long>(nasm, 1) * RG_EQ));
    c->geo_valid = false;
  }

  // ILU(0) schedule: L positions sorted by column; split L/U operands
  std::vector<int> lsp(neq + 1, 0), Lptr(neq + 1, 0), Uptr(neq + 1, 0);
  for (int i = 0; i < neq; i++) {
    int nl = 0, nu = 0;
    for (int q = rowptr[i] + 1; q < rowptr[i + 1]; q++) {
      if (index[q] < i) nl++;
      else if (index[q] > i) nu++;
    }
    Lptr[i + 1] = Lptr[i] + nl;
    Uptr[i + 1] = Uptr[i] + nu;
  }
  lsp = Lptr;
  std::vector<int> lspos(Lptr[neq]), Lcol(Lptr[neq]), Lsrc(Lptr[neq]), Ucol(Uptr[neq]), Usrc(Uptr[neq]);
  par_blocks(neq, [&](long long b, long long e) {
    std::vector<std::pair<int, int>> tmp;
    for (long long i = b; i < e; i++) {
      tmp.clear();
      int l = Lptr[i], u = Uptr[i];
      for (int q = rowptr[i] + 1; q < rowptr[i + 1]; q++) {
        if (index[q] < i) {
          tmp.push_back({index[q], q - rowptr[i]});
          Lcol[l] = index[q];
          Lsrc[l++] = q;
        } else if (index[q] > i) {
          Ucol[u] = index[q];
          Usrc[u++] = q;
        }
      }
      std::sort(tmp.begin(), tmp.end());
      for (size_t k = 0; k < tmp.size(); k++) lspos[lsp[i] + k] = tmp[k].second;
    }
  });
  TRY(upload(c, c->lsort_ptr, lsp.data(), lsp.size()));
  TRY(upload(c, c->lsort_pos, lspos.data(), std::max<size_t>(lspos.size(), 1)));
  TRY(upload(c, c->Lptr, Lptr.data(), Lptr.size()));
  TRY(upload(c, c->Lcol, Lcol.data(), Lcol.size()));
  TRY(upload(c, c->Lsrc, Lsrc.data(), Lsrc.size()));
  TRY(upload(c, c->Uptr, Uptr.data(), Uptr.size()));
  TRY(upload(c, c->Ucol, Ucol.data(), Ucol.size()));
  TRY(upload(c, c->Usrc, Usrc.data(), Usrc.size()));
  // longest dependency chains of the L and U solves (level-set depths)
  {
    std::vector<int> lev(neq, 0);
    int dl = 0;
    for (int i = 0; i < neq; i++) {
      int l = 0;
      for (int q = Lptr[i]; q < Lptr[i + 1]; q++) l = std::max(l, lev[Lcol[q]] + 1);
      lev[i] = l;
      dl = std::max(dl, l + 1);
    }
    int du = 0;
    for (int i = neq - 1; i >= 0; i--) {
      int l = 0;
      for (int q = Uptr[i]; q < Uptr[i + 1]; q++) l = std::max(l, lev[Ucol[q]] + 1);
      lev[i] = l;
      du = std::max(du, l + 1);
    }
    c->depth_L = dl;
    c->depth_U = du;
    c->n_colors = ncol;
  }
  // wavefront solve layouts (level-ordered chunk images) and the level
  // schedule of the factorisation
  {
    const int vtb = (c->prec == RG_PREC_MIXED) ? 4 : 8;
    // stages: what the shared-memory budget leaves after the ring and pinned slots
    const int nst = wave_stages(vtb), ring = wave_ring(vtb);
    const int stage_cap = (int)(((kWaveSmem - (long long)(ring + wave_pin(vtb)) * vtb) / nst) & ~255ll);
    std::vector<int> diag_pos(rowptr.begin(), rowptr.end() - 1);
    // threads per row (RG_WAVE_LANES = 1, 2 or 4 overrides it for the FP32 solve, for tuning)
    int lanes = (vtb == 8) ? kWaveLanes64 : kWaveLanes32;
    if (const char* e = getenv("RG_WAVE_LANES"))
      if (vtb == 4 && (atoi(e) == 1 || atoi(e) == 2 || atoi(e) == 4)) lanes = atoi(e);
    // rows per chunk: one per consumer thread group (RG_WAVE_ROWS lowers the cap, for tuning)
    int rows_cap = kWaveRows / lanes;
    if (const char* e = getenv("RG_WAVE_ROWS")) rows_cap = std::max(32, std::min(rows_cap, atoi(e)));
    // solves whose summation order is free (the mixed path's FP32 solves, the FP64 path):
    // far entries summed by helper blocks (split layouts; RG_WAVE_SPLIT=0 keeps them in
    // the images, read from global memory).  The reference-storage mode keeps the
    // reference's order in every row, so its far entries stay in the images.
    bool split = (c->prec == RG_PREC_MIXED || c->prec == RG_PREC_FP64) && lanes == 1;
    if (const char* e = getenv("RG_WAVE_SPLIT")) split = split && atoi(e) != 0;
    // pinned slots for far sources (RG_WAVE_PIN lowers the count, for tests and tuning)
    int pin = wave_pin(vtb);
    if (const char* e = getenv("RG_WAVE_PIN")) pin = std::max(0, std::min(wave_pin(vtb), atoi(e)));
    WaveLayout wl, wu;
    std::thread tl([&] {
      wl = build_wave_layout(neq, Lptr, Lcol, Lsrc, diag_pos, true, vtb, ring, pin, stage_cap, rows_cap, lanes,
                             split);
    });
    wu = build_wave_layout(neq, Uptr, Ucol, Usrc, diag_pos, false, vtb, ring, pin, stage_cap, rows_cap, lanes,
                           split);
    tl.join();
    for (auto pr : {std::make_pair(&wl, &c->waveL), std::make_pair(&wu, &c->waveU)}) {
      WaveLayout& w = *pr.first;
      WaveDev& d = *pr.second;
      TRY(upload(c, d.img, w.img_host.data(), std::max<size_t>(w.img_host.size(), 16)));
      TRY(upload(c, d.chunks, w.chunks.data(), std::max<size_t>(w.chunks.size(), 1)));
      TRY(upload(c, d.order, w.order.data(), std::max<size_t>(w.order.size(), 1)));
      TRY(upload(c, d.bidx, w.bidx.data(), std::max<size_t>(w.bidx.size(), 1)));
      TRY(upload(c, d.ent_src, w.ent_src.data(), std::max<size_t>(w.ent_src.size(), 1)));
      TRY(upload(c, d.ent_dst, w.ent_dst.data(), std::max<size_t>(w.ent_dst.size(), 1)));
      TRY(upload(c, d.diag_src, w.diag_src.data(), std::max<size_t>(w.diag_src.size(), 1)));
      TRY(upload(c, d.diag_dst, w.diag_dst.data(), std::max<size_t>(w.diag_dst.size(), 1)));
      d.split = split;
      d.nfar = (long long)w.far_src.size();
      if (split) {
        TRY(upload(c, d.far_ptr, w.far_ptr.data(), w.far_ptr.size()));
        TRY(upload(c, d.far_src, w.far_src.data(), std::max<size_t>(w.far_src.size(), 1)));
        TRY(upload(c, d.far_vsrc, w.far_vsrc.data(), std::max<size_t>(w.far_vsrc.size(), 1)));
        TRY(d.far_val.alloc(std::max<size_t>(w.far_src.size(), 1) * (size_t)vtb));
        TRY(d.chunk_ready.alloc(std::max<size_t>(w.chunks.size(), 1)));
        TRY(cudaMemsetAsync(d.chunk_ready.p, 0, d.chunk_ready.bytes(), c->st));
        TRY(d.progress.alloc(1));
        TRY(cudaMemsetAsync(d.progress.p, 0, sizeof(unsigned long long), c->st));
        d.epoch = 0;
      }
      d.nchunks = (long long)w.chunks.size();
      d.nent = (long long)w.ent_src.size();
      d.ndiag = (long long)w.diag_src.size();
      d.stage_bytes = stage_cap;
      d.lanes = lanes;
      d.depth = w.depth;
      d.ring_misses = w.ring_misses;
      d.max_chunk_bytes = 0;
      for (const WaveChunk& ch : w.chunks)
        d.max_chunk_bytes = std::max(d.max_chunk_bytes, ch.img_bytes);
      TRY(cudaStreamSynchronize(c->st));   // host images are freed at scope end
    }
    // a row too wide for one stage (never with P2 triangles: at most ~45 entries)
    // leaves the solves to the dependency-driven kernels
    c->use_wave = (c->waveL.max_chunk_bytes <= stage_cap && c->waveU.max_chunk_bytes <= stage_cap) ? 1 : 0;
    if (const char* e = getenv("RG_NO_WAVE")) c->use_wave = atoi(e) ? 0 : c->use_wave;
    // factor schedule: rows grouped by L level (the L solve's level order)
    std::vector<int> lev(neq, 0), fptr;
    int nlev = 0;
    for (int i = 0; i < neq; i++) {
      int l = 0;
      for (int q = Lptr[i]; q < Lptr[i + 1]; q++) l = std::max(l, lev[Lcol[q]] + 1);
      lev[i] = l;
      nlev = std::max(nlev, l + 1);
    }
    fptr.assign(nlev + 1, 0);
    for (int i = 0; i < neq; i++) fptr[lev[i] + 1]++;
    for (int l = 0; l < nlev; l++) fptr[l + 1] += fptr[l];
    std::vector<int> frows(neq), fill(fptr.begin(), fptr.end() - 1);
    for (int i = 0; i < neq; i++) frows[fill[lev[i]]++] = i;
    TRY(upload(c, c->flev_ptr, fptr.data(), fptr.size()));
    TRY(upload(c, c->flev_rows, frows.data(), frows.size()));
    c->waveL.lev_ptr = fptr;
    // fill map: one short per (sorted L entry, entry of its pivot row)
    std::vector<long long> foff(lspos.size() + 1, 0);
    for (int i = 0; i < neq; i++)
      for (int q = lsp[i]; q < lsp[i + 1]; q++) {
        const int k = index[rowptr[i] + lspos[q]];
        foff[q + 1] = foff[q] + (rowptr[k + 1] - rowptr[k] - 1);
      }
    TRY(upload(c, c->fmap_off, foff.data(), foff.size()));
    std::vector<int> lscol(std::max<size_t>(lspos.size(), 1), 0);
    for (int i = 0; i < neq; i++)
      for (int q = lsp[i]; q < lsp[i + 1]; q++) lscol[q] = index[rowptr[i] + lspos[q]];
    TRY(upload(c, c->lsort_col, lscol.data(), lscol.size()));
    TRY(c->fmap.alloc((size_t)std::max<long long>(foff.back(), 1)));
    TRY(launch_build_fmap(c));
  }
  TRY(c->fflag.alloc(neq));
  TRY(cudaMemsetAsync(c->fflag.p, 0, neq * sizeof(int), c->st));
  c->fepoch = 0;

  // values and work vectors
  const size_t n = neq;
  if (c->prec == RG_PREC_FP64) {
    TRY(c->A64.alloc(nnz));
    TRY(c->LU64.alloc(nnz));
    TRY(c->Lv64.alloc(std::max<size_t>(Lcol.size(), 1)));
    TRY(c->Uv64.alloc(std::max<size_t>(Ucol.size(), 1)));
    TRY(c->Dv64.alloc(n));
  } else {
    TRY(c->A32.alloc(nnz));
    TRY(c->LU32.alloc(nnz));
    TRY(c->Lv32.alloc(std::max<size_t>(Lcol.size(), 1)));
    TRY(c->Uv32.alloc(std::max<size_t>(Ucol.size(), 1)));
    TRY(c->Dv32.alloc(n));
  }
  TRY(c->B.alloc(n));
  for (DBuf<double>* b : {&c->r0, &c->ri, &c->vi, &c->pi, &c->yi, &c->zi, &c->ti, &c->tt, &c->xm, &c->X, &c->tmp})
    TRY(b->alloc(n));
  if (c->prec == RG_PREC_MIXED)
    for (DBuf<float>* b : {&c->f_r0, &c->f_ri, &c->f_vi, &c->f_pi, &c->f_yi, &c->f_zi, &c->f_ti, &c->f_x, &c->f_xm,
                           &c->f_b, &c->f_w})
      TRY(b->alloc(n));
  TRY(c->partial.alloc((size_t)c->num_sms * 8 * 4 + 64));
  c->have_system = false;
  c->have_factor = false;
  TRY(cudaStreamSynchronize(c->st));
  return RG_OK;
}

rg_status rg_set_pattern(rg_ctx* c, int neq, const int* width, const int* index, const int* eqno) {
  const auto t0 = std::chrono::steady_clock::now();
  const rg_status st = set_pattern_impl(c, neq, width, index, eqno);
  if (c) {
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    c->t_ms[8] = ms;
    c->t_ms[9] += ms;
  }
  return st;
}

rg_status rg_set_boundary(rg_ctx* c, const int* nflag, const int* bckind, const double* rot, const double* niox,
                          const double* nioy, const double* bcU, const double* bcS) {
  if (!c) return RG_ERR_ARG;
  TRY(cudaSetDevice(c->device));
  const size_t np = c->np;
  TRY(upload_if(c, c->nflag, nflag, np));
  TRY(upload_if(c, c->bckind, bckind, np));
  TRY(upload_if(c, c->rot, rot, 4 * np));
  TRY(upload_if(c, c->niox, niox, np));
  TRY(upload_if(c, c->nioy, nioy, np));
  TRY(upload_if(c, c->bcU, bcU, np));
  TRY(upload_if(c, c->bcS, bcS, np));
  c->have_boundary = true;
  return RG_OK;
}

rg_status rg_set_state(rg_ctx* c, const double* U, const double* V, const double* S, const double* dUdt,
                       const double* dVdt, const double* dSdt, const double* z, const double* cf, const double* cfw) {
  if (!c) return RG_ERR_ARG;
  TRY(cudaSetDevice(c->device));
  const size_t np = c->np;
  TRY(upload_if(c, c->U, U, np));
  TRY(upload_if(c, c->V, V, np));
  TRY(upload_if(c, c->S, S, np));
  TRY(upload_if(c, c->dUdt, dUdt, np));
  TRY(upload_if(c, c->dVdt, dVdt, np));
  TRY(upload_if(c, c->dSdt, dSdt, np));
  TRY(upload_if(c, c->z, z, np));
  TRY(upload_if(c, c->cf, cf, np));
  TRY(upload_if(c, c->cfw, cfw, np));
  return RG_OK;
}

}  // extern "C"

namespace {
__global__ void k_gather_nodes(int n, const int* __restrict__ idx, const double* __restrict__ S,
                               const double* __restrict__ z, const double* __restrict__ cf, double* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int k = idx[i];
    out[i] = S[k];
    out[n + i] = z[k];
    out[2 * n + i] = cf[k];
  }
}
__global__ void k_scatter_nodes(int n, const int* __restrict__ idx, const double* __restrict__ v,
                                double* __restrict__ S) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) S[idx[i]] = v[i];
}
}  // namespace

static rg_status upload_selection(rg_ctx* c, int n, const int* idx) {
  for (int i = 0; i < n; i++)
    if (idx[i] < 0 || idx[i] >= c->np) return rg_fail(c, RG_ERR_ARG, "node selection: index out of range");
  TRY(c->sel_idx.alloc((size_t)n));
  TRY(c->sel_val.alloc(3 * (size_t)n));
  c->sel_host.resize(3 * (size_t)n);
  TRY(cudaMemcpyAsync(c->sel_idx.p, idx, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, c->st));
  return RG_OK;
}

rg_status rg_gather_nodes(rg_ctx* c, int n, const int* idx, double* S, double* z, double* cf) {
  if (!c || n < 0 || (n > 0 && !idx)) return RG_ERR_ARG;
  if (n == 0) return RG_OK;
  TRY(cudaSetDevice(c->device));
  rg_status st = upload_selection(c, n, idx);
  if (st != RG_OK) return st;
  k_gather_nodes<<<std::min((n + 255) / 256, c->num_sms), 256, 0, rg_counted(c)>>>(n, c->sel_idx.p, c->S.p, c->z.p,
                                                                                  c->cf.p, c->sel_val.p);
  TRY(cudaGetLastError());
  TRY(rg_copy(c, c->sel_host.data(), c->sel_val.p, 3 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
  TRY(cudaStreamSynchronize(c->st));
  for (int i = 0; i < n; i++) {
    if (S) S[idx[i]] = c->sel_host[i];
    if (z) z[idx[i]] = c->sel_host[n + i];
    if (cf) cf[idx[i]] = c->sel_host[2 * (size_t)n + i];
  }
  return RG_OK;
}

rg_status rg_scatter_nodes_S(rg_ctx* c, int n, const int* idx, const double* S) {
  if (!c || n < 0 || (n > 0 && (!idx || !S))) return RG_ERR_ARG;
  if (n == 0) return RG_OK;
  TRY(cudaSetDevice(c->device));
  rg_status st = upload_selection(c, n, idx);
  if (st != RG_OK) return st;
  for (int i = 0; i < n; i++) c->sel_host[i] = S[idx[i]];
  TRY(rg_copy(c, c->sel_val.p, c->sel_host.data(), (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
  k_scatter_nodes<<<std::min((n + 255) / 256, c->num_sms), 256, 0, rg_counted(c)>>>(n, c->sel_idx.p, c->sel_val.p,
                                                                                   c->S.p);
  TRY(cudaGetLastError());
  TRY(cudaStreamSynchronize(c->st));
  return RG_OK;
}

extern "C" {

rg_status rg_get_state(rg_ctx* c, double* U, double* V, double* S, double* z) {
  if (!c) return RG_ERR_ARG;
  TRY(cudaSetDevice(c->device));
  const size_t b = c->np * sizeof(double);
  if (U) TRY(rg_copy(c, U, c->U.p, b, cudaMemcpyDeviceToHost));
  if (V) TRY(rg_copy(c, V, c->V.p, b, cudaMemcpyDeviceToHost));
  if (S) TRY(rg_copy(c, S, c->S.p, b, cudaMemcpyDeviceToHost));
  if (z) TRY(rg_copy(c, z, c->z.p, b, cudaMemcpyDeviceToHost));
  TRY(cudaStreamSynchronize(c->st));
  return RG_OK;
}

rg_status rg_set_relax(rg_ctx* c, double relaxThdt_UV, double relaxThdt_H) {
  if (!c) return RG_ERR_ARG;
  c->rUV = relaxThdt_UV;
  c->rH = relaxThdt_H;
  return RG_OK;
}

rg_status rg_set_fp64_pivots(rg_ctx* c, double depth) {
  if (!c || !(depth >= 0.0)) return rg_fail(c, RG_ERR_ARG, "rg_set_fp64_pivots: depth must be >= 0");
  c->fp64_pivot_depth = depth;
  return RG_OK;
}

rg_status rg_set_wait_limit(rg_ctx* c, long long polls) {
  if (!c || polls < 0) return rg_fail(c, RG_ERR_ARG, "rg_set_wait_limit: negative limit");
  TRY(cudaSetDevice(c->device));
  TRY(cudaMemcpyAsync(c->dev_err.p + 4, &polls, sizeof(long long), cudaMemcpyHostToDevice, c->st));
  TRY(cudaStreamSynchronize(c->st));
  return RG_OK;
}

rg_status rg_set_jacobian(rg_ctx* c, int friction_depth) {
  if (!c) return RG_ERR_ARG;
  if (friction_depth != 0 && friction_depth != 1) return rg_fail(c, RG_ERR_ARG, "rg_set_jacobian: option is 0 or 1");
  c->jac_friction = friction_depth;
  return RG_OK;
}

static rg_status copy_out_system(rg_ctx* c, double* B_out, float* A32_out, double* A64_out, bool lu) {
  if (B_out) TRY(rg_copy(c, B_out, c->B.p, c->neq * sizeof(double), cudaMemcpyDeviceToHost));
  if (c->prec == RG_PREC_FP64) {
    const double* src = lu ? c->LU64.p : c->A64.p;
    if (A64_out) TRY(rg_copy(c, A64_out, src, c->nnz * sizeof(double), cudaMemcpyDeviceToHost));
    if (A32_out) {
      std::vector<double> tmp(c->nnz);
      TRY(rg_copy(c, tmp.data(), src, c->nnz * sizeof(double), cudaMemcpyDeviceToHost));
      TRY(cudaStreamSynchronize(c->st));
      for (int64_t i = 0; i < c->nnz; i++) A32_out[i] = (float)tmp[i];
    }
  } else {
    const float* src = lu ? c->LU32.p : c->A32.p;
    if (A32_out) TRY(rg_copy(c, A32_out, src, c->nnz * sizeof(float), cudaMemcpyDeviceToHost));
    if (A64_out) {
      std::vector<float> tmp(c->nnz);
      TRY(rg_copy(c, tmp.data(), src, c->nnz * sizeof(float), cudaMemcpyDeviceToHost));
      TRY(cudaStreamSynchronize(c->st));
      for (int64_t i = 0; i < c->nnz; i++) A64_out[i] = (double)tmp[i];
    }
  }
  TRY(cudaStreamSynchronize(c->st));
  return RG_OK;
}

rg_status rg_assemble(rg_ctx* c, double* B_out, float* A32_out, double* A64_out) {
  if (!c || c->neq <= 0) return rg_fail(c, RG_ERR_ARG, "rg_assemble: no pattern");
  TRY(cudaSetDevice(c->device));
  TRY(cudaEventRecord(c->ev[0], c->st));
  TRY(prof_begin(c, RG_PROF_ASSEMBLE));
  TRY(launch_assemble(c));
  TRY(prof_end(c));
  TRY(cudaEventRecord(c->ev[1], c->st));
  TRY(cudaEventSynchronize(c->ev[1]));
  float ms = 0;
  TRY(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
  c->t_ms[0] = ms;
  c->have_system = true;   // resident factors (if any) now belong to an earlier matrix of this pattern
  return copy_out_system(c, B_out, A32_out, A64_out, false);
}

rg_status rg_load_system(rg_ctx* c, const float* A32, const double* A64, const double* B) {
  if (!c || c->neq <= 0 || (!A32 == !A64) || !B) return rg_fail(c, RG_ERR_ARG, "rg_load_system: bad arguments");
  TRY(cudaSetDevice(c->device));
  if (c->prec == RG_PREC_FP64) {
    if (A64) {
      TRY(rg_copy(c, c->A64.p, A64, c->nnz * sizeof(double), cudaMemcpyHostToDevice));
    } else {
      std::vector<double> t(A32, A32 + c->nnz);
      TRY(rg_copy(c, c->A64.p, t.data(), c->nnz * sizeof(double), cudaMemcpyHostToDevice));
      TRY(cudaStreamSynchronize(c->st));
    }
  } else {
    if (A32) {
      TRY(rg_copy(c, c->A32.p, A32, c->nnz * sizeof(float), cudaMemcpyHostToDevice));
    } else {
      std::vector<float> t(c->nnz);
      for (int64_t i = 0; i < c->nnz; i++) t[i] = (float)A64[i];
      TRY(rg_copy(c, c->A32.p, t.data(), c->nnz * sizeof(float), cudaMemcpyHostToDevice));
      TRY(cudaStreamSynchronize(c->st));
    }
  }
  TRY(rg_copy(c, c->B.p, B, c->neq * sizeof(double), cudaMemcpyHostToDevice));
  TRY(cudaStreamSynchronize(c->st));
  c->have_system = true;
  return RG_OK;
}

rg_status rg_scale(rg_ctx* c, double* scale) {
  if (!c || !c->have_system) return rg_fail(c, RG_ERR_ARG, "rg_scale: no system");
  TRY(cudaSetDevice(c->device));
  double s = 0;
  TRY(cudaEventRecord(c->ev[2], c->st));
  TRY(launch_scale(c, &s));
  TRY(cudaEventRecord(c->ev[3], c->st));
  TRY(cudaEventSynchronize(c->ev[3]));
  float ms = 0;
  TRY(cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]));
  c->t_ms[1] = ms;
  if (scale) *scale = s;
  if (!(s == s)) return rg_fail(c, RG_ERR_NONFINITE, "rg_scale: non-finite residual norm");
  return RG_OK;
}

rg_status rg_ilu0_factor(rg_ctx* c, float* LU32_out, double* LU64_out) {
  if (!c || !c->have_system) return rg_fail(c, RG_ERR_ARG, "rg_ilu0_factor: no system");
  TRY(cudaSetDevice(c->device));
  TRY(cudaEventRecord(c->ev[4], c->st));
  c->n_factor_calls++;
  if (c->use_level_factor) {
    TRY(prof_begin(c, RG_PROF_FACTOR));
    TRY(launch_factor_level(c));
    TRY(prof_end(c));
    TRY(cudaEventRecord(c->ev[6], c->st));
    TRY(d2h(c, c->err_host, c->dev_err.p, 4 * sizeof(int)));
    TRY(cudaStreamSynchronize(c->st));
    if (c->err_host[0] & 16) {
      // a pivot needs the zero-pivot repair: redo with the dependency-driven kernel
      TRY(cudaMemsetAsync(c->dev_err.p, 0, 4 * sizeof(int), c->st));
      TRY(launch_factor(c));
      c->n_repair_fallbacks++;
    }
  } else {
    TRY(launch_factor(c));
  }
  TRY(launch_split(c));
  if (c->use_wave) TRY(launch_wave_pack(c));
  TRY(cudaEventRecord(c->ev[5], c->st));
  rg_status s = check_device_error(c);
  if (s != RG_OK) return s;
  float ms = 0;
  TRY(cudaEventElapsedTime(&ms, c->ev[4], c->ev[5]));
  c->t_ms[2] = ms;
  if (c->use_level_factor) {
    TRY(cudaEventElapsedTime(&ms, c->ev[4], c->ev[6]));
    c->t_ms[5] = ms;   // level-scheduled kernel alone
  }
  c->have_factor = true;
  if (LU32_out || LU64_out) return copy_out_system(c, nullptr, LU32_out, LU64_out, true);
  return RG_OK;
}

rg_status rg_ilu0_apply_f32(rg_ctx* c, const float* B, float* X) {
  if (!c || !c->have_factor || !B || !X) return rg_fail(c, RG_ERR_ARG, "rg_ilu0_apply_f32: no factors");
  if (c->prec != RG_PREC_MIXED) return rg_fail(c, RG_ERR_ARG, "rg_ilu0_apply_f32: mixed-precision contexts only");
  TRY(cudaSetDevice(c->device));
  TRY(rg_copy(c, c->f_pi.p, B, c->neq * sizeof(float), cudaMemcpyHostToDevice));
  TRY(launch_ilu_apply_f(c, c->f_pi.p, c->f_w.p, c->f_yi.p));
  rg_status s = check_device_error(c);
  if (s != RG_OK) return s;
  TRY(rg_copy(c, X, c->f_yi.p, c->neq * sizeof(float), cudaMemcpyDeviceToHost));
  TRY(cudaStreamSynchronize(c->st));
  return RG_OK;
}

rg_status rg_ilu0_apply(rg_ctx* c, const double* B, double* X) {
  if (!c || !c->have_factor || !B || !X) return rg_fail(c, RG_ERR_ARG, "rg_ilu0_apply: no factors");
  TRY(cudaSetDevice(c->device));
  TRY(rg_copy(c, c->ri.p, B, c->neq * sizeof(double), cudaMemcpyHostToDevice));
  TRY(cudaEventRecord(c->ev[6], c->st));
  TRY(launch_ilu_apply_d(c, c->ri.p, c->zi.p));
  TRY(cudaEventRecord(c->ev[7], c->st));
  rg_status s = check_device_error(c);
  if (s != RG_OK) return s;
  float ms = 0;
  TRY(cudaEventElapsedTime(&ms, c->ev[6], c->ev[7]));
  c->t_ms[5] = ms;
  TRY(rg_copy(c, X, c->zi.p, c->neq * sizeof(double), cudaMemcpyDeviceToHost));
  TRY(cudaStreamSynchronize(c->st));
  return RG_OK;
}

rg_status rg_spmv(rg_ctx* c, const double* x, double* r) {
  if (!c || !c->have_system || !x || !r) return rg_fail(c, RG_ERR_ARG, "rg_spmv: no system");
  TRY(cudaSetDevice(c->device));
  TRY(rg_copy(c, c->pi.p, x, c->neq * sizeof(double), cudaMemcpyHostToDevice));
  TRY(cudaEventRecord(c->ev[8], c->st));
  TRY(launch_spmv_d(c, c->pi.p, c->vi.p));
  TRY(cudaEventRecord(c->ev[9], c->st));
  TRY(rg_copy(c, r, c->vi.p, c->neq * sizeof(double), cudaMemcpyDeviceToHost));
  TRY(cudaStreamSynchronize(c->st));
  float ms = 0;
  TRY(cudaEventElapsedTime(&ms, c->ev[8], c->ev[9]));
  c->t_ms[4] = ms;
  return RG_OK;
}

rg_status rg_bicgstab(rg_ctx* c, int maxIter, double maxDiff, double* X_out, int* iters, double* accuracy) {
  if (!c || !c->have_factor || maxIter <= 0) return rg_fail(c, RG_ERR_ARG, "rg_bicgstab: no factors");
  TRY(cudaSetDevice(c->device));
  TRY(cudaEventRecord(c->ev[10], c->st));
  rg_status s = run_bicgstab(c, maxIter, maxDiff, iters, accuracy);
  TRY(cudaEventRecord(c->ev[11], c->st));
  rg_status d = check_device_error(c);
  if (d != RG_OK) return d;
  if (s != RG_OK && s != RG_NOT_CONVERGED) return s;
  float ms = 0;
  TRY(cudaEventElapsedTime(&ms, c->ev[10], c->ev[11]));
  c->t_ms[3] = ms;
  TRY(prof_flush(c));
  if (X_out) {
    TRY(rg_copy(c, X_out, c->X.p, c->neq * sizeof(double), cudaMemcpyDeviceToHost));
    TRY(cudaStreamSynchronize(c->st));
  }
  return s;
}

rg_status rg_solve(rg_ctx* c, int maxIter, double maxDiff, double* X_out, double* scale_out, int* iters_out) {
  if (!c || c->neq <= 0 || !c->have_boundary) return rg_fail(c, RG_ERR_ARG, "rg_solve: pattern/boundary missing");
  rg_status s = rg_assemble(c, nullptr, nullptr, nullptr);
  if (s != RG_OK) return s;
  s = rg_scale(c, scale_out);
  if (s != RG_OK) return s;
  s = rg_ilu0_factor(c, nullptr, nullptr);
  if (s != RG_OK) return s;
  return rg_bicgstab(c, maxIter, maxDiff, X_out, iters_out, nullptr);
}

rg_status rg_set_update_lists(rg_ctx* c, int np_model, const int* model_nodes, int ne_region,
                              const int* region_nodes, const double* zor) {
  if (!c || np_model < 0 || ne_region < 0 || (np_model && !model_nodes) || (ne_region && !region_nodes) || !zor)
    return rg_fail(c, RG_ERR_ARG, "rg_set_update_lists: bad arguments");
  TRY(cudaSetDevice(c->device));
  for (int i = 0; i < np_model; i++)
    if (model_nodes[i] < 0 || model_nodes[i] >= c->np) return rg_fail(c, RG_ERR_ARG, "bad model node");
  for (int i = 0; i < 6 * ne_region; i++)
    if (region_nodes[i] < -1 || region_nodes[i] >= c->np) return rg_fail(c, RG_ERR_ARG, "bad region node");
  c->np_model = np_model;
  c->ne_region = ne_region;
  TRY(upload(c, c->model_nodes, model_nodes, std::max(np_model, 1)));
  TRY(upload(c, c->region_nodes, region_nodes, 6 * (size_t)std::max(ne_region, 1)));
  TRY(upload(c, c->zor, zor, c->np));
  c->h_region_nodes.assign(region_nodes, region_nodes + 6 * (size_t)ne_region);
  TRY(cudaStreamSynchronize(c->st));
  return RG_OK;
}

rg_status rg_newton_update(rg_ctx* c, const rg_update_opts* o, double* stats) {
  if (!c || !o || c->neq <= 0 || !c->model_nodes.p) return rg_fail(c, RG_ERR_ARG, "rg_newton_update: not set up");
  if (o->relax_method != 0 && o->relax_method != 2)
    return rg_fail(c, RG_ERR_ARG, "rg_newton_update: relaxation method must be 0 or 2");
  TRY(cudaSetDevice(c->device));
  TRY(cudaEventRecord(c->ev[12], c->st));
  TRY(launch_update(c, o, stats));
  TRY(cudaEventRecord(c->ev[13], c->st));
  TRY(cudaEventSynchronize(c->ev[13]));
  float ms = 0;
  TRY(cudaEventElapsedTime(&ms, c->ev[12], c->ev[13]));
  c->t_ms[6] = ms;
  return RG_OK;
}

rg_status rg_set_friction(rg_ctx* c, const double* elem_n, const double* elem_areafact) {
  if (!c || !elem_n || !elem_areafact || c->h_region_nodes.empty())
    return rg_fail(c, RG_ERR_ARG, "rg_set_friction: call rg_set_update_lists first");
  TRY(cudaSetDevice(c->device));
  const int ner = c->ne_region;
  std::vector<int> cnt(c->np + 1, 0);
  for (int e = 0; e < ner; e++)
    for (int i = 0; i < 6; i++) {
      int k = c->h_region_nodes[6 * (size_t)e + i];
      if (k >= 0) cnt[k + 1]++;
    }
  for (int k = 0; k < c->np; k++) cnt[k + 1] += cnt[k];
  std::vector<int> el(cnt[c->np]), pos(cnt.begin(), cnt.end() - 1);
  for (int e = 0; e < ner; e++)
    for (int i = 0; i < 6; i++) {
      int k = c->h_region_nodes[6 * (size_t)e + i];
      if (k >= 0) el[pos[k]++] = e;
    }
  TRY(upload(c, c->fr_ptr, cnt.data(), cnt.size()));
  TRY(upload(c, c->fr_el, el.data(), std::max<size_t>(el.size(), 1)));
  TRY(upload(c, c->elem_n, elem_n, std::max(ner, 1)));
  TRY(upload(c, c->elem_af, elem_areafact, std::max(ner, 1)));
  TRY(cudaStreamSynchronize(c->st));
  return RG_OK;
}

rg_status rg_friction(rg_ctx* c, double* cf_out) {
  if (!c || !c->fr_ptr.p) return rg_fail(c, RG_ERR_ARG, "rg_friction: call rg_set_friction first");
  TRY(cudaSetDevice(c->device));
  TRY(cudaEventRecord(c->ev[14], c->st));
  TRY(launch_friction(c));
  TRY(cudaEventRecord(c->ev[15], c->st));
  if (cf_out) TRY(rg_copy(c, cf_out, c->cf.p, c->np * sizeof(double), cudaMemcpyDeviceToHost));
  TRY(cudaStreamSynchronize(c->st));
  float ms = 0;
  TRY(cudaEventElapsedTime(&ms, c->ev[14], c->ev[15]));
  c->t_ms[7] = ms;
  return RG_OK;
}

// ---- MODEL::Continuity (Contin.cpp:43-170): discharge through control sections
namespace {
// one block per section; thread t integrates a contiguous run of the section's
// line elements in order, then the block sums the runs in a fixed tree order, so
// the result does not depend on timing.  Three Gauss points (GPdeg 5), quadratic
// U, V and linear depth (clipped at 0) along the line, the unnormalised normal
// (dN.y, -dN.x) (SHAPE::shapeOfLine, Line.cpp:43-160).
__global__ void k_continuity(int nsect, const int* __restrict__ sec_ptr, const int* __restrict__ seg,
                             const double* __restrict__ x, const double* __restrict__ y,
                             const double* __restrict__ U, const double* __restrict__ V,
                             const double* __restrict__ S, const double* __restrict__ z, double* __restrict__ q) {
  __shared__ double sx[256], sy[256];
  const int k = blockIdx.x;
  if (k >= nsect) return;
  const int b = sec_ptr[k], e = sec_ptr[k + 1], cnt = e - b;
  const int per = (cnt + blockDim.x - 1) / blockDim.x;
  const int lo = b + threadIdx.x * per, hi = min(e, lo + per);
  const double gx = sqrt(0.6);
  const double gp[3] = {-gx, 0.0, gx}, gw[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
  double qx = 0.0, qy = 0.0;
  for (int t = lo; t < hi; t++) {
    const int n0 = seg[3 * t], n1 = seg[3 * t + 1], n2 = seg[3 * t + 2];
    for (int g = 0; g < 3; g++) {
      const double xg = gp[g];
      const double M0 = (1.0 - xg) / 2.0, M1 = (1.0 + xg) / 2.0;
      const double N0 = xg * (xg - 1.0) / 2.0, N1 = xg * (xg + 1.0) / 2.0, N2 = 1.0 - xg * xg;
      const double d0 = xg - 0.5, d1 = xg + 0.5, d2 = -2.0 * xg;
      const double nx = d0 * y[n0] + d1 * y[n1] + d2 * y[n2];
      const double ny = -d0 * x[n0] - d1 * x[n1] - d2 * x[n2];
      double H = M0 * (S[n0] - z[n0]) + M1 * (S[n1] - z[n1]);
      if (H <= 0.0) H = 0.0;
      const double u = N0 * U[n0] + N1 * U[n1] + N2 * U[n2];
      const double v = N0 * V[n0] + N1 * V[n1] + N2 * V[n2];
      qx += gw[g] * H * u * nx;
      qy += gw[g] * H * v * ny;
    }
  }
  sx[threadIdx.x] = qx;
  sy[threadIdx.x] = qy;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      sx[threadIdx.x] += sx[threadIdx.x + o];
      sy[threadIdx.x] += sy[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    q[2 * k] = sx[0];
    q[2 * k + 1] = sy[0];
  }
}
}  // namespace

rg_status rg_continuity(rg_ctx* c, int nseg, const int* seg_nodes, const int* seg_section, int nsect, double* Qx,
                        double* Qy) {
  if (!c || nseg < 0 || nsect <= 0 || (nseg > 0 && (!seg_nodes || !seg_section)) || !Qx || !Qy)
    return rg_fail(c, RG_ERR_ARG, "rg_continuity: bad arguments");
  TRY(cudaSetDevice(c->device));
  // sort the line elements by section (stable: each section keeps the control file's order)
  std::vector<int> ptr(nsect + 1, 0), nodes(3 * (size_t)nseg);
  for (int t = 0; t < nseg; t++) {
    const int k = seg_section[t] - 1;
    if (k < 0 || k >= nsect) return rg_fail(c, RG_ERR_ARG, "rg_continuity: section number out of range");
    for (int i = 0; i < 3; i++)
      if (seg_nodes[3 * t + i] < 0 || seg_nodes[3 * t + i] >= c->np)
        return rg_fail(c, RG_ERR_ARG, "rg_continuity: node out of range");
    ptr[k + 1]++;
  }
  for (int k = 0; k < nsect; k++) ptr[k + 1] += ptr[k];
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (int t = 0; t < nseg; t++) {
    const int d = fill[seg_section[t] - 1]++;
    for (int i = 0; i < 3; i++) nodes[3 * (size_t)d + i] = seg_nodes[3 * t + i];
  }
  TRY(upload(c, c->sec_ptr, ptr.data(), ptr.size()));
  TRY(upload(c, c->sec_nodes, nodes.data(), nodes.size()));
  TRY(c->sec_q.alloc(2 * (size_t)nsect));
  k_continuity<<<nsect, 256, 0, rg_counted(c)>>>(nsect, c->sec_ptr.p, c->sec_nodes.p, c->x.p, c->y.p, c->U.p, c->V.p,
                                                  c->S.p, c->z.p, c->sec_q.p);
  TRY(cudaGetLastError());
  std::vector<double> q(2 * (size_t)nsect);
  TRY(d2h(c, q.data(), c->sec_q.p, q.size() * sizeof(double)));
  TRY(cudaStreamSynchronize(c->st));
  for (int k = 0; k < nsect; k++) {
    Qx[k] = q[2 * k];
    Qy[k] = q[2 * k + 1];
  }
  return RG_OK;
}

rg_status rg_set_elements(rg_ctx* c, int ne, const int* elem_nodes, const int* elem_nnd, const int* elem_flag,
                          const double* elem_vt) {
  if (!c || ne <= 0 || !elem_nodes || !elem_nnd || !elem_flag || !elem_vt)
    return rg_fail(c, RG_ERR_ARG, "rg_set_elements: bad arguments");
  for (int e = 0; e < ne; e++) {
    if (elem_nnd[e] != 6 && elem_nnd[e] != 3) return rg_fail(c, RG_ERR_ARG, "rg_set_elements: bad node count");
    for (int i = 0; i < elem_nnd[e]; i++)
      if (elem_nodes[6 * e + i] < 0 || elem_nodes[6 * e + i] >= c->np)
        return rg_fail(c, RG_ERR_ARG, "rg_set_elements: node out of range");
  }
  TRY(cudaSetDevice(c->device));
  c->ne = ne;
  c->geo_valid = false;
  TRY(upload(c, c->enodes, elem_nodes, 6 * (size_t)ne));
  TRY(upload(c, c->ennd, elem_nnd, ne));
  TRY(upload(c, c->eflag, elem_flag, ne));
  TRY(upload(c, c->evt, elem_vt, ne));
  c->h_enodes.assign(elem_nodes, elem_nodes + 6 * (size_t)ne);
  c->h_ennd.assign(elem_nnd, elem_nnd + ne);
  c->h_eflag.assign(elem_flag, elem_flag + ne);
  c->neq = 0;   // a pattern for the new element list must follow
  c->have_system = c->have_factor = false;
  TRY(cudaStreamSynchronize(c->st));
  return RG_OK;
}

rg_status rg_set_old(rg_ctx* c, const double* U, const double* V, const double* S, const double* dUdt,
                     const double* dVdt, const double* dSdt) {
  if (!c) return RG_ERR_ARG;
  TRY(cudaSetDevice(c->device));
  const size_t np = c->np;
  TRY(upload_if(c, c->oU, U, np));
  TRY(upload_if(c, c->oV, V, np));
  TRY(upload_if(c, c->oS, S, np));
  TRY(upload_if(c, c->odUdt, dUdt, np));
  TRY(upload_if(c, c->odVdt, dVdt, np));
  TRY(upload_if(c, c->odSdt, dSdt, np));
  return RG_OK;
}

rg_status rg_get_dt(rg_ctx* c, double* dUdt, double* dVdt, double* dSdt) {
  if (!c) return RG_ERR_ARG;
  TRY(cudaSetDevice(c->device));
  const size_t b = c->np * sizeof(double);
  if (dUdt) TRY(rg_copy(c, dUdt, c->dUdt.p, b, cudaMemcpyDeviceToHost));
  if (dVdt) TRY(rg_copy(c, dVdt, c->dVdt.p, b, cudaMemcpyDeviceToHost));
  if (dSdt) TRY(rg_copy(c, dSdt, c->dSdt.p, b, cudaMemcpyDeviceToHost));
  TRY(cudaStreamSynchronize(c->st));
  return RG_OK;
}

rg_status rg_timegrad(rg_ctx* c, double dt, double theta) {
  if (!c || !c->oU.p || !(dt > 0.0) || !(fabs(theta) > 1.0e-10))
    return rg_fail(c, RG_ERR_ARG, "rg_timegrad: previous time level not set");
  TRY(cudaSetDevice(c->device));
  const double iTheta = 1.0 - 1.0 / theta, thdt = 1.0 / dt / theta;
  int nb = (c->np + 255) / 256;
  if (nb > c->num_sms * 8) nb = c->num_sms * 8;
  k_timegrad<<<nb, 256, 0, rg_counted(c)>>>(c->np, c->nflag.p, c->U.p, c->V.p, c->S.p, c->oU.p, c->oV.p, c->oS.p,
                                    c->odUdt.p, c->odVdt.p, c->odSdt.p, c->dUdt.p, c->dVdt.p, c->dSdt.p, iTheta,
                                    thdt);
  TRY(cudaGetLastError());
  return RG_OK;
}

rg_status rg_zero_velocity(rg_ctx* c, int n, const int* nodes) {
  if (!c || n < 0 || (n && !nodes)) return RG_ERR_ARG;
  if (n == 0) return RG_OK;
  for (int i = 0; i < n; i++)
    if (nodes[i] < 0 || nodes[i] >= c->np) return rg_fail(c, RG_ERR_ARG, "rg_zero_velocity: node out of range");
  TRY(cudaSetDevice(c->device));
  TRY(upload(c, c->zero_nodes, nodes, n));
  k_zero_uv<<<(n + 255) / 256, 256, 0, rg_counted(c)>>>(n, c->zero_nodes.p, c->U.p, c->V.p);
  TRY(cudaGetLastError());
  return RG_OK;
}

rg_status rg_get_stats(rg_ctx* c, int64_t* out, int n) {
  if (!c || !out) return RG_ERR_ARG;
  int64_t v[15] = {c->neq, c->nnz, c->depth_L, c->depth_U, c->n_colors, (int64_t)c->Lcol.n,
                    c->waveL.nchunks, c->waveU.nchunks, c->waveL.ring_misses, c->waveU.ring_misses,
                    c->n_repair_fallbacks, c->n_factor_calls, c->h2d_bytes, c->d2h_bytes, c->n_launches};
  for (int i = 0; i < n && i < 15; i++) out[i] = v[i];
  return RG_OK;
}

rg_status rg_profile(rg_ctx* c, int enable, int reset) {
  if (!c) return RG_ERR_ARG;
  TRY(cudaSetDevice(c->device));
  if (c->prof_ev.empty() && enable) {
    c->prof_ev.resize(2 * rg_ctx::kProfPairs, nullptr);
    c->prof_cls.resize(rg_ctx::kProfPairs, 0);
    for (cudaEvent_t& e : c->prof_ev) TRY(cudaEventCreate(&e));
  }
  TRY(prof_flush(c));
  if (reset) {
    for (int k = 0; k < rg_ctx::kProfClasses; k++) {
      c->prof_launches[k] = 0;
      c->prof_ms[k] = 0.0;
    }
  }
  c->prof_on = enable != 0;
  return RG_OK;
}

rg_status rg_profile_read(rg_ctx* c, double* out, int n) {
  if (!c || !out) return RG_ERR_ARG;
  TRY(cudaSetDevice(c->device));
  TRY(prof_flush(c));
  for (int k = 0; k < rg_ctx::kProfClasses && 2 * k + 1 < n; k++) {
    out[2 * k] = (double)c->prof_launches[k];
    out[2 * k + 1] = c->prof_ms[k];
  }
  return RG_OK;
}

rg_status rg_event_record(rg_ctx* c, int slot) {
  if (!c || slot < 0 || slot >= 8) return RG_ERR_ARG;
  TRY(cudaSetDevice(c->device));
  if (!c->user_ev_ready) {
    for (int i = 0; i < 8; i++) TRY(cudaEventCreate(&c->user_ev[i]));
    c->user_ev_ready = true;
  }
  TRY(cudaEventRecord(c->user_ev[slot], c->st));
  return RG_OK;
}

rg_status rg_event_elapsed(rg_ctx* c, int a, int b, double* ms) {
  if (!c || !c->user_ev_ready || a < 0 || b < 0 || a >= 8 || b >= 8 || !ms) return RG_ERR_ARG;
  TRY(cudaEventSynchronize(c->user_ev[b]));
  float f = 0;
  TRY(cudaEventElapsedTime(&f, c->user_ev[a], c->user_ev[b]));
  *ms = f;
  return RG_OK;
}

rg_status rg_get_timings(rg_ctx* c, double* ms, int n) {
  if (!c || !ms) return RG_ERR_ARG;
  for (int i = 0; i < n && i < 10; i++) ms[i] = c->t_ms[i];
  return RG_OK;
}

}  // extern "C"
