// ILU(0) apply on device vectors without allocating: the intermediate vector
// between the L and U solves lives in a fixed file-scope device array instead
// of the context's own work vector.

#include "rg_internal.cuh"

#include <cstdio>

namespace {

// Intermediate of the two triangular solves, RG_NOALLOC_MAX_EQ doubles (2 MiB).
// Nothing in it has to start at zero: every call writes all neq entries (the
// forward solve, or the sentinel fill of the dependency-driven path) before
// any entry is read.
static __device__ __align__(256) double g_noalloc_scratch[RG_NOALLOC_MAX_EQ];

// address of the scratch array, looked up once per device
constexpr int kMaxDevices = 64;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

}  // namespace

extern "C" rg_status rg_ilu0_apply_dev_noalloc(rg_ctx* c, const double* b_dev, double* x_dev) {
  if (!c) return RG_ERR_ARG;
  if (c->neq > RG_NOALLOC_MAX_EQ) {
    char msg[160];
    snprintf(msg, sizeof msg,
             "rg_ilu0_apply_dev_noalloc: %d equations exceed the fixed scratch of %d; use rg_ilu0_apply", c->neq,
             RG_NOALLOC_MAX_EQ);
    return rg_fail(c, RG_ERR_ARG, msg);
  }
  if (!c->have_factor || !b_dev || !x_dev)
    return rg_fail(c, RG_ERR_ARG, "rg_ilu0_apply_dev_noalloc: no factors or a NULL vector");
  if (c->device < 0 || c->device >= kMaxDevices) return rg_fail(c, RG_ERR_ARG, "rg_ilu0_apply_dev_noalloc: device");
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return rg_cuda(c, e, "cudaSetDevice");
  if (!g_scratch_ptr[c->device]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return rg_cuda(c, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_scratch_ptr[c->device] = static_cast<double*>(p);
  }
  e = launch_ilu_apply_w(c, b_dev, g_scratch_ptr[c->device], x_dev);
  if (e != cudaSuccess) return rg_cuda(c, e, "rg_ilu0_apply_dev_noalloc launch");
  // the context's pinned error word (allocated with the context) reports waits that ran out
  e = cudaMemcpyAsync(c->err_host, c->dev_err.p, 4 * sizeof(int), cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) return rg_cuda(c, e, "rg_ilu0_apply_dev_noalloc sync");
  if (c->err_host[0] != 0) {
    char msg[160];
    snprintf(msg, sizeof msg, "rg_ilu0_apply_dev_noalloc: device wait gave up (kernel %d: row %d waited for %d)",
             c->err_host[1], c->err_host[2], c->err_host[3]);
    cudaMemsetAsync(c->dev_err.p, 0, 4 * sizeof(int), c->st);
    cudaStreamSynchronize(c->st);
    return rg_fail(c, RG_ERR_DEVICE_WAIT, msg);
  }
  return RG_OK;
}
