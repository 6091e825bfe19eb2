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
  {
    // the dependency-driven solves overwrite x with sentinels before reading b: the
    // two vectors must not overlap
    const char* b0 = reinterpret_cast<const char*>(b_dev);
    const char* x0 = reinterpret_cast<const char*>(x_dev);
    const size_t bytes = (size_t)c->neq * sizeof(double);
    if (b0 < x0 + bytes && x0 < b0 + bytes)
      return rg_fail(c, RG_ERR_ARG, "rg_ilu0_apply_dev_noalloc: b_dev and x_dev overlap");
  }
  if (!device_slot_ok(c)) return rg_fail(c, RG_ERR_ARG, "rg_ilu0_apply_dev_noalloc: device");
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
  // the context's pinned error word (allocated with the context) reports waits that ran
  // out, zero pivots and rows that are too wide; it is read and cleared here
  return check_device_error(c);
}
