// k_noalloc.cu -- fused direct-SCF gam_4 Fock build for callers that must
// not allocate device memory.
//
// The regular device entry point (neoxc_dev_gam4_dscf) obtains its scratch
// buffer -- one partial Fock row per CTA plus one partial per proton pair --
// from cudaMallocAsync on every call.  Some callers cannot allow that: a
// host code that has handed all device memory to its own pool allocator
// (a Fortran SCF driver sharing the GPU with a memory-hungry integral
// phase), or one that runs inside a strict memory budget where a transient
// allocation can fail at the worst moment, in the middle of an SCF
// iteration.  This variant keeps its scratch in a fixed array compiled into
// the library instead, so a call allocates nothing: the caller passes the
// inputs and outputs and the library uses only memory that exists from load
// time.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/neoxc.h"
#include "neoxc_internal.h"

namespace neoxc {

// Capacity of the built-in scratch, in doubles (2 MiB + 16 KiB).  The call
// needs npbf^2 * nebf^3 + npbf^2 of them, e.g. 110,656 at nebf=12, npbf=8
// and 262,208 at nebf=16, npbf=8.  Every GPU that loads the library keeps
// this array until the process exits.
constexpr size_t kNoAllocScratchDoubles = 264192;

namespace {

static __device__ __align__(256) double g_gam4_scratch[kNoAllocScratchDoubles];

std::mutex g_mu;
double* g_scratch_addr[64] = {nullptr};

// Device address of the scratch array on the current device.  The array's
// name is only a host-side handle, so its device address is looked up once
// per device (with that device current) and cached.  The stream must belong
// to the current device: the address is that device's copy, and kernels on
// another device's stream would write that other GPU's array.
int scratch_on_current_device(cudaStream_t stream, double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return set_last_error(NEOXC_ERR_CUDA, "no CUDA device: %s",
                          cudaGetErrorString(e));
  if (dev < 0 || dev >= 64)
    return set_last_error(NEOXC_ERR_CUDA, "device id %d out of range", dev);
  int sdev = dev;
  e = cudaStreamGetDevice(stream, &sdev);
  if (e != cudaSuccess)
    return set_last_error(NEOXC_ERR_ARG, "stream: %s", cudaGetErrorString(e));
  if (sdev != dev)
    return set_last_error(NEOXC_ERR_ARG,
                          "neoxc_dev_gam4_dscf_noalloc: the stream belongs to "
                          "device %d but device %d is current; make the "
                          "stream's device current", sdev, dev);
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_gam4_scratch);
    if (e != cudaSuccess || !p)
      return set_last_error(NEOXC_ERR_CUDA,
                            "cudaGetSymbolAddress(gam_4 scratch) failed: %s",
                            cudaGetErrorString(e));
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[dev];
  return NEOXC_OK;
}

}  // namespace
}  // namespace neoxc

extern "C" int neoxc_dev_gam4_dscf_noalloc(void* stream, int64_t ne,
                                           int64_t np, const double* d_gee,
                                           const double* d_g2s,
                                           const double* d_DE,
                                           const double* d_DP,
                                           double* d_focke, double* d_fockp,
                                           double* d_E) {
  using namespace neoxc;
  if (ne < 1 || np < 1 || !d_gee || !d_g2s || !d_DE || !d_DP || !d_focke ||
      !d_fockp || !d_E)
    return set_last_error(NEOXC_ERR_ARG, "argument check failed: sizes/pointers");
  if (ne > kGam4MaxNE || np > kGam4MaxNP)
    return set_last_error(NEOXC_ERR_UNSUPPORTED,
                          "gam_4 element kernels: ne <= %d, np <= %lld",
                          kGam4MaxNE, (long long)kGam4MaxNP);
  const size_t need = gam4_partial_doubles((int)ne, (int)np);
  if (need > kNoAllocScratchDoubles)
    return set_last_error(
        NEOXC_ERR_UNSUPPORTED,
        "neoxc_dev_gam4_dscf_noalloc: nebf=%lld, npbf=%lld needs %zu scratch "
        "doubles but the built-in array holds %zu (npbf^2*nebf^3 + npbf^2 "
        "must not exceed it); use neoxc_dev_gam4_dscf for larger systems",
        (long long)ne, (long long)np, need, kNoAllocScratchDoubles);
  double* scratch = nullptr;
  int rc = scratch_on_current_device((cudaStream_t)stream, &scratch);
  if (rc) return rc;
  // Every scratch element the kernels read is written earlier in the same
  // call, so nothing needs clearing between calls.
  cudaError_t e = launch_gam4_dscf((int)ne, (int)np, d_gee, d_g2s, d_DE, d_DP,
                                   scratch, d_focke, d_fockp, d_E,
                                   (cudaStream_t)stream);
  if (e != cudaSuccess)
    return set_last_error(NEOXC_ERR_CUDA, "gam_4 launch: %s",
                          cudaGetErrorString(e));
  return NEOXC_OK;
}
