// pz_explicit_terms_noalloc: the explicit terms of one instance without any
// device allocation.
//
// pz_explicit_terms takes device memory for its intermediates (the radial
// products dVsT and dVsOm, 2 * n_m_max * n_r_max complex values) with
// cudaMallocAsync on every call.  Some callers cannot allocate at that point:
// a host that is capturing its own CUDA graph (allocation calls are not
// allowed inside a stream capture in the modes such hosts use), or a host
// whose device memory is entirely handed out by its own pool allocator with
// no headroom for other allocations.  This variant runs the same two kernels
// with the intermediates placed in the file-scope array below instead.
//
// The array is a fixed part of the library image: every GPU that loads the
// library holds PZ_NOALLOC_MAX_MN * 2 complex values (1 MiB) until the process
// exits.  All calls on a device share it, so calls that overlap on the GPU (on
// different streams, or from different handles) race on it; order them.  The
// first kernel writes every element the second one reads, so nothing has to
// be cleared between calls even though the array keeps the last call's data.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "pizza_gpu.h"
#include "pz_internal.h"
#include "pz_stage.h"

#define PZ_NOALLOC_MAX_DEVICES 64

// n_m_max * n_r_max complex values per intermediate, two intermediates
static __device__ __align__(256) double2 pz_noalloc_scratch[2 * PZ_NOALLOC_MAX_MN];

namespace {
std::mutex g_mutex;
double2* g_scratch[PZ_NOALLOC_MAX_DEVICES] = {};   // device address of the array, per device
}  // namespace

extern "C" int pz_explicit_terms_noalloc(pz_handle* h, int inst, const double* us, const double* up,
                                         const double* om, const double* temp, double* dTdt_expl,
                                         double* dpsidt_expl, double* dtr, double* dth) {
  PzExplArgs a;
  int N = 0, M = 0, P = 0;
  cudaStream_t s = nullptr;
  int rc = pz_expl_args(h, inst, us, up, om, temp, dTdt_expl, dpsidt_expl, dtr, dth, &a, &N, &M, &P, &s);
  if (rc != PZ_OK) return rc;
  if ((long long)N * M > PZ_NOALLOC_MAX_MN) {
    const std::string msg = "pz_explicit_terms_noalloc: n_m_max*n_r_max = " + std::to_string((long long)N * M) +
                            " exceeds the maximum " + std::to_string(PZ_NOALLOC_MAX_MN) +
                            " of the static scratch array; use pz_explicit_terms";
    return pz_record_error(h, PZ_E_ARG, msg.c_str());
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return pz_record_error(h, PZ_E_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= PZ_NOALLOC_MAX_DEVICES) return pz_record_error(h, PZ_E_ARG, "device index too large");
  double2* base = nullptr;
  {
    // set-up, once per device, with that device current: the device address
    // of the array (the host-side symbol is only a stand-in)
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, pz_noalloc_scratch);
      if (e != cudaSuccess) {
        const std::string msg = std::string("pz_explicit_terms_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
        return pz_record_error(h, PZ_E_CUDA, msg.c_str());
      }
      g_scratch[dev] = static_cast<double2*>(p);
    }
    base = g_scratch[dev];
  }
  a.s_dVsT = base;
  a.s_dVsOm = base + PZ_NOALLOC_MAX_MN;
  e = pz_launch_explicit_terms(a, N, M, P, s);
  if (e != cudaSuccess) return pz_record_error(h, PZ_E_CUDA, cudaGetErrorString(e));
  return PZ_OK;
}
