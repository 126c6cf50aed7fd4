// evr_noalloc.cu -- H.psi entry point that allocates nothing.
//
// Callers such as a Fortran host that owns all device memory through its own pool, or
// code that must not enter the CUDA allocator at that point of its run, cannot let the
// library call cudaMalloc on the H.psi path.  evr_hpsi_noalloc runs the FP64 H.psi
// pipeline with every scratch buffer (item counter, term-basis output, per-CTA work
// buffers) carved out of one fixed, file-scope device array.  The array costs every GPU
// that loads the library kNoAllocScratchBytes of device memory until the process exits.
#include <mutex>

#include "evr_internal.h"

namespace {

// 32 MiB: enough for small and medium problems (for example the 4-mode level-5 Smolyak
// problem of the tests); larger problems are rejected with EVR_EINVAL.
constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device.  The array's name in host
// code is only a host-side handle, so the address is looked up once per device (with
// that device current) and cached.
int scratch_address(evr_ctx* c, unsigned char** out) {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (c->device < 0 || c->device >= kMaxDevices) return evr::set_error(c, EVR_EINVAL, "device index");
  if (!g_scratch_ptr[c->device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      (void)cudaGetLastError();
      return evr::set_error(c, EVR_EDEVICE, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    }
    g_scratch_ptr[c->device] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[c->device];
  return EVR_OK;
}

}  // namespace

extern "C" int evr_hpsi_noalloc(evr_ctx* c, const double* psi, int64_t ld_psi, double* hpsi, int64_t ld_hpsi,
                                int nvec, void* stream) {
  if (!c) return EVR_EINVAL;
  if (c->host_only) return evr::set_error(c, EVR_EDEVICE, "host-only context (created with device < 0)");
  if (!psi || !hpsi || nvec < 1 || ld_psi < nvec || ld_hpsi < nvec)
    return evr::set_error(c, EVR_EINVAL, "evr_hpsi_noalloc: null pointer, nvec < 1 or ld < nvec");
  if (cudaSetDevice(c->device) != cudaSuccess) {
    (void)cudaGetLastError();
    return evr::set_error(c, EVR_EDEVICE, "cudaSetDevice");
  }
  unsigned char* scratch = nullptr;
  int rc = scratch_address(c, &scratch);
  if (rc) return rc;
  cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
  return evr::hpsi_scratch(c, psi, ld_psi, hpsi, ld_hpsi, nvec, scratch, kNoAllocScratchBytes, s);
}
