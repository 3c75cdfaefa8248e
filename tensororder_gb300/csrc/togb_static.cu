// togb_contract_static_f64: contract a whole program without allocating any
// device memory.
//
// Some callers cannot call cudaMalloc.  A host application that hands the
// whole device to its own memory pool (a framework caching allocator sized to
// nearly all of HBM, a serving process with a fixed memory budget) gets
// failures or fragmentation from a library that allocates behind its back,
// and cudaMalloc/cudaFree synchronise the device, which stalls every other
// stream of a latency-bound pipeline.  Such a caller owns the input and output
// buffers and needs the library to bring its own scratch.
//
// The scratch is the file-scope array below: TOGB_STATIC_SCRATCH_BYTES of
// device memory that every GPU which loads this library holds until the
// process exits.  The first call in a CUDA context looks up the array's
// device address with cudaGetSymbolAddress while that device is current (in
// host code the symbol is only a host-side stand-in: handing it to a kernel
// would fault, or on systems where the GPU can reach host memory read the
// wrong memory).  The address is cached per device together with the unique id
// of the context it was looked up in; after a cudaDeviceReset the primary
// context is new, the module is loaded again and the array may move, so the
// next call looks it up again.  Make the first call in each context before any
// stream capture begins.  Every call shares the one array and leaves its contents behind;
// the accumulator is cleared at the start of each call, and calls whose work
// overlaps on the GPU race on the array, so serialise them (one stream, or
// events between streams).
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "togb.h"
#include "togb_internal.h"

static __device__ __align__(256) unsigned char g_togb_static_scratch[TOGB_STATIC_SCRATCH_BYTES];

namespace {

using togb::kMaxDevices;
std::mutex g_setup_mutex;
void* g_scratch_address[kMaxDevices] = {};
unsigned long long g_scratch_context[kMaxDevices] = {};  // cuCtxGetId of the context the address belongs to

// The two driver calls, resolved through the runtime so the library carries no
// link-time dependency on the driver library.
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

template <class Fn>
Fn driver_fn(const char* name) {
  void* f = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return (Fn)f;
}

}  // namespace

extern "C" togb_status togb_contract_static_f64(const togb_program_desc* desc, const double* d_leaf_values,
                                                double* d_out, void* stream) {
  if (!desc || !d_leaf_values || !d_out) return togb::report(TOGB_ERR_INVALID, "null argument");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return togb::report(TOGB_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return togb::report(TOGB_ERR_UNSUPPORTED, "device index out of range");
  // The id of the current context tells whether a cached address is still
  // valid.  With no context current yet (this is the process's first CUDA
  // call), cudaSetDevice creates and binds the device's primary context; a
  // context the caller made current is left as it is.
  static const CtxGetCurrentFn get_current = driver_fn<CtxGetCurrentFn>("cuCtxGetCurrent");
  static const CtxGetIdFn get_id = driver_fn<CtxGetIdFn>("cuCtxGetId");
  if (!get_current || !get_id) return togb::report(TOGB_ERR_CUDA, "driver context queries unavailable");
  CUcontext ctx = nullptr;
  unsigned long long ctx_id = 0;
  if (get_current(&ctx) == CUDA_SUCCESS && !ctx && (e = cudaSetDevice(dev)) != cudaSuccess)
    return togb::report(TOGB_ERR_CUDA, cudaGetErrorString(e));
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &ctx_id) != CUDA_SUCCESS)
    return togb::report(TOGB_ERR_CUDA, "no current CUDA context for the static scratch");
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_address[dev] || g_scratch_context[dev] != ctx_id) {
      void* addr = nullptr;
      e = cudaGetSymbolAddress(&addr, g_togb_static_scratch);
      if (e != cudaSuccess || !addr) {
        cudaGetLastError();
        return togb::report(TOGB_ERR_CUDA, (std::string("static scratch lookup failed: ") +
                                            cudaGetErrorString(e)).c_str());
      }
      g_scratch_address[dev] = addr;
      g_scratch_context[dev] = ctx_id;
    }
    scratch = g_scratch_address[dev];
  }
  return togb::static_contract_f64(desc, d_leaf_values, (char*)scratch, TOGB_STATIC_SCRATCH_BYTES, d_out,
                                   (cudaStream_t)stream);
}
