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
// process exits.  The first call on a device looks up the array's device
// address with cudaGetSymbolAddress while that device is current (in host
// code the symbol is only a host-side stand-in: handing it to a kernel would
// fault, or on systems where the GPU can reach host memory read the wrong
// memory).  Make that first call on each device before any stream capture
// begins.  Every call shares the one array and leaves its contents behind;
// the accumulator is cleared at the start of each call, and calls whose work
// overlaps on the GPU race on the array, so serialise them (one stream, or
// events between streams).
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "togb.h"
#include "togb_internal.h"

static __device__ __align__(256) unsigned char g_togb_static_scratch[TOGB_STATIC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 256;
std::mutex g_setup_mutex;
void* g_scratch_address[kMaxDevices] = {};

}  // namespace

extern "C" togb_status togb_contract_static_f64(const togb_program_desc* desc, const double* d_leaf_values,
                                                double* d_out, void* stream) {
  if (!desc || !d_leaf_values || !d_out) return togb::report(TOGB_ERR_INVALID, "null argument");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return togb::report(TOGB_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return togb::report(TOGB_ERR_UNSUPPORTED, "device index out of range");
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_address[dev]) {
      void* addr = nullptr;
      e = cudaGetSymbolAddress(&addr, g_togb_static_scratch);
      if (e != cudaSuccess || !addr) {
        cudaGetLastError();
        return togb::report(TOGB_ERR_CUDA, (std::string("static scratch lookup failed: ") +
                                            cudaGetErrorString(e)).c_str());
      }
      g_scratch_address[dev] = addr;
    }
    scratch = g_scratch_address[dev];
  }
  return togb::static_contract_f64(desc, d_leaf_values, (char*)scratch, TOGB_STATIC_SCRATCH_BYTES, d_out,
                                   (cudaStream_t)stream);
}
