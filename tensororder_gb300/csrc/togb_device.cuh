// Device helpers shared by the kernel files: deposit addressing, slice
// offsets and the split form's power-of-two bookkeeping.
#pragma once
#include <cstdint>

#include "togb_internal.h"

namespace togb {
namespace {

__device__ __forceinline__ int64_t deposit(const int64_t* s, uint64_t x) {
  int64_t off = 0;
  while (x) {
    const int i = __ffsll((long long)x) - 1;
    off += s[i];
    x &= x - 1;
  }
  return off;
}

__device__ __forceinline__ int64_t dep(const Runs& r, uint64_t x) {
  int64_t off = 0;
  for (int i = 0; i < r.n; ++i)
    off += (int64_t)((x >> r.src[i]) & ((1ull << r.len[i]) - 1)) << r.dst[i];
  return off;
}

__device__ __forceinline__ int64_t slice_offset(const OpDesc& o, int b, int64_t s) {
  if (o.batch_stride) return (int64_t)b * o.batch_stride;
  int64_t off = 0;
  for (int j = 0; j < o.n_slice_terms; ++j)
    if ((s >> o.slice_shift[j]) & 1) off += o.slice_stride[j];
  return off;
}

// Power-of-two normaliser that brings a slice maximum into [1, 2).
__device__ __forceinline__ int shift_from_max(uint32_t bits) {
  if (bits == 0) return 0;
  const int e = (int)((bits >> 23) & 0xff);
  int sh = (e == 0) ? 126 : 127 - e;
  return max(-126, min(126, sh));
}

__device__ __forceinline__ float pow2f(int sh) { return __int_as_float((127 + sh) << 23); }

__device__ __forceinline__ int op_shift(const OpDesc& o, int b) {
  return o.max_ptr ? shift_from_max(o.max_ptr[b * o.meta_step]) : o.leaf_shift;
}

__device__ __forceinline__ int op_exp(const OpDesc& o, int b) { return o.exp_ptr ? o.exp_ptr[b * o.meta_step] : 0; }

}  // namespace
}  // namespace togb
