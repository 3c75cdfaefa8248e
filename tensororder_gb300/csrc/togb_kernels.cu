// CUDA kernels of the contraction path (sm_103a).
//
// Two join kernels cover every pairwise contraction of binary-index tensors:
//
//  * k_direct -- one thread per output entry, a K-long dot product with
//    deposit addressing.  Used when one GEMM extent is small (outer products,
//    matrix-vector shapes, the tiny joins that dominate the join count).
//  * k_tiled  -- 64x64x16 shared-memory tiled GEMM, 4x4 register blocking.
//    Tiles are gathered through per-CTA offset tables, so any axis
//    permutation of either operand is read in place (no transpose pass).
//
// Both are templated on the form:
//  * MODE 0 (FP64): FP64 storage and FMA.
//  * MODE 1 (split): FP32 storage; each (tensor, slice) carries a
//    power-of-two exponent.  Inputs are normalised on load so that their
//    slice maximum lies in [1, 2) (exact scaling), products accumulate with
//    FP32 FMA, and the output records its exponent and its maximum (atomicMax
//    on the IEEE bits, valid because every entry is >= 0).
#include <cuda_runtime.h>

#include "togb_internal.h"

namespace togb {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int64_t deposit(const int64_t* s, uint64_t x) {
  int64_t off = 0;
  while (x) {
    const int i = __ffsll((long long)x) - 1;
    off += s[i];
    x &= x - 1;
  }
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
  return o.max_ptr ? shift_from_max(o.max_ptr[b]) : o.leaf_shift;
}

__device__ __forceinline__ int op_exp(const OpDesc& o, int b) { return o.exp_ptr ? o.exp_ptr[b] : 0; }

template <int MODE, class T>
__global__ void __launch_bounds__(kThreads) k_direct(const __grid_constant__ JoinDesc jd,
                                                     const int64_t* __restrict__ d_s0, int nslices) {
  const int mnb = jd.mb + jd.nb;
  const int64_t total = (int64_t)nslices << mnb;
  const int64_t total_pad = (total + 31) & ~(int64_t)31;
  const int64_t s0 = d_s0 ? *d_s0 : 0;
  const int K = 1 << jd.kb;
  const T* __restrict__ A = (const T*)jd.a.ptr;
  const T* __restrict__ B = (const T*)jd.b.ptr;
  T* __restrict__ C = (T*)jd.c_ptr;
  const uint64_t nmask = (1ull << jd.nb) - 1;
  const uint64_t mnmask = (1ull << mnb) - 1;
  const int group = mnb >= 5 ? 32 : (1 << mnb);  // lanes that share one slice
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total_pad;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const bool valid = idx < total;
    T acc = 0;
    int b = 0;
    uint64_t mn = 0;
    int sa = 0, sb = 0;
    if (valid) {
      b = (int)(idx >> mnb);
      mn = (uint64_t)idx & mnmask;
      const uint64_t m = mn >> jd.nb, n = mn & nmask;
      const int64_t s = s0 + b;
      const T* pa = A + slice_offset(jd.a, b, s) + deposit(jd.a.s_outer, m);
      const T* pb = B + slice_offset(jd.b, b, s) + deposit(jd.b.s_outer, n);
      T fa = 1, fb = 1;
      if (MODE == 1) {
        sa = op_shift(jd.a, b);
        sb = op_shift(jd.b, b);
        fa = (T)pow2f(sa);
        fb = (T)pow2f(sb);
      }
      int64_t ka = 0, kb = 0;
      for (int k = 0; k < K; ++k) {
        if (MODE == 1)
          acc = fmaf((float)pa[ka] * (float)fa, (float)pb[kb] * (float)fb, (float)acc);
        else
          acc = fma(pa[ka], pb[kb], acc);
        const int t = __ffs(~k) - 1;
        ka += jd.a.dk[t];
        kb += jd.b.dk[t];
      }
      C[(int64_t)b * jd.c_batch_stride + deposit(jd.c_s_m, m) + deposit(jd.c_s_n, n)] = acc;
    }
    if (MODE == 1) {
      uint32_t bits = valid ? __float_as_uint((float)acc) : 0u;
      for (int off = 1; off < group; off <<= 1) bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, off));
      if (valid && (threadIdx.x & (group - 1)) == 0) atomicMax(&jd.c_max[b], bits);
      if (valid && mn == 0) jd.c_exp[b] = op_exp(jd.a, b) + op_exp(jd.b, b) - sa - sb;
    }
  }
}

template <int MODE, class T>
__global__ void __launch_bounds__(kThreads) k_tiled(const __grid_constant__ JoinDesc jd,
                                                    const int64_t* __restrict__ d_s0, int nslices,
                                                    int tiles_n_bits) {
  constexpr int BM = 64, BN = 64, BK = 16;
  constexpr int PAD = sizeof(T) == 8 ? 2 : 4;
  __shared__ __align__(16) T As[BK][BM + PAD];
  __shared__ __align__(16) T Bs[BK][BN + PAD];
  __shared__ int64_t tAm[BM], tBn[BN], tCm[BM], tCn[BN], tAk[BK], tBk[BK];
  __shared__ uint32_t red[kThreads / 32];

  const int b = blockIdx.y + blockIdx.z * gridDim.y;
  if (b >= nslices) return;
  const int tid = threadIdx.x;
  const int64_t s = (d_s0 ? *d_s0 : 0) + b;
  const uint64_t tile = blockIdx.x;
  const uint64_t m0 = (tile >> tiles_n_bits) * BM;
  const uint64_t n0 = (tile & ((1ull << tiles_n_bits) - 1)) * BN;
  const int64_t M = 1ll << jd.mb, N = 1ll << jd.nb, K = 1ll << jd.kb;
  const int mlim = (int)min((int64_t)BM, M - (int64_t)m0);
  const int nlim = (int)min((int64_t)BN, N - (int64_t)n0);
  const int klim = (int)min((int64_t)BK, K);

  if (tid < BM) {
    tAm[tid] = deposit(jd.a.s_outer, tid);
    tCm[tid] = deposit(jd.c_s_m, tid);
  } else if (tid < BM + BN) {
    const int i = tid - BM;
    tBn[i] = deposit(jd.b.s_outer, i);
    tCn[i] = deposit(jd.c_s_n, i);
  } else if (tid < BM + BN + BK) {
    const int i = tid - BM - BN;
    tAk[i] = deposit(jd.a.s_k, i);
    tBk[i] = deposit(jd.b.s_k, i);
  }
  const T* __restrict__ A = (const T*)jd.a.ptr + slice_offset(jd.a, b, s) + deposit(jd.a.s_outer, m0);
  const T* __restrict__ B = (const T*)jd.b.ptr + slice_offset(jd.b, b, s) + deposit(jd.b.s_outer, n0);
  int sa = 0, sb = 0;
  T fa = 1, fb = 1;
  if (MODE == 1) {
    sa = op_shift(jd.a, b);
    sb = op_shift(jd.b, b);
    fa = (T)pow2f(sa);
    fb = (T)pow2f(sb);
  }
  __syncthreads();

  const int tx = tid & 15, ty = tid >> 4;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0;

  for (int64_t k0 = 0; k0 < K; k0 += BK) {
    const int64_t dak = deposit(jd.a.s_k, (uint64_t)k0);
    const int64_t dbk = deposit(jd.b.s_k, (uint64_t)k0);
#pragma unroll
    for (int r = 0; r < (BM * BK) / kThreads; ++r) {
      const int e = tid + kThreads * r;
      int i, kk;
      if (jd.a.k_fast) { kk = e & (BK - 1); i = e >> 4; } else { i = e & (BM - 1); kk = e >> 6; }
      T v = 0;
      if (i < mlim && kk < klim) v = A[dak + tAm[i] + tAk[kk]];
      if (MODE == 1) v *= fa;
      As[kk][i] = v;
    }
#pragma unroll
    for (int r = 0; r < (BN * BK) / kThreads; ++r) {
      const int e = tid + kThreads * r;
      int i, kk;
      if (jd.b.k_fast) { kk = e & (BK - 1); i = e >> 4; } else { i = e & (BN - 1); kk = e >> 6; }
      T v = 0;
      if (i < nlim && kk < klim) v = B[dbk + tBn[i] + tBk[kk]];
      if (MODE == 1) v *= fb;
      Bs[kk][i] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }

  T* __restrict__ C = (T*)jd.c_ptr + (int64_t)b * jd.c_batch_stride + deposit(jd.c_s_m, m0) +
                      deposit(jd.c_s_n, n0);
  uint32_t bits = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int row = ty * 4 + i;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int col = tx * 4 + j;
      if (row < mlim && col < nlim) {
        C[tCm[row] + tCn[col]] = acc[i][j];
        if (MODE == 1) bits = max(bits, __float_as_uint((float)acc[i][j]));
      }
    }
  }
  if (MODE == 1) {
    for (int off = 16; off > 0; off >>= 1) bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, off));
    if ((tid & 31) == 0) red[tid >> 5] = bits;
    __syncthreads();
    if (tid == 0) {
      uint32_t m = 0;
      for (int w = 0; w < kThreads / 32; ++w) m = max(m, red[w]);
      atomicMax(&jd.c_max[b], m);
      if (tile == 0) jd.c_exp[b] = op_exp(jd.a, b) + op_exp(jd.b, b) - sa - sb;
    }
  }
}

// Compensated (Neumaier) accumulation of every slice's root tensor, in slice
// order, into the FP64 accumulator.
template <int MODE, class T>
__global__ void k_root(const __grid_constant__ RootDesc rd, const int64_t* __restrict__ d_s0, int nslices) {
  const int64_t E = 1ll << rd.r.outer_bits;
  const int64_t s0 = d_s0 ? *d_s0 : 0;
  const T* __restrict__ R = (const T*)rd.r.ptr;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    double sum = rd.acc_sum[e], comp = rd.acc_comp[e];
    const int64_t oe = deposit(rd.r.s_outer, (uint64_t)e);
    for (int b = 0; b < nslices; ++b) {
      double x = (double)R[slice_offset(rd.r, b, s0 + b) + oe];
      if (MODE == 1) x = ldexp(x, op_exp(rd.r, b));
      const double t = sum + x;
      if (fabs(sum) >= fabs(x)) comp += (sum - t) + x; else comp += (x - t) + sum;
      sum = t;
    }
    rd.acc_sum[e] = sum;
    rd.acc_comp[e] = comp;
  }
}

__global__ void k_set_s0(int64_t* p, int64_t v) { *p = v; }

template <class T>
__global__ void __launch_bounds__(kThreads) k_probe(T* out, int iters, T seed) {
  T a0 = seed + (T)threadIdx.x, a1 = a0 + (T)1, a2 = a0 + (T)2, a3 = a0 + (T)3;
  T a4 = a0 + (T)4, a5 = a0 + (T)5, a6 = a0 + (T)6, a7 = a0 + (T)7;
  const T m = (T)0.999999, c = (T)1e-7;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
    a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
  }
  const T r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (r == (T)-1) out[0] = r;
}

int grid_for(int64_t work) {
  const int64_t blocks = (work + kThreads - 1) / kThreads;
  const int64_t cap = 152 * 32;
  return (int)(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
}

}  // namespace

cudaError_t launch_join(int mode, int kernel, const JoinDesc& jd, const int64_t* s0, int nslices,
                        cudaStream_t st) {
  if (kernel == K_TILED) {
    const int tm_bits = jd.mb > 6 ? jd.mb - 6 : 0;
    const int tn_bits = jd.nb > 6 ? jd.nb - 6 : 0;
    const uint64_t tiles = 1ull << (tm_bits + tn_bits);
    if (tiles > 0x7fffffffull) return cudaErrorInvalidValue;
    const int gy = nslices < 65535 ? nslices : 65535;
    const int gz = (nslices + gy - 1) / gy;
    dim3 grid((unsigned)tiles, gy, gz);
    if (mode == 0) k_tiled<0, double><<<grid, kThreads, 0, st>>>(jd, s0, nslices, tn_bits);
    else k_tiled<1, float><<<grid, kThreads, 0, st>>>(jd, s0, nslices, tn_bits);
  } else {
    const int64_t work = (int64_t)nslices << (jd.mb + jd.nb);
    const int g = grid_for(work);
    if (mode == 0) k_direct<0, double><<<g, kThreads, 0, st>>>(jd, s0, nslices);
    else k_direct<1, float><<<g, kThreads, 0, st>>>(jd, s0, nslices);
  }
  return cudaGetLastError();
}

cudaError_t launch_root(int mode, const RootDesc& rd, const int64_t* s0, int nslices, cudaStream_t st) {
  const int g = grid_for(1ll << rd.r.outer_bits);
  if (mode == 0) k_root<0, double><<<g, kThreads, 0, st>>>(rd, s0, nslices);
  else k_root<1, float><<<g, kThreads, 0, st>>>(rd, s0, nslices);
  return cudaGetLastError();
}

cudaError_t launch_set_s0(int64_t* d_s0, int64_t value, cudaStream_t st) {
  k_set_s0<<<1, 1, 0, st>>>(d_s0, value);
  return cudaGetLastError();
}

cudaError_t probe_peak(int kind, cudaStream_t st, double* flops) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  void* out = nullptr;
  cudaError_t e = cudaMalloc(&out, 16);
  if (e != cudaSuccess) return e;
  const int blocks = sms * 8;
  const int iters = kind == 0 ? 4096 : 65536;
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  for (int rep = 0; rep < 2; ++rep) {  // first pass warms clocks
    cudaEventRecord(t0, st);
    if (kind == 0) k_probe<double><<<blocks, kThreads, 0, st>>>((double*)out, iters, 1.0);
    else k_probe<float><<<blocks, kThreads, 0, st>>>((float*)out, iters, 1.0f);
    cudaEventRecord(t1, st);
  }
  e = cudaEventSynchronize(t1);
  float ms = 0;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(out);
  if (e != cudaSuccess) return e;
  *flops = 2.0 * 8.0 * iters * (double)blocks * kThreads / (ms * 1e-3);
  return cudaGetLastError();
}

}  // namespace togb
