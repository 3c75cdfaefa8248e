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
//  * k_reduce -- one CTA per (slice, output entry) for joins with a few
//    outputs and a long K (the root of a tree is a 1x1xK dot product): strided
//    per-thread partial sums (compensated in the split form), then a pairwise
//    tree across the CTA.
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
      const int64_t oa = slice_offset(jd.a, b, s) + dep(jd.a.r_outer, m);
      const int64_t ob = slice_offset(jd.b, b, s) + dep(jd.b.r_outer, n);
      const T* pa = A + oa;
      const T* pb = B + ob;
      int64_t ka = 0, kb = 0;
      if (MODE == 1) {
        sa = op_shift(jd.a, b);
        sb = op_shift(jd.b, b);
        const float fa = pow2f(sa), fb = pow2f(sb);
        // Leaf operands carry an FP32 residual: a*(hi+lo) = a*hi + a*lo keeps
        // the leaf weights' rounding from becoming a per-variable bias.
        const float* alo = jd.a.ptr_lo ? (const float*)jd.a.ptr_lo + oa : nullptr;
        const float* blo = jd.b.ptr_lo ? (const float*)jd.b.ptr_lo + ob : nullptr;
        float f = 0.f;
        for (int k = 0; k < K; ++k) {
          const float av = (float)pa[ka] * fa, bv = (float)pb[kb] * fb;
          if (alo) f = fmaf(alo[ka] * fa, bv, f);
          if (blo) f = fmaf(av, blo[kb] * fb, f);
          f = fmaf(av, bv, f);
          const int t = __ffs(~k) - 1;
          ka += jd.a.dk[t];
          kb += jd.b.dk[t];
        }
        acc = (T)f;
      } else {
        for (int k = 0; k < K; ++k) {
          acc = fma(pa[ka], pb[kb], acc);
          const int t = __ffs(~k) - 1;
          ka += jd.a.dk[t];
          kb += jd.b.dk[t];
        }
      }
      C[(int64_t)b * jd.c_batch_stride + dep(jd.r_cm, m) + dep(jd.r_cn, n)] = acc;
    }
    if (MODE == 1) {
      uint32_t bits = valid ? __float_as_uint((float)acc) : 0u;
      for (int off = 1; off < group; off <<= 1) bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, off));
      if (valid && (threadIdx.x & (group - 1)) == 0) atomicMax(&jd.c_max[b], bits);
      if (valid && mn == 0) jd.c_exp[b] = op_exp(jd.a, b) + op_exp(jd.b, b) - sa - sb;
    }
  }
}

__device__ __forceinline__ void load4(const float* p, float* v) {
  const float4 x = *reinterpret_cast<const float4*>(p);
  v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
}
__device__ __forceinline__ void load4(const double* p, double* v) {
  const double2 x = reinterpret_cast<const double2*>(p)[0], y = reinterpret_cast<const double2*>(p)[1];
  v[0] = x.x; v[1] = x.y; v[2] = y.x; v[3] = y.y;
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
      load4(&As[kk][ty * 4], av);
      load4(&Bs[kk][tx * 4], bv);
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

// One CTA per (slice, output entry): thread t sums k = t, t+256, ... (k bits
// below 8 come from t, the rest advance with the dk deltas), then a pairwise
// tree over the CTA.  The split form keeps a Kahan-compensated FP32 partial.
template <int MODE, class T>
__global__ void __launch_bounds__(kThreads) k_reduce(const __grid_constant__ JoinDesc jd,
                                                     const int64_t* __restrict__ d_s0, int nslices) {
  constexpr int LOGT = 8;  // kThreads == 1 << LOGT
  __shared__ double red_hi[kThreads / 32];
  __shared__ double red_lo[kThreads / 32];
  const int mnb = jd.mb + jd.nb;
  const int64_t blk = blockIdx.x + (int64_t)blockIdx.y * gridDim.x;
  const int b = (int)(blk >> mnb);
  if (b >= nslices) return;
  const uint64_t mn = (uint64_t)blk & ((1ull << mnb) - 1);
  const uint64_t m = mn >> jd.nb, n = mn & ((1ull << jd.nb) - 1);
  const int64_t s = (d_s0 ? *d_s0 : 0) + b;
  const int tid = threadIdx.x;
  const int64_t oa = slice_offset(jd.a, b, s) + dep(jd.a.r_outer, m);
  const int64_t ob = slice_offset(jd.b, b, s) + dep(jd.b.r_outer, n);
  const T* __restrict__ A = (const T*)jd.a.ptr + oa;
  const T* __restrict__ B = (const T*)jd.b.ptr + ob;
  // Offsets of k = tid, and the per-step delta when k advances by 2^LOGT.
  int64_t ka = dep(jd.a.r_k, (uint64_t)tid), kb = dep(jd.b.r_k, (uint64_t)tid);
  int64_t pa8 = 0, pb8 = 0;
  for (int i = 0; i < LOGT && i < jd.kb; ++i) { pa8 += jd.a.s_k[i]; pb8 += jd.b.s_k[i]; }
  const int64_t steps = (jd.kb > LOGT) ? (1ll << (jd.kb - LOGT)) : (tid < (1 << jd.kb) ? 1 : 0);
  int sa = 0, sb = 0;
  double hi = 0.0, lo = 0.0;
  if (MODE == 1) {
    sa = op_shift(jd.a, b);
    sb = op_shift(jd.b, b);
    const float fa = pow2f(sa), fb = pow2f(sb);
    const float* alo = jd.a.ptr_lo ? (const float*)jd.a.ptr_lo + oa : nullptr;
    const float* blo = jd.b.ptr_lo ? (const float*)jd.b.ptr_lo + ob : nullptr;
    float sum = 0.f, c = 0.f;
    for (int64_t j = 0; j < steps; ++j) {
      const float av = (float)A[ka] * fa, bv = (float)B[kb] * fb;
      float y = av * bv;
      if (alo) y = fmaf(alo[ka] * fa, bv, y);
      if (blo) y = fmaf(av, blo[kb] * fb, y);
      y -= c;
      const float t = sum + y;
      c = (t - sum) - y;
      sum = t;
      const int t8 = __ffsll(~(unsigned long long)j) - 1 + LOGT;
      if (t8 < TOGB_MAXBITS) { ka += jd.a.dk[t8] + pa8; kb += jd.b.dk[t8] + pb8; }
    }
    hi = (double)sum;
    lo = -(double)c;
  } else {
    double sum = 0.0;
    for (int64_t j = 0; j < steps; ++j) {
      sum = fma((double)A[ka], (double)B[kb], sum);
      const int t8 = __ffsll(~(unsigned long long)j) - 1 + LOGT;
      if (t8 < TOGB_MAXBITS) { ka += jd.a.dk[t8] + pa8; kb += jd.b.dk[t8] + pb8; }
    }
    hi = sum;
  }
  // Pairwise tree: warp shuffles, then across warps.
  for (int off = 16; off > 0; off >>= 1) {
    hi += __shfl_xor_sync(0xffffffffu, hi, off);
    lo += __shfl_xor_sync(0xffffffffu, lo, off);
  }
  if ((tid & 31) == 0) { red_hi[tid >> 5] = hi; red_lo[tid >> 5] = lo; }
  __syncthreads();
  if (tid == 0) {
    double h = 0.0, l = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) { h += red_hi[w]; l += red_lo[w]; }
    const double total = h + l;
    T* C = (T*)jd.c_ptr + (int64_t)b * jd.c_batch_stride + dep(jd.r_cm, m) + dep(jd.r_cn, n);
    *C = (T)total;
    if (MODE == 1) {
      atomicMax(&jd.c_max[b], __float_as_uint((float)total));
      if (mn == 0) jd.c_exp[b] = op_exp(jd.a, b) + op_exp(jd.b, b) - sa - sb;
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
    const int64_t oe = dep(rd.r.r_outer, (uint64_t)e);
    for (int b = 0; b < nslices; ++b) {
      const int64_t o = slice_offset(rd.r, b, s0 + b) + oe;
      double x = (double)R[o];
      if (MODE == 1) {
        if (rd.r.ptr_lo) x += (double)((const float*)rd.r.ptr_lo)[o];
        x = ldexp(x, op_exp(rd.r, b));
      }
      const double t = sum + x;
      if (fabs(sum) >= fabs(x)) comp += (sum - t) + x; else comp += (x - t) + sum;
      sum = t;
    }
    rd.acc_sum[e] = sum;
    rd.acc_comp[e] = comp;
  }
}

__global__ void k_set_s0(int64_t* p, int64_t v) { *p = v; }

__global__ void k_finalize(const double* __restrict__ acc, int64_t E, double* __restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = acc[e] + acc[E + e];
}

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
  } else if (kernel == K_REDUCE) {
    const int64_t blocks = (int64_t)nslices << (jd.mb + jd.nb);
    const unsigned gx = (unsigned)(blocks < 65536 ? blocks : 65536);
    const unsigned gy = (unsigned)((blocks + gx - 1) / gx);
    if (gy > 65535) return cudaErrorInvalidValue;
    if (mode == 0) k_reduce<0, double><<<dim3(gx, gy), kThreads, 0, st>>>(jd, s0, nslices);
    else k_reduce<1, float><<<dim3(gx, gy), kThreads, 0, st>>>(jd, s0, nslices);
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

cudaError_t launch_finalize(const double* acc, int64_t E, double* out, cudaStream_t st) {
  k_finalize<<<grid_for(E), kThreads, 0, st>>>(acc, E, out);
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
