// CUDA kernels of the contraction path (sm_103a).
//
// The CUDA-core join kernels (the tensor-core GEMM joins are in togb_umma_ws.cu
// and togb_umma.cu) cover every pairwise contraction of binary-index tensors:
//
//  * k_direct -- one thread per output entry, a K-long dot product with
//    deposit addressing.  Used when one GEMM extent is small (outer products,
//    matrix-vector shapes, the tiny joins that dominate the join count).  Two
//    variants take over when the shapes allow, with the same arithmetic per
//    output: k_direct_staged (short K, operand rows staged per output tile)
//    and k_stream (a long operand against a tiny one, 16-byte vectors).
//  * k_tiled  -- 64x64x16 shared-memory tiled GEMM, 4x4 register blocking.
//    Tiles are gathered through per-CTA offset tables, so any axis
//    permutation of either operand is read in place (no transpose pass).
//  * k_reduce -- one CTA per (slice, output entry) for joins with a few
//    outputs and a long K (the root of a tree is a 1x1xK dot product): strided
//    per-thread partial sums (compensated in the split form), then a pairwise
//    tree across the CTA.  k_reduce_vec reads contiguous K runs as vectors.
//  * k_once_list -- one launch for a list of slice-invariant thread-per-output
//    joins, CTAs claiming output tiles in dependency order.
//
// They are templated on the form:
//  * MODE 0 (FP64): FP64 storage and FMA.
//  * MODE 1 (split): FP32 storage; each (tensor, slice) carries a
//    power-of-two exponent.  Inputs are normalised on load so that their
//    slice maximum lies in [1, 2) (exact scaling), products accumulate with
//    FP32 FMA, and the output records its exponent and its maximum (atomicMax
//    on the IEEE bits, valid because every entry is >= 0).
#include <cuda_runtime.h>

#include <atomic>
#include <cstring>
#include <type_traits>

#include "togb_internal.h"
#include "togb_device.cuh"

namespace togb {
namespace {

constexpr int kThreads = 256;

// Element type of the int forms: 64-bit words.  MODE 2 (int form) wraps
// modulo 2^64, which gives int64 and uint64 sums and products bit for bit;
// MODE 3 (residue form) keeps residues modulo a prime p < 2^28.
using u64 = unsigned long long;

// The FP64 form's multiply-add is an FMA; the int form's wraps.
__device__ __forceinline__ double mad(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float mad(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ u64 mad(u64 a, u64 b, u64 c) { return a * b + c; }

// x mod p for x < 2^63 by Barrett reduction, m = floor((2^64 - 1) / p):
// q = floor(x * m / 2^64) is floor(x / p) or one less (x * m / 2^64 falls short
// of x / p by less than x / 2^64 + x / (p 2^64) < 1), so one conditional
// subtraction finishes.
__device__ __forceinline__ u64 mod_reduce(u64 x, u64 p, u64 m) {
  const u64 r = x - __umul64hi(x, m) * p;
  return r >= p ? r - p : r;
}

// The form's multiply-add and sum of two words.  Residues a, b, c < p < 2^28
// give a * b + c < 2^57.  The modulus arguments are unused outside MODE 3.
template <int MODE, class T>
__device__ __forceinline__ T madm(T a, T b, T c, u64 p, u64 m) {
  if constexpr (MODE == 3) return mod_reduce(a * b + c, p, m);
  else return mad(a, b, c);
}
template <int MODE>
__device__ __forceinline__ u64 addm(u64 a, u64 b, u64 p) {
  if constexpr (MODE == 3) {
    const u64 s = a + b;
    return s >= p ? s - p : s;
  } else {
    return a + b;
  }
}

// 16-byte vector of an element type.
template <class T> struct Vec16;
template <> struct Vec16<float> { using type = float4; };
template <> struct Vec16<double> { using type = double2; };
template <> struct Vec16<u64> { using type = ulonglong2; };

// Sum of one word per thread over the CTA in the form's arithmetic (MODE 2
// wrapping, MODE 3 modulo p); the total in thread 0.  Every thread of the CTA
// must call it.
template <int MODE>
__device__ __forceinline__ u64 block_sum(u64 v, u64 p) {
  __shared__ u64 red[kThreads / 32];
  for (int off = 16; off > 0; off >>= 1) v = addm<MODE>(v, __shfl_xor_sync(0xffffffffu, v, off), p);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  u64 t = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kThreads / 32; ++w) t = addm<MODE>(t, red[w], p);
  return t;
}

// Dot product of one output over K.  KK > 0: K == KK <= 16, offsets from the
// per-join table and every load issued before the FMAs; KK == 0: any K, offsets
// advanced with the dk deltas.  Split form: inputs scaled by fa/fb (exact powers
// of two), leaf residuals folded in.
template <int MODE, class T, int KK>
__device__ __forceinline__ T dot_k(const JoinDesc& jd, const T* __restrict__ A, const T* __restrict__ B,
                                   int64_t oa, int64_t ob, int K, float fa, float fb) {
  if constexpr (KK > 0) {
    T av[KK], bv[KK];
#pragma unroll
    for (int k = 0; k < KK; ++k) {
      av[k] = A[oa + jd.a.ktab[k]];
      bv[k] = B[ob + jd.b.ktab[k]];
    }
    if (MODE == 1) {
      float f = 0.f;
      if (jd.a.ptr_lo) {
        const float* lo = (const float*)jd.a.ptr_lo + oa;
#pragma unroll
        for (int k = 0; k < KK; ++k) f = fmaf(lo[jd.a.ktab[k]] * fa, (float)bv[k] * fb, f);
      }
      if (jd.b.ptr_lo) {
        const float* lo = (const float*)jd.b.ptr_lo + ob;
#pragma unroll
        for (int k = 0; k < KK; ++k) f = fmaf((float)av[k] * fa, lo[jd.b.ktab[k]] * fb, f);
      }
#pragma unroll
      for (int k = 0; k < KK; ++k) f = fmaf((float)av[k] * fa, (float)bv[k] * fb, f);
      return (T)f;
    } else {
      T acc = 0;
#pragma unroll
      for (int k = 0; k < KK; ++k) acc = madm<MODE, T>(av[k], bv[k], acc, jd.mod_p, jd.mod_m);
      return acc;
    }
  } else {
    int64_t ka = 0, kb = 0;
    if (MODE == 1) {
      // FP32 partials of 16 terms, added into a compensated (Neumaier) sum:
      // the error stays near 16 rounding errors whatever K is.
      const float* alo = jd.a.ptr_lo ? (const float*)jd.a.ptr_lo + oa : nullptr;
      const float* blo = jd.b.ptr_lo ? (const float*)jd.b.ptr_lo + ob : nullptr;
      float sum = 0.f, comp = 0.f;
      for (int k0 = 0; k0 < K; k0 += 16) {
        float f = 0.f;
        for (int k = k0; k < k0 + 16 && k < K; ++k) {
          const float av = (float)A[oa + ka] * fa, bv = (float)B[ob + kb] * fb;
          if (alo) f = fmaf(alo[ka] * fa, bv, f);
          if (blo) f = fmaf(av, blo[kb] * fb, f);
          f = fmaf(av, bv, f);
          const int t = __ffs(~k) - 1;
          ka += jd.a.dk[t];
          kb += jd.b.dk[t];
        }
        const float t = sum + f;
        comp += fabsf(sum) >= fabsf(f) ? (sum - t) + f : (f - t) + sum;
        sum = t;
      }
      return (T)(sum + comp);
    } else {
      T acc = 0;
      for (int k = 0; k < K; ++k) {
        acc = madm<MODE, T>(A[oa + ka], B[ob + kb], acc, jd.mod_p, jd.mod_m);
        const int t = __ffs(~k) - 1;
        ka += jd.a.dk[t];
        kb += jd.b.dk[t];
      }
      return acc;
    }
  }
}

__device__ __forceinline__ void store_vec(float* p, const float* v) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void store_vec(double* p, const double* v) {
  reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
}
__device__ __forceinline__ void store_vec(u64* p, const u64* v) {
  reinterpret_cast<ulonglong2*>(p)[0] = make_ulonglong2(v[0], v[1]);
  reinterpret_cast<ulonglong2*>(p)[1] = make_ulonglong2(v[2], v[3]);
}

// Thread-per-output kernel: each thread computes VEC consecutive outputs in
// the output's own address order (slice-major), so every store is a
// contiguous vector store whatever order the consumer asked for; 2*VEC*K
// loads are in flight at once.  The operand offsets of an output address q
// are sums of per-bit contributions (address bit -> m or n bit -> operand
// stride), so each block tabulates them for q's four 6-bit digits in shared
// memory: an output costs two table reads per operand, not a walk over the
// bit runs of its layouts.
template <int MODE, class T, int KK, int VEC>
__global__ void __launch_bounds__(kThreads) k_direct(const __grid_constant__ JoinDesc jd,
                                                     const int64_t* __restrict__ d_s0, int nslices) {
  __shared__ int32_t tabA[4][64], tabB[4][64];
  const int mnb = jd.mb + jd.nb;
  const uint64_t nmask = (1ull << jd.nb) - 1;
  const uint64_t mnmask = (1ull << mnb) - 1;
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    const int lvl = i >> 6;
    const uint64_t q = ((uint64_t)(i & 63) << (6 * lvl)) & mnmask;
    const uint64_t m = jd.c_natural ? (q >> jd.nb) : (uint64_t)dep(jd.r_inv_m, q);
    const uint64_t n = jd.c_natural ? (q & nmask) : (uint64_t)dep(jd.r_inv_n, q);
    tabA[lvl][i & 63] = (int32_t)dep(jd.a.r_outer, m);
    tabB[lvl][i & 63] = (int32_t)dep(jd.b.r_outer, n);
  }
  __syncthreads();
  const int64_t groups = ((int64_t)nslices << mnb) / VEC;
  const int64_t groups_pad = (groups + 31) & ~(int64_t)31;
  const int64_t per_slice = (1ll << mnb) / VEC;  // groups per slice (power of two)
  const int lanes = per_slice >= 32 ? 32 : (int)per_slice;
  const int64_t s0 = d_s0 ? *d_s0 : 0;
  const int K = 1 << jd.kb;
  const T* __restrict__ A = (const T*)jd.a.ptr;
  const T* __restrict__ B = (const T*)jd.b.ptr;
  T* __restrict__ C = (T*)jd.c_ptr;
  // Split form: each lane group keeps the running maximum of its current slice
  // across iterations and publishes it (one atomic per group) only when the
  // slice changes, so a large single-slice output costs a few atomics per warp
  // rather than one per iteration.  Every flush decision is warp-uniform.
  uint32_t carry = 0;
  int carry_b = -1;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < groups_pad;
       g += (int64_t)gridDim.x * blockDim.x) {
    const bool valid = g < groups;
    const int64_t idx0 = g * VEC;
    const int b = valid ? (int)(idx0 >> mnb) : 0;
    uint32_t bits = 0;
    int sa = 0, sb = 0;
    if (valid) {
      const int64_t s = s0 + b;
      const uint64_t q0 = (uint64_t)idx0 & mnmask;  // output address within the slice
      int64_t soa = slice_offset(jd.a, b, s), sob = slice_offset(jd.b, b, s);
      if (mnb > 24) {  // address bits above the tables
        const uint64_t qh = q0 & ~((1ull << 24) - 1);
        const uint64_t m = jd.c_natural ? (qh >> jd.nb) : (uint64_t)dep(jd.r_inv_m, qh);
        const uint64_t n = jd.c_natural ? (qh & nmask) : (uint64_t)dep(jd.r_inv_n, qh);
        soa += dep(jd.a.r_outer, m);
        sob += dep(jd.b.r_outer, n);
      }
      soa += tabA[3][(q0 >> 18) & 63] + tabA[2][(q0 >> 12) & 63] + tabA[1][(q0 >> 6) & 63];
      sob += tabB[3][(q0 >> 18) & 63] + tabB[2][(q0 >> 12) & 63] + tabB[1][(q0 >> 6) & 63];
      float fa = 1.f, fb = 1.f;
      if (MODE == 1) {
        sa = op_shift(jd.a, b);
        sb = op_shift(jd.b, b);
        fa = pow2f(sa);
        fb = pow2f(sb);
      }
      T out[VEC];
#pragma unroll
      for (int j = 0; j < VEC; ++j) {
        const int lo = (int)((q0 + j) & 63);  // VEC divides 64: the upper digits are shared
        out[j] = dot_k<MODE, T, KK>(jd, A, B, soa + tabA[0][lo], sob + tabB[0][lo], K, fa, fb);
      }
      if (VEC == 4) {
        store_vec(C + idx0, out);  // program outputs are dense per slice: address = linear index
      } else {
#pragma unroll
        for (int j = 0; j < VEC; ++j) C[idx0 + j] = out[j];
      }
      if (MODE == 1) {
#pragma unroll
        for (int j = 0; j < VEC; ++j) bits = max(bits, __float_as_uint((float)out[j]));
        if ((idx0 & (int64_t)mnmask) == 0) jd.c_exp[b] = op_exp(jd.a, b) + op_exp(jd.b, b) - sa - sb;
      }
    }
    if (MODE == 1) {
      if (__any_sync(0xffffffffu, valid && b != carry_b)) {
        uint32_t v = carry;
        for (int off = 1; off < lanes; off <<= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, off));
        if (carry_b >= 0 && (threadIdx.x & (lanes - 1)) == 0) atomicMax(&jd.c_max[carry_b], v);
        carry = 0;
        carry_b = -1;
      }
      if (valid) {
        carry = max(carry, bits);
        carry_b = b;
      }
    }
  }
  if (MODE == 1) {
    uint32_t v = carry;
    for (int off = 1; off < lanes; off <<= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, off));
    if (carry_b >= 0 && (threadIdx.x & (lanes - 1)) == 0) atomicMax(&jd.c_max[carry_b], v);
  }
}

// Thread-per-output kernel with staged operands, for short K (KK <= 16).
// Each CTA takes tiles of 2^T consecutive output addresses of one slice.  The
// T lowest address bits belong to lm bits of m and ln bits of n (lm + ln = T),
// so a tile reads just 2^lm rows of A and 2^ln rows of B: the CTA loads those
// rows (K values each; in the split form already scaled to the slice maximum)
// into shared memory, then every thread computes four consecutive outputs from
// shared memory and stores them as one vector.
// Output addresses are dense per slice, so a tile is one contiguous run.
// When one operand does not vary with the slice, every CTA walks a contiguous
// range of tiles with the slice index fastest and keeps that operand's rows
// staged while the tile position stays the same: only the other operand's
// rows are loaded again for each slice.
struct StageInfo {
  int T, lm, ln;
  int slice_fast;       // tiles ordered slice-fastest in contiguous CTA ranges
  int a_inv, b_inv;     // the operand is the same for every slice
  int a_row_bits[14];   // A s_outer index of the r-th staged m bit
  int b_row_bits[14];
};

// One staged row of KK values from shared memory, in 16-byte (or 8-byte)
// pieces where the row size allows.
template <class T, int KK>
__device__ __forceinline__ void lds_row(const T* __restrict__ p, T* v) {
  constexpr int BYTES = KK * (int)sizeof(T);
  if constexpr (BYTES % 16 == 0) {
#pragma unroll
    for (int c = 0; c < BYTES / 16; ++c) {
      if constexpr (sizeof(T) == 4) {
        const float4 x = reinterpret_cast<const float4*>(p)[c];
        v[4 * c] = x.x; v[4 * c + 1] = x.y; v[4 * c + 2] = x.z; v[4 * c + 3] = x.w;
      } else {
        const typename Vec16<T>::type x = reinterpret_cast<const typename Vec16<T>::type*>(p)[c];
        v[2 * c] = x.x; v[2 * c + 1] = x.y;
      }
    }
  } else if constexpr (BYTES == 8 && sizeof(T) == 4) {
    const float2 x = reinterpret_cast<const float2*>(p)[0];
    v[0] = x.x; v[1] = x.y;
  } else {
#pragma unroll
    for (int k = 0; k < KK; ++k) v[k] = p[k];
  }
}

template <int MODE, class T, int KK>
__global__ void __launch_bounds__(kThreads) k_direct_staged(const __grid_constant__ JoinDesc jd,
                                                            const __grid_constant__ StageInfo si,
                                                            const int64_t* __restrict__ d_s0, int nslices) {
  extern __shared__ __align__(16) unsigned char sm_dyn[];
  __shared__ uint16_t IA[3][64], IB[3][64];
  const int TB = si.T;
  const int rowsA = 1 << si.lm, rowsB = 1 << si.ln;
  // Dynamic shared memory: A rows, B rows, leaf residual rows, row offsets.
  T* As = reinterpret_cast<T*>(sm_dyn);
  T* Bs = As + (size_t)rowsA * KK;
  float* Alo = reinterpret_cast<float*>(Bs + (size_t)rowsB * KK);
  float* Blo = Alo + (jd.a.ptr_lo ? (size_t)rowsA * KK : 0);
  int32_t* offA = reinterpret_cast<int32_t*>(Blo + (jd.b.ptr_lo ? (size_t)rowsB * KK : 0));
  int32_t* offB = offA + rowsA;
  const int mnb = jd.mb + jd.nb;
  const uint64_t nmask = (1ull << jd.nb) - 1;
  const uint64_t lowmask = (1ull << TB) - 1;
  // Compaction tables: tile-local address q -> staged row of A and of B.
  for (int i = threadIdx.x; i < 192; i += blockDim.x) {
    const int lvl = i >> 6, x = i & 63;
    const uint64_t q = ((uint64_t)x << (6 * lvl)) & lowmask;
    const uint64_t m = jd.c_natural ? (q >> jd.nb) : (uint64_t)dep(jd.r_inv_m, q);
    const uint64_t n = jd.c_natural ? (q & nmask) : (uint64_t)dep(jd.r_inv_n, q);
    uint32_t ra = 0, rb = 0;
    for (int r = 0; r < si.lm; ++r) ra |= (uint32_t)((m >> si.a_row_bits[r]) & 1) << r;
    for (int r = 0; r < si.ln; ++r) rb |= (uint32_t)((n >> si.b_row_bits[r]) & 1) << r;
    IA[lvl][x] = (uint16_t)ra;
    IB[lvl][x] = (uint16_t)rb;
  }
  // Offsets of the staged rows relative to the tile's base row.
  for (int r = threadIdx.x; r < rowsA; r += blockDim.x) {
    int64_t o = 0;
    for (int b = 0; b < si.lm; ++b)
      if ((r >> b) & 1) o += jd.a.s_outer[si.a_row_bits[b]];
    offA[r] = (int32_t)o;
  }
  for (int r = threadIdx.x; r < rowsB; r += blockDim.x) {
    int64_t o = 0;
    for (int b = 0; b < si.ln; ++b)
      if ((r >> b) & 1) o += jd.b.s_outer[si.b_row_bits[b]];
    offB[r] = (int32_t)o;
  }
  __syncthreads();
  const T* __restrict__ A = (const T*)jd.a.ptr;
  const T* __restrict__ B = (const T*)jd.b.ptr;
  T* __restrict__ C = (T*)jd.c_ptr;
  const int64_t s0 = d_s0 ? *d_s0 : 0;
  const int64_t tiles_per_slice = 1ll << (mnb - TB);
  const int64_t ntiles = (int64_t)nslices * tiles_per_slice;
  const int per_thread = (1 << TB) / (4 * kThreads);  // vector groups per thread: 1 to 16
  int64_t t_begin, t_end, t_step;
  if (si.slice_fast) {
    const int64_t chunk = (ntiles + gridDim.x - 1) / gridDim.x;
    t_begin = (int64_t)blockIdx.x * chunk;
    t_end = min(ntiles, t_begin + chunk);
    t_step = 1;
  } else {
    t_begin = blockIdx.x;
    t_end = ntiles;
    t_step = gridDim.x;
  }
  // Split form: the slice maximum is carried across this CTA's tiles and
  // published (one atomic per warp) only when the slice changes.
  uint32_t carry = 0;
  int carry_b = -1;
  int ja[4], jb[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    ja[j] = IA[0][j];
    jb[j] = IB[0][j];
  }
  int64_t staged_pos = -1;  // tile position whose rows are staged
  int staged_b = -1;        // slice whose rows are staged
  // Slice-fastest ranges step (pos, b) without a division per tile.
  int64_t pos_f = si.slice_fast ? t_begin / nslices : 0;
  int b_f = si.slice_fast ? (int)(t_begin - pos_f * nslices) : 0;
  const int tps_bits = mnb - TB;
  for (int64_t t = t_begin; t < t_end; t += t_step) {
    int b;
    int64_t pos;
    if (si.slice_fast) {
      pos = pos_f;
      b = b_f;
      if (++b_f == nslices) {
        b_f = 0;
        ++pos_f;
      }
    } else {
      b = (int)(t >> tps_bits);
      pos = t & (tiles_per_slice - 1);
    }
    if (MODE == 1 && b != carry_b) {  // block-uniform
      uint32_t v = carry;
      for (int off = 16; off > 0; off >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, off));
      if (carry_b >= 0 && (threadIdx.x & 31) == 0) atomicMax(&jd.c_max[carry_b], v);
      carry = 0;
      carry_b = b;
    }
    const uint64_t qh = (uint64_t)pos << TB;  // tile base address within the slice
    const int64_t s = s0 + b;
    int sa = 0, sb = 0;
    float fa = 1.f, fb = 1.f;
    if (MODE == 1) {
      sa = op_shift(jd.a, b);
      sb = op_shift(jd.b, b);
      fa = pow2f(sa);
      fb = pow2f(sb);
    }
    const bool newA = pos != staged_pos || (!si.a_inv && b != staged_b);
    const bool newB = pos != staged_pos || (!si.b_inv && b != staged_b);
    if (newA || newB) {  // block-uniform
      const uint64_t mh = jd.c_natural ? (qh >> jd.nb) : (uint64_t)dep(jd.r_inv_m, qh);
      const uint64_t nh = jd.c_natural ? (qh & nmask) : (uint64_t)dep(jd.r_inv_n, qh);
      __syncthreads();  // the previous tile's reads of the staged rows are done
      if (newA) {
        const int64_t baseA = slice_offset(jd.a, b, s) + dep(jd.a.r_outer, mh);
        for (int e = threadIdx.x; e < rowsA * KK; e += blockDim.x) {
          const int r = e / KK, k = e - r * KK;
          const int64_t o = baseA + offA[r] + jd.a.ktab[k];
          if (MODE == 1) {  // staged already scaled (exact powers of two)
            As[e] = (T)((float)A[o] * fa);
            if (jd.a.ptr_lo) Alo[e] = ((const float*)jd.a.ptr_lo)[o] * fa;
          } else {
            As[e] = A[o];
          }
        }
      }
      if (newB) {
        const int64_t baseB = slice_offset(jd.b, b, s) + dep(jd.b.r_outer, nh);
        for (int e = threadIdx.x; e < rowsB * KK; e += blockDim.x) {
          const int r = e / KK, k = e - r * KK;
          const int64_t o = baseB + offB[r] + jd.b.ktab[k];
          if (MODE == 1) {
            Bs[e] = (T)((float)B[o] * fb);
            if (jd.b.ptr_lo) Blo[e] = ((const float*)jd.b.ptr_lo)[o] * fb;
          } else {
            Bs[e] = B[o];
          }
        }
      }
      staged_pos = pos;
      staged_b = b;
      __syncthreads();
    }
    uint32_t bits = 0;
#pragma unroll 1
    for (int i = 0; i < per_thread; ++i) {
      const int q0 = 4 * (threadIdx.x + kThreads * i);
      // The row tables are OR-linear in the address bits: the two lowest
      // bits (j) contribute IA[0][j] / IB[0][j] to every group.
      const int ra0 = IA[0][q0 & 63] | IA[1][(q0 >> 6) & 63] | IA[2][(q0 >> 12) & 63];
      const int rb0 = IB[0][q0 & 63] | IB[1][(q0 >> 6) & 63] | IB[2][(q0 >> 12) & 63];
      T out[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int ra = ra0 | ja[j];
        const int rb = rb0 | jb[j];
        T ar[KK], br[KK];
        lds_row<T, KK>(As + ra * KK, ar);
        lds_row<T, KK>(Bs + rb * KK, br);
        if (MODE == 1) {
          float f = 0.f;
          if (jd.a.ptr_lo) {
            float al[KK];
            lds_row<float, KK>(Alo + ra * KK, al);
#pragma unroll
            for (int k = 0; k < KK; ++k) f = fmaf(al[k], (float)br[k], f);
          }
          if (jd.b.ptr_lo) {
            float bl[KK];
            lds_row<float, KK>(Blo + rb * KK, bl);
#pragma unroll
            for (int k = 0; k < KK; ++k) f = fmaf((float)ar[k], bl[k], f);
          }
#pragma unroll
          for (int k = 0; k < KK; ++k) f = fmaf((float)ar[k], (float)br[k], f);
          out[j] = (T)f;
          bits = max(bits, __float_as_uint(f));
        } else {
          T acc = 0;
#pragma unroll
          for (int k = 0; k < KK; ++k) acc = madm<MODE, T>(ar[k], br[k], acc, jd.mod_p, jd.mod_m);
          out[j] = acc;
        }
      }
      store_vec(C + (int64_t)b * jd.c_batch_stride + qh + q0, out);
    }
    if (MODE == 1) {
      carry = max(carry, bits);
      if (qh == 0 && threadIdx.x == 0) jd.c_exp[b] = op_exp(jd.a, b) + op_exp(jd.b, b) - sa - sb;
    }
  }
  if (MODE == 1) {
    uint32_t v = carry;
    for (int off = 16; off > 0; off >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, off));
    if (carry_b >= 0 && (threadIdx.x & 31) == 0) atomicMax(&jd.c_max[carry_b], v);
  }
}

// Streaming variant for joins of a long operand A with a tiny B (K <= 4 with
// N*K <= 16, or K = 8 with N = 1; split form, A without a leaf residual): C[m][n] = sum_k A[m][k] * B[n][k]
// with C row-major (natural).  A's two lowest m bits are either its two lowest
// address bits (KFAST false: each k gives one 16-byte vector of four
// consecutive m) or lie directly above all of its k bits (KFAST true: four
// consecutive m and every k form one run of 4*K values).  Each thread takes
// four consecutive m of one slice: it reads A as K vectors, keeps the slice's
// B (and its residual) in registers, and writes its 4*N outputs, which are
// contiguous, as N vectors.  The arithmetic order per output is dot_k's, so
// the results equal k_direct's bit for bit.
template <int KK, int NN, bool KFAST>
__global__ void __launch_bounds__(kThreads, (KK * NN <= 4 || (KK * NN == 8 && KK >= 2)) ? 4 : (KK * NN == 8 ? 3 : 2))
    k_stream(const __grid_constant__ JoinDesc jd,
                                                     const int64_t* __restrict__ d_s0, int nslices) {
  const int qb = jd.mb - 2;  // log2 of the quads of m per slice
  const int64_t quads = (int64_t)nslices << qb;
  const int64_t quads_pad = (quads + 31) & ~(int64_t)31;
  const int lanes = qb >= 5 ? 32 : (1 << qb);
  const int mnb = jd.mb + jd.nb;
  const int64_t s0 = d_s0 ? *d_s0 : 0;
  const float* __restrict__ A = (const float*)jd.a.ptr;
  const float* __restrict__ B = (const float*)jd.b.ptr;
  const float* __restrict__ Blo = (const float*)jd.b.ptr_lo;
  float* __restrict__ C = (float*)jd.c_ptr;
  // Per-slice state, reloaded when a thread's slice changes.
  int cur = -1, sa = 0, sb = 0;
  float fa = 1.f;
  int64_t abase = 0;
  float bv[KK][NN], bl[KK][NN];
  uint32_t carry = 0;
  int carry_b = -1;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < quads_pad;
       g += (int64_t)gridDim.x * blockDim.x) {
    const bool valid = g < quads;
    const int b = valid ? (int)(g >> qb) : 0;
    uint32_t bits = 0;
    if (valid) {
      if (b != cur) {
        cur = b;
        const int64_t s = s0 + b;
        sa = op_shift(jd.a, b);
        sb = op_shift(jd.b, b);
        fa = pow2f(sa);
        const float fb = pow2f(sb);
        abase = slice_offset(jd.a, b, s);
        const int64_t bbase = slice_offset(jd.b, b, s);
#pragma unroll
        for (int n = 0; n < NN; ++n) {
          const int64_t o = bbase + dep(jd.b.r_outer, (uint64_t)n);
#pragma unroll
          for (int k = 0; k < KK; ++k) {
            bv[k][n] = B[o + jd.b.ktab[k]] * fb;
            bl[k][n] = Blo ? Blo[o + jd.b.ktab[k]] * fb : 0.f;
          }
        }
      }
      const uint64_t m0 = ((uint64_t)g & ((1ull << qb) - 1)) << 2;
      const int64_t ao = abase + dep(jd.a.r_outer, m0);
      float av[4][KK];
      if constexpr (KFAST) {
        float x[4 * KK];
#pragma unroll
        for (int v = 0; v < KK; ++v) {
          const float4 t = *reinterpret_cast<const float4*>(A + ao + 4 * v);
          x[4 * v] = t.x; x[4 * v + 1] = t.y; x[4 * v + 2] = t.z; x[4 * v + 3] = t.w;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int k = 0; k < KK; ++k) av[i][k] = x[i * KK + k] * fa;
      } else {
#pragma unroll
        for (int k = 0; k < KK; ++k) {
          const float4 t = *reinterpret_cast<const float4*>(A + ao + jd.a.ktab[k]);
          av[0][k] = t.x * fa; av[1][k] = t.y * fa; av[2][k] = t.z * fa; av[3][k] = t.w * fa;
        }
      }
      float out[4 * NN];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int n = 0; n < NN; ++n) {
          float f = 0.f;
          if (Blo) {
#pragma unroll
            for (int k = 0; k < KK; ++k) f = fmaf(av[i][k], bl[k][n], f);
          }
#pragma unroll
          for (int k = 0; k < KK; ++k) f = fmaf(av[i][k], bv[k][n], f);
          out[i * NN + n] = f;
          bits = max(bits, __float_as_uint(f));
        }
      float* c = C + ((int64_t)b << mnb) + (int64_t)m0 * NN;
#pragma unroll
      for (int v = 0; v < NN; ++v)
        reinterpret_cast<float4*>(c)[v] = make_float4(out[4 * v], out[4 * v + 1], out[4 * v + 2], out[4 * v + 3]);
      if (m0 == 0) jd.c_exp[b] = op_exp(jd.a, b) + op_exp(jd.b, b) - sa - sb;
    }
    // Slice maximum: carried per lane group, published when the slice changes
    // (warp-uniform decisions, as in k_direct).
    if (__any_sync(0xffffffffu, valid && b != carry_b)) {
      uint32_t v = carry;
      for (int off = 1; off < lanes; off <<= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, off));
      if (carry_b >= 0 && (threadIdx.x & (lanes - 1)) == 0) atomicMax(&jd.c_max[carry_b], v);
      carry = 0;
      carry_b = -1;
    }
    if (valid) {
      carry = max(carry, bits);
      carry_b = b;
    }
  }
  uint32_t v = carry;
  for (int off = 1; off < lanes; off <<= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, off));
  if (carry_b >= 0 && (threadIdx.x & (lanes - 1)) == 0) atomicMax(&jd.c_max[carry_b], v);
}

// Component j (a compile-time constant after unrolling) of a float4.
__device__ __forceinline__ float f4_at(const float4& v, int j) {
  return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}

// k_stream's arithmetic with more loads in flight, for slices of at least
// 32*U quads: each warp takes a block of 32*U consecutive quads of one slice
// (lane l owns quads l, l + 32, ..., so every load and store instruction of
// the warp covers consecutive 16-byte vectors), loads the slice's B and
// normalisers once per block and issues all U*KK vector loads of A before any
// arithmetic.  Per output the FMAs run in k_stream's order, so the results are
// the same bits.
template <int KK, int NN, bool KFAST, int LOGU>
__global__ void __launch_bounds__(kThreads) k_stream_blk(const __grid_constant__ JoinDesc jd,
                                                         const int64_t* __restrict__ d_s0, int nslices) {
  constexpr int U = 1 << LOGU;
  const int wb = jd.mb - 2 - 5 - LOGU;  // log2 of the warp blocks per slice
  const int64_t blocks = (int64_t)nslices << wb;
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int mnb = jd.mb + jd.nb;
  const int64_t s0 = d_s0 ? *d_s0 : 0;
  const float* __restrict__ A = (const float*)jd.a.ptr;
  const float* __restrict__ B = (const float*)jd.b.ptr;
  const float* __restrict__ Blo = (const float*)jd.b.ptr_lo;
  float* __restrict__ C = (float*)jd.c_ptr;
  for (int64_t blk = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; blk < blocks; blk += nwarps) {
    const int b = (int)(blk >> wb);
    const int64_t s = s0 + b;
    const uint64_t q0 = ((uint64_t)blk & ((1ull << wb) - 1)) << (5 + LOGU);  // first quad of the block
    const int64_t abase = slice_offset(jd.a, b, s);
    float4 x[U][KK];
#pragma unroll
    for (int i = 0; i < U; ++i) {
      const uint64_t m0 = (q0 + (uint64_t)(lane + 32 * i)) << 2;
      const int64_t ao = abase + dep(jd.a.r_outer, m0);
#pragma unroll
      for (int v = 0; v < KK; ++v)
        x[i][v] = *reinterpret_cast<const float4*>(A + ao + (KFAST ? 4 * v : jd.a.ktab[v]));
    }
    const int sa = op_shift(jd.a, b), sb = op_shift(jd.b, b);
    const float fa = pow2f(sa), fb = pow2f(sb);
    const int64_t bbase = slice_offset(jd.b, b, s);
    float bv[KK][NN], bl[KK][NN];
#pragma unroll
    for (int n = 0; n < NN; ++n) {
      const int64_t o = bbase + dep(jd.b.r_outer, (uint64_t)n);
#pragma unroll
      for (int k = 0; k < KK; ++k) {
        bv[k][n] = B[o + jd.b.ktab[k]] * fb;
        bl[k][n] = Blo ? Blo[o + jd.b.ktab[k]] * fb : 0.f;
      }
    }
    uint32_t bits = 0;
#pragma unroll
    for (int i = 0; i < U; ++i) {
      float av[4][KK];
      if constexpr (KFAST) {
        // one run of 4*KK values: element r of the run is m = r / KK, k = r % KK
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int k = 0; k < KK; ++k) av[q][k] = f4_at(x[i][(q * KK + k) >> 2], (q * KK + k) & 3) * fa;
      } else {
#pragma unroll
        for (int k = 0; k < KK; ++k) {
          av[0][k] = x[i][k].x * fa; av[1][k] = x[i][k].y * fa; av[2][k] = x[i][k].z * fa; av[3][k] = x[i][k].w * fa;
        }
      }
      float out[4 * NN];
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int n = 0; n < NN; ++n) {
          float f = 0.f;
          if (Blo) {
#pragma unroll
            for (int k = 0; k < KK; ++k) f = fmaf(av[q][k], bl[k][n], f);
          }
#pragma unroll
          for (int k = 0; k < KK; ++k) f = fmaf(av[q][k], bv[k][n], f);
          out[q * NN + n] = f;
          bits = max(bits, __float_as_uint(f));
        }
      const uint64_t m0 = (q0 + (uint64_t)(lane + 32 * i)) << 2;
      float* c = C + ((int64_t)b << mnb) + (int64_t)m0 * NN;
#pragma unroll
      for (int v = 0; v < NN; ++v)
        reinterpret_cast<float4*>(c)[v] = make_float4(out[4 * v], out[4 * v + 1], out[4 * v + 2], out[4 * v + 3]);
    }
    // The whole warp is in slice b: one maximum per block.
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, off));
    if (lane == 0) {
      atomicMax(&jd.c_max[b], bits);
      if (q0 == 0) jd.c_exp[b] = op_exp(jd.a, b) + op_exp(jd.b, b) - sa - sb;
    }
  }
}

// ---------------------------------------------------------------------------
// Fused slice-invariant joins (OnceList).  Operands written earlier in the
// same launch by other CTAs are read through L2 (ld.global.cg): L1 is not
// coherent, and the arena of a fused list is never reused, so no stale line
// can be hit.  The arithmetic of every output is dot_k's (the KK > 0 order for
// K <= 16, the compensated 16-term chunks above), so the results equal the
// unfused launches bit for bit.

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Operand values of one output for K <= KMAX (split form: already scaled),
// every load issued before any is used.
template <int MODE, class T, int KMAX>
__device__ __forceinline__ void once_load(const OnceJoin& oj, int64_t oa, int64_t ob, int K, float fa, float fb,
                                          T* av, T* bv, float* al, float* bl) {
#pragma unroll
  for (int k = 0; k < KMAX; ++k) {
    if (k < K) {
      const T x = __ldcg((const T*)oj.a + oa + oj.a_ktab[k]);
      const T y = __ldcg((const T*)oj.b + ob + oj.b_ktab[k]);
      if (MODE == 1) {
        av[k] = (T)((float)x * fa);
        bv[k] = (T)((float)y * fb);
        al[k] = oj.a_lo ? __ldcg(oj.a_lo + oa + oj.a_ktab[k]) * fa : 0.f;
        bl[k] = oj.b_lo ? __ldcg(oj.b_lo + ob + oj.b_ktab[k]) * fb : 0.f;
      } else {
        av[k] = x;
        bv[k] = y;
      }
    }
  }
}

// dot_k's KK > 0 order on loaded values: A residual terms, B residual terms,
// then the main terms.
template <int MODE, class T, int KMAX>
__device__ __forceinline__ T once_dot(const OnceJoin& oj, int K, const T* av, const T* bv, const float* al,
                                      const float* bl) {
  if (MODE == 1) {
    float f = 0.f;
    if (oj.a_lo) {
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) f = fmaf(al[k], (float)bv[k], f);
    }
    if (oj.b_lo) {
#pragma unroll
      for (int k = 0; k < KMAX; ++k)
        if (k < K) f = fmaf((float)av[k], bl[k], f);
    }
#pragma unroll
    for (int k = 0; k < KMAX; ++k)
      if (k < K) f = fmaf((float)av[k], (float)bv[k], f);
    return (T)f;
  } else {
    T acc = 0;
#pragma unroll
    for (int k = 0; k < KMAX; ++k)
      if (k < K) acc = madm<MODE, T>(av[k], bv[k], acc, oj.mod_p, oj.mod_m);
    return acc;
  }
}

// 8 < K <= 16: the KK > 0 order with the loads inside each pass.
template <int MODE, class T>
__device__ T once_dot_serial(const OnceJoin& oj, int64_t oa, int64_t ob, int K, float fa, float fb) {
  const T* A = (const T*)oj.a;
  const T* B = (const T*)oj.b;
  if (MODE == 1) {
    float f = 0.f;
    if (oj.a_lo)
      for (int k = 0; k < K; ++k)
        f = fmaf(__ldcg(oj.a_lo + oa + oj.a_ktab[k]) * fa, (float)__ldcg(B + ob + oj.b_ktab[k]) * fb, f);
    if (oj.b_lo)
      for (int k = 0; k < K; ++k)
        f = fmaf((float)__ldcg(A + oa + oj.a_ktab[k]) * fa, __ldcg(oj.b_lo + ob + oj.b_ktab[k]) * fb, f);
    for (int k = 0; k < K; ++k)
      f = fmaf((float)__ldcg(A + oa + oj.a_ktab[k]) * fa, (float)__ldcg(B + ob + oj.b_ktab[k]) * fb, f);
    return (T)f;
  } else {
    T acc = 0;
    for (int k = 0; k < K; ++k)
      acc = madm<MODE, T>(__ldcg(A + oa + oj.a_ktab[k]), __ldcg(B + ob + oj.b_ktab[k]), acc, oj.mod_p, oj.mod_m);
    return acc;
  }
}

// K > 16: dot_k's compensated 16-term chunks (split form), k offsets from the runs.
template <int MODE, class T>
__device__ T once_dot_long(const OnceJoin& oj, int64_t oa, int64_t ob, int K, float fa, float fb) {
  const T* A = (const T*)oj.a;
  const T* B = (const T*)oj.b;
  if (MODE == 1) {
    float sum = 0.f, comp = 0.f;
    for (int k0 = 0; k0 < K; k0 += 16) {
      float f = 0.f;
      for (int k = k0; k < k0 + 16 && k < K; ++k) {
        const int64_t ka = dep(oj.a_k, (uint64_t)k), kb = dep(oj.b_k, (uint64_t)k);
        const float av = (float)__ldcg(A + oa + ka) * fa, bv = (float)__ldcg(B + ob + kb) * fb;
        if (oj.a_lo) f = fmaf(__ldcg(oj.a_lo + oa + ka) * fa, bv, f);
        if (oj.b_lo) f = fmaf(av, __ldcg(oj.b_lo + ob + kb) * fb, f);
        f = fmaf(av, bv, f);
      }
      const float t = sum + f;
      comp += fabsf(sum) >= fabsf(f) ? (sum - t) + f : (f - t) + sum;
      sum = t;
    }
    return (T)(sum + comp);
  } else {
    T acc = 0;
    for (int k = 0; k < K; ++k)
      acc = madm<MODE, T>(__ldcg(A + oa + dep(oj.a_k, (uint64_t)k)), __ldcg(B + ob + dep(oj.b_k, (uint64_t)k)), acc,
                          oj.mod_p, oj.mod_m);
    return acc;
  }
}

template <int MODE, class T>
__global__ void __launch_bounds__(kThreads, 3) k_once_list(const __grid_constant__ OnceList ol) {
  __shared__ __align__(16) OnceJoin sj;
  __shared__ int s_tile, s_join, s_bad;
  __shared__ uint32_t s_bits[kThreads / 32];
  volatile int32_t* err = ol.err;
  int cur = -1;  // join whose descriptor is in shared memory (block-uniform)
  int pre = -1;  // thread 0: the next tile, claimed while the current one is computed
  for (;;) {
    if (threadIdx.x == 0) {
      const int t = pre >= 0 ? pre : (int)atomicAdd(ol.counters, 1u);
      pre = -1;
      int j = -1, bad = 0;
      if (t < ol.total_tiles) {
        j = ol.tile_join[t];
        const int da = ol.deps[2 * j], db = ol.deps[2 * j + 1];
        const uint32_t na = da >= 0 ? (uint32_t)(ol.tile_first[da + 1] - ol.tile_first[da]) : 0u;
        const uint32_t nb = db >= 0 ? (uint32_t)(ol.tile_first[db + 1] - ol.tile_first[db]) : 0u;
        const long long t0 = clock64();
        for (;;) {
          const uint32_t ga = da >= 0 ? ld_acquire_u32(ol.counters + 1 + da) : 0u;
          const uint32_t gb = db >= 0 ? ld_acquire_u32(ol.counters + 1 + db) : 0u;
          if (ga >= na && gb >= nb) break;
          if (*err || clock64() - t0 > ol.wait_cycles) {
            bad = 1;
            break;
          }
        }
        if (bad) atomicExch((int*)ol.err, 1);
        __threadfence();
      }
      s_tile = t;
      s_join = j;
      s_bad = bad;
    }
    __syncthreads();
    const int j = s_join;
    if (j < 0 || s_bad) return;  // block-uniform
    // Claiming ahead keeps the order argument: the claimed tile is started as
    // soon as this one is published.
    if (threadIdx.x == 0) pre = (int)atomicAdd(ol.counters, 1u);
    const int tile = s_tile - ol.tile_first[j];
    if (j != cur) {
      const uint32_t* src = reinterpret_cast<const uint32_t*>(ol.joins + j);
      uint32_t* dst = reinterpret_cast<uint32_t*>(&sj);
      for (int i = threadIdx.x; i < (int)(sizeof(OnceJoin) / 4); i += kThreads) dst[i] = src[i];
      __syncthreads();
      cur = j;
    }
    const int mnb = sj.mb + sj.nb;
    const int64_t outs = 1ll << mnb;
    const int64_t q0 = (int64_t)tile * kOnceTile + 4 * threadIdx.x;
    uint32_t bits = 0;
    if (q0 < outs) {
      const uint64_t nmask = (1ull << sj.nb) - 1;
      int sa = 0, sb = 0;
      float fa = 1.f, fb = 1.f;
      if (MODE == 1) {
        sa = sj.a_max ? shift_from_max(__ldcg(sj.a_max)) : sj.a_shift;
        sb = sj.b_max ? shift_from_max(__ldcg(sj.b_max)) : sj.b_shift;
        fa = pow2f(sa);
        fb = pow2f(sb);
      }
      const int K = 1 << sj.kb;
      const int cnt = outs - q0 < 4 ? (int)(outs - q0) : 4;
      // Operand offsets of output q0 + v (q0 itself past the end of the join).
      auto offsets = [&](int v, int64_t& oa, int64_t& ob) {
        const uint64_t q = (uint64_t)(q0 + (v < cnt ? v : 0));
        const uint64_t m = sj.natural ? (q >> sj.nb) : (uint64_t)dep(sj.inv_m, q);
        const uint64_t n = sj.natural ? (q & nmask) : (uint64_t)dep(sj.inv_n, q);
        oa = dep(sj.a_outer, m);
        ob = dep(sj.b_outer, n);
      };
      T out[4];
      if (K <= 4) {  // independent outputs: the compiler overlaps their loads
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          int64_t oa, ob;
          offsets(v, oa, ob);
          T av[4], bv[4];
          float al[4], bl[4];
          once_load<MODE, T, 4>(sj, oa, ob, K, fa, fb, av, bv, al, bl);
          out[v] = once_dot<MODE, T, 4>(sj, K, av, bv, al, bl);
        }
      } else if (K <= 8) {
#pragma unroll 1
        for (int v = 0; v < 4; ++v) {
          int64_t oa, ob;
          offsets(v, oa, ob);
          T av[8], bv[8];
          float al[8], bl[8];
          once_load<MODE, T, 8>(sj, oa, ob, K, fa, fb, av, bv, al, bl);
          out[v] = once_dot<MODE, T, 8>(sj, K, av, bv, al, bl);
        }
      } else if (K <= 16) {
#pragma unroll 1
        for (int v = 0; v < 4; ++v) {
          int64_t oa, ob;
          offsets(v, oa, ob);
          out[v] = once_dot_serial<MODE, T>(sj, oa, ob, K, fa, fb);
        }
      } else {
#pragma unroll 1
        for (int v = 0; v < 4; ++v) {
          int64_t oa, ob;
          offsets(v, oa, ob);
          out[v] = once_dot_long<MODE, T>(sj, oa, ob, K, fa, fb);
        }
      }
      T* C = (T*)sj.c;
      if (cnt == 4) {
        store_vec(C + q0, out);
      } else {
        for (int v = 0; v < cnt; ++v) C[q0 + v] = out[v];
      }
      if (MODE == 1) {
        for (int v = 0; v < cnt; ++v) bits = max(bits, __float_as_uint((float)out[v]));
        if (q0 == 0) {
          const int ea = sj.a_exp ? __ldcg(sj.a_exp) : 0, eb = sj.b_exp ? __ldcg(sj.b_exp) : 0;
          *sj.c_exp = ea + eb - sa - sb;
        }
      }
    }
    if (MODE == 1) {
      for (int off = 16; off > 0; off >>= 1) bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, off));
      if ((threadIdx.x & 31) == 0) s_bits[threadIdx.x >> 5] = bits;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      if (MODE == 1) {
        uint32_t v = 0;
        for (int w = 0; w < kThreads / 32; ++w) v = max(v, s_bits[w]);
        if (v) atomicMax(sj.c_max, v);
      }
      __threadfence();
      atomicAdd(ol.counters + 1 + j, 1u);
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
__device__ __forceinline__ void load4(const u64* p, u64* v) {
  const ulonglong2 x = reinterpret_cast<const ulonglong2*>(p)[0], y = reinterpret_cast<const ulonglong2*>(p)[1];
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
  // Split form: each 16-wide K chunk accumulates into fresh FP32 partials,
  // which are added into a compensated (Neumaier) running sum, so the error
  // does not grow with K.
  T acc[4][4], comp[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = comp[i][j] = 0;

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
    if constexpr (MODE != 1) {
#pragma unroll
      for (int kk = 0; kk < BK; ++kk) {
        T av[4], bv[4];
        load4(&As[kk][ty * 4], av);
        load4(&Bs[kk][tx * 4], bv);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = mad(av[i], bv[j], acc[i][j]);
      }
      if constexpr (MODE == 3) {
        // Residues below p < 2^28: a chunk adds BK = 16 products below 2^56
        // to a residue, less than 2^61, so one reduction per chunk suffices.
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = mod_reduce(acc[i][j], jd.mod_p, jd.mod_m);
      }
    } else {
      T part[4][4];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) part[i][j] = 0;
#pragma unroll
      for (int kk = 0; kk < BK; ++kk) {
        T av[4], bv[4];
        load4(&As[kk][ty * 4], av);
        load4(&Bs[kk][tx * 4], bv);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) part[i][j] = fma(av[i], bv[j], part[i][j]);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const T t = acc[i][j] + part[i][j];
          comp[i][j] += fabs(acc[i][j]) >= fabs(part[i][j]) ? (acc[i][j] - t) + part[i][j] : (part[i][j] - t) + acc[i][j];
          acc[i][j] = t;
        }
    }
    __syncthreads();
  }
  if (MODE == 1) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] += comp[i][j];
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
  if constexpr (MODE >= 2) {  // int forms: an exact sum in the form's arithmetic
    u64 sum = 0;
    constexpr int U = 4;
    for (int64_t j0 = 0; j0 < steps; j0 += U) {
      u64 y[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        y[u] = (j0 + u < steps) ? madm<MODE, T>(A[ka], B[kb], 0ull, jd.mod_p, jd.mod_m) : 0ull;
        const int t8 = __ffsll(~(unsigned long long)(j0 + u)) - 1 + LOGT;
        if (t8 < TOGB_MAXBITS) { ka += jd.a.dk[t8] + pa8; kb += jd.b.dk[t8] + pb8; }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) sum = addm<MODE>(sum, y[u], jd.mod_p);
    }
    const u64 total = block_sum<MODE>(sum, jd.mod_p);
    if (tid == 0) ((T*)jd.c_ptr)[(int64_t)b * jd.c_batch_stride + dep(jd.r_cm, m) + dep(jd.r_cn, n)] = total;
    return;
  }
  int sa = 0, sb = 0;
  double hi = 0.0, lo = 0.0;
  if constexpr (MODE == 1) {
    sa = op_shift(jd.a, b);
    sb = op_shift(jd.b, b);
    const float fa = pow2f(sa), fb = pow2f(sb);
    const float* alo = jd.a.ptr_lo ? (const float*)jd.a.ptr_lo + oa : nullptr;
    const float* blo = jd.b.ptr_lo ? (const float*)jd.b.ptr_lo + ob : nullptr;
    float sum = 0.f, c = 0.f;
    constexpr int U = 4;
    for (int64_t j0 = 0; j0 < steps; j0 += U) {
      int64_t oa_[U], ob_[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        oa_[u] = ka;
        ob_[u] = kb;
        const int t8 = __ffsll(~(unsigned long long)(j0 + u)) - 1 + LOGT;
        if (t8 < TOGB_MAXBITS) { ka += jd.a.dk[t8] + pa8; kb += jd.b.dk[t8] + pb8; }
      }
      float y[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        y[u] = 0.f;
        if (j0 + u < steps) {
          const float av = (float)A[oa_[u]] * fa, bv = (float)B[ob_[u]] * fb;
          y[u] = av * bv;
          if (alo) y[u] = fmaf(alo[oa_[u]] * fa, bv, y[u]);
          if (blo) y[u] = fmaf(av, blo[ob_[u]] * fb, y[u]);
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const float yy = y[u] - c;
        const float t = sum + yy;
        c = (t - sum) - yy;
        sum = t;
      }
    }
    hi = (double)sum;
    lo = -(double)c;
  } else {
    double sum = 0.0;
    constexpr int U = 4;
    for (int64_t j0 = 0; j0 < steps; j0 += U) {
      double y[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        y[u] = (j0 + u < steps) ? (double)A[ka] * (double)B[kb] : 0.0;
        const int t8 = __ffsll(~(unsigned long long)(j0 + u)) - 1 + LOGT;
        if (t8 < TOGB_MAXBITS) { ka += jd.a.dk[t8] + pa8; kb += jd.b.dk[t8] + pb8; }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) sum += y[u];
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

// k_reduce for operands whose K axis is contiguous (unit stride, offsets
// aligned to 16 bytes, no leaf residual): each thread reads 16-byte vectors of
// both operands, four vectors deep, and adds 16-term partials into a
// compensated sum; a pairwise tree across the CTA finishes the entry.
template <int MODE, class T>
__global__ void __launch_bounds__(kThreads) k_reduce_vec(const __grid_constant__ JoinDesc jd,
                                                         const int64_t* __restrict__ d_s0, int nslices) {
  constexpr int VW = 16 / sizeof(T);  // elements per vector
  using V = typename Vec16<T>::type;
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
  const V* __restrict__ A = reinterpret_cast<const V*>((const T*)jd.a.ptr + slice_offset(jd.a, b, s) + dep(jd.a.r_outer, m));
  const V* __restrict__ B = reinterpret_cast<const V*>((const T*)jd.b.ptr + slice_offset(jd.b, b, s) + dep(jd.b.r_outer, n));
  const int64_t nv = (1ll << jd.kb) / VW;
  int sa = 0, sb = 0;
  T fa = 1, fb = 1;
  if (MODE == 1) {
    sa = op_shift(jd.a, b);
    sb = op_shift(jd.b, b);
    fa = (T)pow2f(sa);
    fb = (T)pow2f(sb);
  }
  T sum = 0, comp = 0;
  constexpr int U = 4;
  for (int64_t v0 = tid; v0 < nv; v0 += (int64_t)U * kThreads) {
    V av[U], bv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t v = v0 + (int64_t)u * kThreads;
      if (v < nv) {
        av[u] = A[v];
        bv[u] = B[v];
      } else {
        memset(&av[u], 0, sizeof(V));
        memset(&bv[u], 0, sizeof(V));
      }
    }
    T part = 0;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const T* x = reinterpret_cast<const T*>(&av[u]);
      const T* y = reinterpret_cast<const T*>(&bv[u]);
#pragma unroll
      for (int q = 0; q < VW; ++q) part = madm<MODE, T>(x[q] * fa, y[q] * fb, part, jd.mod_p, jd.mod_m);
    }
    if constexpr (MODE >= 2) {
      sum = addm<MODE>(sum, part, jd.mod_p);
    } else {
      const T t = sum + part;
      comp += fabs(sum) >= fabs(part) ? (sum - t) + part : (part - t) + sum;
      sum = t;
    }
  }
  if constexpr (MODE >= 2) {  // int forms: an exact sum over the CTA
    const u64 total = block_sum<MODE>(sum, jd.mod_p);
    if (tid == 0) ((T*)jd.c_ptr)[(int64_t)b * jd.c_batch_stride + dep(jd.r_cm, m) + dep(jd.r_cn, n)] = total;
    return;
  }
  double hi = (double)sum, lo = (double)comp;
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
// order, into the FP64 accumulator (the int form adds wrapping words).
template <int MODE, class T>
__global__ void k_root(const __grid_constant__ RootDesc rd, const int64_t* __restrict__ d_s0, int nslices) {
  const int64_t E = 1ll << rd.r.outer_bits;
  const int64_t s0 = d_s0 ? *d_s0 : 0;
  const T* __restrict__ R = (const T*)rd.r.ptr;
  if constexpr (MODE >= 2) {  // int forms: the accumulator's sums are words of the form
    u64* acc = reinterpret_cast<u64*>(rd.acc_sum);
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
      u64 sum = acc[e];
      const int64_t oe = dep(rd.r.r_outer, (uint64_t)e);
      for (int b = 0; b < nslices; ++b) sum = addm<MODE>(sum, R[slice_offset(rd.r, b, s0 + b) + oe], rd.mod_p);
      acc[e] = sum;
    }
  } else {
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
}

// Exact sum of two doubles as a rounded sum plus its rounding error (Neumaier's
// branch of Knuth's two-sum).
__device__ __forceinline__ double two_sum_err(double a, double b, double t) {
  return fabs(a) >= fabs(b) ? (a - t) + b : (b - t) + a;
}

// The root reduction for roots of few entries (a count has one): one CTA per
// root entry.  Thread i takes slices i, i + 256, ... in slice order into a
// compensated sum; the 256 (sum, compensation) pairs are then combined by a
// fixed pairwise tree of two-sums and the chunk's total is added into the
// accumulator.  The combination order depends only on the slice count, so
// every run gives the same bits; the error stays a few units in the last
// place of the total (compensated at every level).
template <int MODE, class T>
__global__ void __launch_bounds__(kThreads) k_root_tree(const __grid_constant__ RootDesc rd,
                                                        const int64_t* __restrict__ d_s0, int nslices) {
  __shared__ double ss[kThreads], sc[kThreads];
  const int64_t e = blockIdx.x;
  const int64_t s0 = d_s0 ? *d_s0 : 0;
  const T* __restrict__ R = (const T*)rd.r.ptr;
  const int64_t oe = dep(rd.r.r_outer, (uint64_t)e);
  if constexpr (MODE >= 2) {  // int forms: an exact sum, added into the accumulator's word
    u64 isum = 0;
    for (int b = threadIdx.x; b < nslices; b += kThreads)
      isum = addm<MODE>(isum, R[slice_offset(rd.r, b, s0 + b) + oe], rd.mod_p);
    const u64 total = block_sum<MODE>(isum, rd.mod_p);
    if (threadIdx.x == 0) {
      u64* acc = reinterpret_cast<u64*>(rd.acc_sum) + e;
      *acc = addm<MODE>(*acc, total, rd.mod_p);
    }
    return;
  }
  double sum = 0.0, comp = 0.0;
  for (int b = threadIdx.x; b < nslices; b += kThreads) {
    const int64_t o = slice_offset(rd.r, b, s0 + b) + oe;
    double x = (double)R[o];
    if (MODE == 1) {
      if (rd.r.ptr_lo) x += (double)((const float*)rd.r.ptr_lo)[o];
      x = ldexp(x, op_exp(rd.r, b));
    }
    const double t = sum + x;
    comp += two_sum_err(sum, x, t);
    sum = t;
  }
  ss[threadIdx.x] = sum;
  sc[threadIdx.x] = comp;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      const double a = ss[threadIdx.x], b = ss[threadIdx.x + w];
      const double t = a + b;
      sc[threadIdx.x] += sc[threadIdx.x + w] + two_sum_err(a, b, t);
      ss[threadIdx.x] = t;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double a = rd.acc_sum[e], b = ss[0];
    const double t = a + b;
    rd.acc_comp[e] += sc[0] + two_sum_err(a, b, t);
    rd.acc_sum[e] = t;
  }
}

// The fused root: the count's slice values from the partials its operand's
// tensor-core epilogue wrote.  A warp per slice adds the slice's partials
// (lane-strided, then a fixed shuffle tree), applies the slice's exponents
// and writes the value over the slice's first partial.  The last CTA to
// finish (a device counter, no waiting) adds the slice values with
// k_root_tree's compensated tree, adds the total into the accumulator and
// resets the counter.  Every order is fixed: the same bits every run.
__global__ void __launch_bounds__(kThreads) k_root_parts(const __grid_constant__ RootDesc rd, int nslices) {
  __shared__ double ss[kThreads], sc[kThreads];
  __shared__ int last;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.x * (kThreads / 32) + warp;
  if (b < nslices) {
    double* P = rd.part + (int64_t)b * rd.part_stride;
    double t = 0.0;
    for (int i = lane; i < rd.npart; i += 32) t += P[i];
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    if (lane == 0) P[0] = ldexp(t, rd.px_exp[b] + rd.py_exp[(int64_t)b * rd.py_step]);
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(rd.done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  double sum = 0.0, comp = 0.0;
  for (int s = threadIdx.x; s < nslices; s += kThreads) {
    const double x = __ldcg(rd.part + (int64_t)s * rd.part_stride);
    const double t = sum + x;
    comp += two_sum_err(sum, x, t);
    sum = t;
  }
  ss[threadIdx.x] = sum;
  sc[threadIdx.x] = comp;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      const double a = ss[threadIdx.x], c = ss[threadIdx.x + w];
      const double t = a + c;
      sc[threadIdx.x] += sc[threadIdx.x + w] + two_sum_err(a, c, t);
      ss[threadIdx.x] = t;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double a = rd.acc_sum[0], c = ss[0];
    const double t = a + c;
    rd.acc_comp[0] += sc[0] + two_sum_err(a, c, t);
    rd.acc_sum[0] = t;
    *rd.done = 0;
  }
}

__global__ void k_set_s0(int64_t* p, int64_t v) { *p = v; }

// One CTA per leaf: the values of OrTensor / VariableTensor leaves from their
// parameters (index bit R-1-a is axis a, row-major like the host layout).
__global__ void k_build_leaves(const LeafBuild* __restrict__ items, double* __restrict__ v64,
                               float* __restrict__ v32, float* __restrict__ v32lo) {
  const LeafBuild it = items[blockIdx.x];
  const uint64_t n = 1ull << it.rank;
  const uint64_t all = n - 1;
  for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) {
    double v;
    if (it.kind == TOGB_LEAF_VARIABLE) {
      v = it.rank == 0 ? it.w_neg + it.w_pos : (i == 0 ? it.w_neg : (i == all ? it.w_pos : 0.0));
    } else {
      const uint64_t F = it.false_idx;
      if (it.out_pos < 0) {
        v = i == F ? 0.0 : 1.0;
      } else {
        const uint64_t bo = 1ull << it.out_pos;
        if (i == F) v = 1.0;
        else if (i == (F ^ bo)) v = 0.0;
        else v = ((i ^ F) & bo) ? 1.0 : 0.0;  // the output axis at its false value gives 0
      }
    }
    const float hi = (float)v;
    v64[it.off + i] = v;
    v32[it.off + i] = hi;
    v32lo[it.off + i] = (float)(v - (double)hi);
  }
}

// The int form's leaves: each FP64 leaf value converted toward zero, the
// conversion numpy applies when a float is stored into an int64 tensor.
__global__ void k_leaf_int(const double* __restrict__ v64, u64* __restrict__ out, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (u64)__double2ll_rz(v64[i]);
}

// The residue form's leaves: the same integer value modulo p, in [0, p).
__global__ void k_leaf_mod(const double* __restrict__ v64, u64* __restrict__ out, int64_t n, long long p) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const long long r = __double2ll_rz(v64[i]) % p;
    out[i] = (u64)(r < 0 ? r + p : r);
  }
}

__global__ void k_finalize(const double* __restrict__ acc, int64_t E, double* __restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = acc[e] + acc[E + e];
}

template <class T>
__global__ void __launch_bounds__(kThreads) k_probe(T* out, int iters, T seed) {
  // Operands come from a runtime value so no constant-bank operand is involved.
  const T m = seed * (T)0.999999, c = seed * (T)1e-7;
  T a[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) a[i] = seed + (T)(threadIdx.x + i);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int j = 0; j < 16; ++j) a[j] = fma(a[j], m, c);
  }
  T r = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) r += a[i];
  if (r == (T)-1) out[0] = r;
}

// FP64 tensor-core probe: independent mma.sync m8n8k4 FP64 accumulations.
__global__ void __launch_bounds__(kThreads) k_probe_dmma(double* out, int iters) {
  double a = 1.0 + threadIdx.x * 1e-6, b = 0.5;
  double c[8][2];
#pragma unroll
  for (int i = 0; i < 8; ++i) { c[i][0] = 0.0; c[i][1] = 0.0; }
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                   : "+d"(c[i][0]), "+d"(c[i][1])
                   : "d"(a), "d"(b));
  }
  double r = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) r += c[i][0] + c[i][1];
  if (r == -1.0) out[0] = r;
}

// An operand k_reduce_vec can read: unit-stride K, no leaf residual, and every
// possible base offset (slice, outer index) and the pointer 16-byte aligned.
bool reduce_vec_ok(const OpDesc& o, int mode) {
  const int64_t vw = mode == 1 ? 4 : 2;
  if (o.ptr_lo) return false;
  if (o.r_k.n != 1 || o.r_k.src[0] != 0 || o.r_k.dst[0] != 0) return false;
  if (((uintptr_t)o.ptr & 15) != 0 || o.batch_stride % vw != 0) return false;
  for (int j = 0; j < o.n_slice_terms; ++j)
    if (o.slice_stride[j] % vw != 0) return false;
  for (int i = 0; i < o.outer_bits; ++i)
    if (o.s_outer[i] % vw != 0) return false;
  return true;
}

int grid_for(int64_t work) {
  const int64_t blocks = (work + kThreads - 1) / kThreads;
  const int64_t cap = 152 * 32;
  return (int)(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
}

// One resident wave of the staged kernel (contiguous tile ranges need every
// CTA resident at once to stay balanced), at most one CTA per tile.
template <class Kern>
void staged_launch(Kern kern, const JoinDesc& jd, const StageInfo& si, const int64_t* s0, int nslices,
                   int64_t tiles, size_t bytes, cudaStream_t st) {
  const int sms = sm_count();
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, bytes) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const int64_t wave = (int64_t)sms * per_sm;
  const int grid = (int)(tiles < wave ? tiles : wave);
  kern<<<grid, kThreads, bytes, st>>>(jd, si, s0, nslices);
}

// The staged thread-per-output variant applies to K <= 16 when a tile of 2^T
// (T in [10, 14]) output addresses touches at least 4 rows of each operand
// (rows are reused) and the staged rows fit 64 KB.  Returns true when launched.
// Tiles of 2^T output addresses, T in [10, 14]: the largest T whose launch
// still has a tile for every resident CTA (about 152 x 8), else the smallest.
bool staged_plan(int mode, const JoinDesc& jd, int nslices, StageInfo& si, size_t& bytes) {
  const int mnb = jd.mb + jd.nb;
  if (jd.kb > 4 || mnb < 10) return false;
  const int K = 1 << jd.kb;
  const size_t es = mode == 1 ? 4 : 8;
  bool found = false;
  StageInfo best{};
  size_t best_bytes = 0;
  for (int T = mnb < 14 ? mnb : 14; T >= 10; --T) {
    StageInfo c{};
    int lm = 0, ln = 0;
    for (int i = 0; i < jd.mb; ++i)
      if (jd.c_s_m[i] < (1ll << T)) c.a_row_bits[lm++] = i;
    for (int i = 0; i < jd.nb; ++i)
      if (jd.c_s_n[i] < (1ll << T)) c.b_row_bits[ln++] = i;
    if (lm + ln != T || lm < 2 || ln < 2) continue;
    size_t b = ((size_t)1 << lm) * K * es + ((size_t)1 << ln) * K * es;
    if (mode == 1) b += (jd.a.ptr_lo ? ((size_t)1 << lm) * K * 4 : 0) + (jd.b.ptr_lo ? ((size_t)1 << ln) * K * 4 : 0);
    b += 4 * (((size_t)1 << lm) + ((size_t)1 << ln));  // row offsets
    if (b > 64 * 1024) continue;
    c.T = T;
    c.lm = lm;
    c.ln = ln;
    c.a_inv = jd.a.batch_stride == 0 && jd.a.n_slice_terms == 0;
    c.b_inv = jd.b.batch_stride == 0 && jd.b.n_slice_terms == 0;
    best = c;
    best_bytes = b;
    found = true;
    if (((int64_t)nslices << (mnb - T)) >= 152 * 8) break;  // largest T with enough tiles
  }
  if (found) {
    si = best;
    bytes = best_bytes;
  }
  return found;
}

bool launch_staged(int mode, const JoinDesc& jd, const int64_t* s0, int nslices, cudaStream_t st) {
  StageInfo si;
  size_t bytes = 0;
  if (!staged_plan(mode, jd, nslices, si, bytes)) return false;
  si.slice_fast = nslices > 1 && (si.a_inv || si.b_inv);
  const int64_t tiles = (int64_t)nslices << (jd.mb + jd.nb - si.T);
#define TOGB_STAGED(KK)                                                                                    \
  {                                                                                                        \
    if (mode == 0) staged_launch(k_direct_staged<0, double, KK>, jd, si, s0, nslices, tiles, bytes, st);   \
    else if (mode == 2) staged_launch(k_direct_staged<2, u64, KK>, jd, si, s0, nslices, tiles, bytes, st); \
    else if (mode == 3) staged_launch(k_direct_staged<3, u64, KK>, jd, si, s0, nslices, tiles, bytes, st); \
    else staged_launch(k_direct_staged<1, float, KK>, jd, si, s0, nslices, tiles, bytes, st);              \
  }
  switch (jd.kb) {
    case 0: TOGB_STAGED(1) break;
    case 1: TOGB_STAGED(2) break;
    case 2: TOGB_STAGED(4) break;
    case 3: TOGB_STAGED(8) break;
    default: TOGB_STAGED(16) break;
  }
#undef TOGB_STAGED
  return true;
}

// Streaming variant (k_stream): split form, natural output, M >= 4, K <= 4,
// N * K <= 16, A without a leaf residual, and A's four consecutive m either
// one vector per k or one run with every k, every base offset 16-byte aligned.
// Returns true when launched.
bool stream_ok(int mode, const JoinDesc& jd, bool& kfast) {
  // K <= 4, or K = 8 against a single column (N = 1).
  if (mode != 1 || !jd.c_natural || jd.mb < 2 || jd.kb > 3 || (jd.kb == 3 && jd.nb > 0) || jd.a.ptr_lo)
    return false;
  const int K = 1 << jd.kb, N = 1 << jd.nb;
  if (N * K > 16) return false;
  const OpDesc& a = jd.a;
  if (a.s_outer[0] == 1 && a.s_outer[1] == 2) {
    kfast = false;
  } else if (jd.kb >= 1 && a.s_outer[0] == K && a.s_outer[1] == 2 * K) {
    for (int j = 0; j < jd.kb; ++j)
      if (a.s_k[j] != (1ll << j)) return false;
    kfast = true;
  } else {
    return false;
  }
  if (((uintptr_t)a.ptr & 15) || ((uintptr_t)jd.c_ptr & 15)) return false;
  if (a.batch_stride % 4) return false;
  for (int j = 0; j < a.n_slice_terms; ++j)
    if (a.slice_stride[j] % 4) return false;
  for (int i = 2; i < jd.mb; ++i)
    if (a.s_outer[i] % 4) return false;
  if (!kfast)
    for (int j = 0; j < jd.kb; ++j)
      if (a.s_k[j] % 4) return false;
  return true;
}

// k_stream_blk for one (KK, NN): U = 2^LOGU quads per lane, one warp per
// block of 32*U quads, at most 16 CTAs per SM walking the blocks.
template <int KK, int NN, int LOGU>
void launch_stream_blk(const JoinDesc& jd, bool kfast, const int64_t* s0, int nslices, cudaStream_t st) {
  const int64_t warps = (int64_t)nslices << (jd.mb - 7 - LOGU);
  const int64_t ctas = (warps + kThreads / 32 - 1) / (kThreads / 32);
  const int64_t cap = (int64_t)sm_count() * 16;
  const int g = (int)(ctas < cap ? ctas : cap);
  if (kfast) k_stream_blk<KK, NN, true, LOGU><<<g, kThreads, 0, st>>>(jd, s0, nslices);
  else k_stream_blk<KK, NN, false, LOGU><<<g, kThreads, 0, st>>>(jd, s0, nslices);
}

bool launch_stream(int mode, const JoinDesc& jd, const int64_t* s0, int nslices, cudaStream_t st) {
  bool kfast = false;
  if (!stream_ok(mode, jd, kfast)) return false;
  // Slices of at least one warp block (32 lanes x U quads): the block variant,
  // four quads per lane (two when K = 4 or N >= 8, which hold more values).
  const int logu = (jd.kb >= 2 || jd.nb >= 3) ? 1 : 2;
  if (jd.mb >= 7 + logu) {
    switch (jd.kb * 8 + jd.nb) {
      case 0: launch_stream_blk<1, 1, 2>(jd, false, s0, nslices, st); return true;
      case 1: launch_stream_blk<1, 2, 2>(jd, false, s0, nslices, st); return true;
      case 2: launch_stream_blk<1, 4, 2>(jd, false, s0, nslices, st); return true;
      case 3: launch_stream_blk<1, 8, 1>(jd, false, s0, nslices, st); return true;
      case 4: launch_stream_blk<1, 16, 1>(jd, false, s0, nslices, st); return true;
      case 8: launch_stream_blk<2, 1, 2>(jd, kfast, s0, nslices, st); return true;
      case 9: launch_stream_blk<2, 2, 2>(jd, kfast, s0, nslices, st); return true;
      case 10: launch_stream_blk<2, 4, 2>(jd, kfast, s0, nslices, st); return true;
      case 11: launch_stream_blk<2, 8, 1>(jd, kfast, s0, nslices, st); return true;
      case 16: launch_stream_blk<4, 1, 1>(jd, kfast, s0, nslices, st); return true;
      case 17: launch_stream_blk<4, 2, 1>(jd, kfast, s0, nslices, st); return true;
      case 18: launch_stream_blk<4, 4, 1>(jd, kfast, s0, nslices, st); return true;
      case 24: launch_stream_blk<8, 1, 1>(jd, kfast, s0, nslices, st); return true;
      default: break;
    }
  }
  const int64_t quads = (int64_t)nslices << (jd.mb - 2);
  const int g = grid_for(quads);
#define TOGB_STREAM(KK, NN)                                                                \
  {                                                                                        \
    if (kfast) k_stream<KK, NN, true><<<g, kThreads, 0, st>>>(jd, s0, nslices);            \
    else k_stream<KK, NN, false><<<g, kThreads, 0, st>>>(jd, s0, nslices);                 \
  }
  switch (jd.kb * 8 + jd.nb) {
    case 0: k_stream<1, 1, false><<<g, kThreads, 0, st>>>(jd, s0, nslices); break;
    case 1: k_stream<1, 2, false><<<g, kThreads, 0, st>>>(jd, s0, nslices); break;
    case 2: k_stream<1, 4, false><<<g, kThreads, 0, st>>>(jd, s0, nslices); break;
    case 3: k_stream<1, 8, false><<<g, kThreads, 0, st>>>(jd, s0, nslices); break;
    case 4: k_stream<1, 16, false><<<g, kThreads, 0, st>>>(jd, s0, nslices); break;
    case 8: TOGB_STREAM(2, 1) break;
    case 9: TOGB_STREAM(2, 2) break;
    case 10: TOGB_STREAM(2, 4) break;
    case 11: TOGB_STREAM(2, 8) break;
    case 16: TOGB_STREAM(4, 1) break;
    case 17: TOGB_STREAM(4, 2) break;
    case 18: TOGB_STREAM(4, 4) break;
    case 24: TOGB_STREAM(8, 1) break;
    default: return false;
  }
#undef TOGB_STREAM
  return true;
}

}  // namespace

int sm_count() {
  // Per device, filled on first use; concurrent first calls store the same value.
  static std::atomic<int> sms[kMaxDevices];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return 1;
  }
  int n = sms[dev].load(std::memory_order_relaxed);
  if (n <= 0) {
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
      cudaGetLastError();
      return 1;
    }
    sms[dev].store(n, std::memory_order_relaxed);
  }
  return n;
}

int direct_variant(int mode, const JoinDesc& jd) {
  bool kfast = false;
  if (stream_ok(mode, jd, kfast)) return kfast ? 3 : 2;
  StageInfo si;
  size_t bytes = 0;
  return staged_plan(mode, jd, 1 << 20, si, bytes) ? 1 : 0;
}

cudaError_t launch_join(int mode, int kernel, const JoinDesc& jd, const int64_t* s0, int nslices,
                        cudaStream_t st) {
  if (kernel == K_UMMA && mode == 1) return launch_umma(jd, nullptr, nullptr, s0, nslices, st);
  if (kernel == K_TILED || kernel == K_UMMA) {
    const int tm_bits = jd.mb > 6 ? jd.mb - 6 : 0;
    const int tn_bits = jd.nb > 6 ? jd.nb - 6 : 0;
    const uint64_t tiles = 1ull << (tm_bits + tn_bits);
    if (tiles > 0x7fffffffull) return cudaErrorInvalidValue;
    const int gy = nslices < 65535 ? nslices : 65535;
    const int gz = (nslices + gy - 1) / gy;
    dim3 grid((unsigned)tiles, gy, gz);
    if (mode == 0) k_tiled<0, double><<<grid, kThreads, 0, st>>>(jd, s0, nslices, tn_bits);
    else if (mode == 2) k_tiled<2, u64><<<grid, kThreads, 0, st>>>(jd, s0, nslices, tn_bits);
    else if (mode == 3) k_tiled<3, u64><<<grid, kThreads, 0, st>>>(jd, s0, nslices, tn_bits);
    else k_tiled<1, float><<<grid, kThreads, 0, st>>>(jd, s0, nslices, tn_bits);
  } else if (kernel == K_REDUCE) {
    const int64_t blocks = (int64_t)nslices << (jd.mb + jd.nb);
    const unsigned gx = (unsigned)(blocks < 65536 ? blocks : 65536);
    const unsigned gy = (unsigned)((blocks + gx - 1) / gx);
    if (gy > 65535) return cudaErrorInvalidValue;
    const bool vec = reduce_vec_ok(jd.a, mode) && reduce_vec_ok(jd.b, mode) && jd.kb >= 10;
    if (vec) {
      if (mode == 0) k_reduce_vec<0, double><<<dim3(gx, gy), kThreads, 0, st>>>(jd, s0, nslices);
      else if (mode == 2) k_reduce_vec<2, u64><<<dim3(gx, gy), kThreads, 0, st>>>(jd, s0, nslices);
      else if (mode == 3) k_reduce_vec<3, u64><<<dim3(gx, gy), kThreads, 0, st>>>(jd, s0, nslices);
      else k_reduce_vec<1, float><<<dim3(gx, gy), kThreads, 0, st>>>(jd, s0, nslices);
    } else {
      if (mode == 0) k_reduce<0, double><<<dim3(gx, gy), kThreads, 0, st>>>(jd, s0, nslices);
      else if (mode == 2) k_reduce<2, u64><<<dim3(gx, gy), kThreads, 0, st>>>(jd, s0, nslices);
      else if (mode == 3) k_reduce<3, u64><<<dim3(gx, gy), kThreads, 0, st>>>(jd, s0, nslices);
      else k_reduce<1, float><<<dim3(gx, gy), kThreads, 0, st>>>(jd, s0, nslices);
    }
  } else if (launch_stream(mode, jd, s0, nslices, st)) {
    // long operand against a tiny one: streaming variant launched
  } else if (launch_staged(mode, jd, s0, nslices, st)) {
    // short-K join with reused operand rows: staged variant launched
  } else {
    const int mnb = jd.mb + jd.nb;
    const int vec = mnb >= 2 ? 4 : 1;
    const int64_t groups = ((int64_t)nslices << mnb) / vec;
    const int g = grid_for(groups);
#define TOGB_DIRECT(KK)                                                                          \
    if (vec == 4) {                                                                              \
      if (mode == 0) k_direct<0, double, KK, 4><<<g, kThreads, 0, st>>>(jd, s0, nslices);       \
      else if (mode == 2) k_direct<2, u64, KK, 4><<<g, kThreads, 0, st>>>(jd, s0, nslices);     \
      else if (mode == 3) k_direct<3, u64, KK, 4><<<g, kThreads, 0, st>>>(jd, s0, nslices);     \
      else k_direct<1, float, KK, 4><<<g, kThreads, 0, st>>>(jd, s0, nslices);                  \
    } else {                                                                                     \
      if (mode == 0) k_direct<0, double, KK, 1><<<g, kThreads, 0, st>>>(jd, s0, nslices);       \
      else if (mode == 2) k_direct<2, u64, KK, 1><<<g, kThreads, 0, st>>>(jd, s0, nslices);     \
      else if (mode == 3) k_direct<3, u64, KK, 1><<<g, kThreads, 0, st>>>(jd, s0, nslices);     \
      else k_direct<1, float, KK, 1><<<g, kThreads, 0, st>>>(jd, s0, nslices);                  \
    }
    switch (jd.kb) {
      case 0: TOGB_DIRECT(1) break;
      case 1: TOGB_DIRECT(2) break;
      case 2: TOGB_DIRECT(4) break;
      case 3: TOGB_DIRECT(8) break;
      case 4: TOGB_DIRECT(16) break;
      default: TOGB_DIRECT(0) break;
    }
#undef TOGB_DIRECT
  }
  return cudaGetLastError();
}

cudaError_t launch_once_list(int mode, const OnceList& ol, cudaStream_t st) {
  if (ol.n <= 0 || ol.total_tiles <= 0) return cudaSuccess;
  const int sms = sm_count();
  int per_sm = 0;
  cudaError_t e = mode == 0   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_once_list<0, double>, kThreads, 0)
                  : mode == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_once_list<2, u64>, kThreads, 0)
                  : mode == 3 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_once_list<3, u64>, kThreads, 0)
                              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_once_list<1, float>, kThreads, 0);
  if (e != cudaSuccess || per_sm < 1) per_sm = 1;
  const int64_t wave = (int64_t)sms * per_sm;
  const int grid = (int)(ol.total_tiles < wave ? ol.total_tiles : wave);
  if (mode == 0) k_once_list<0, double><<<grid, kThreads, 0, st>>>(ol);
  else if (mode == 2) k_once_list<2, u64><<<grid, kThreads, 0, st>>>(ol);
  else if (mode == 3) k_once_list<3, u64><<<grid, kThreads, 0, st>>>(ol);
  else k_once_list<1, float><<<grid, kThreads, 0, st>>>(ol);
  return cudaGetLastError();
}

cudaError_t launch_root(int mode, const RootDesc& rd, const int64_t* s0, int nslices, cudaStream_t st) {
  const int64_t E = 1ll << rd.r.outer_bits;
  if (rd.part) {  // fused root (a count): a warp per slice, the last CTA adds them up
    k_root_parts<<<(unsigned)((nslices + kThreads / 32 - 1) / (kThreads / 32)), kThreads, 0, st>>>(rd, nslices);
    return cudaGetLastError();
  }
  if (E <= 1024) {  // few root entries: a CTA per entry, slices across its threads
    if (mode == 0) k_root_tree<0, double><<<(unsigned)E, kThreads, 0, st>>>(rd, s0, nslices);
    else if (mode == 2) k_root_tree<2, u64><<<(unsigned)E, kThreads, 0, st>>>(rd, s0, nslices);
    else if (mode == 3) k_root_tree<3, u64><<<(unsigned)E, kThreads, 0, st>>>(rd, s0, nslices);
    else k_root_tree<1, float><<<(unsigned)E, kThreads, 0, st>>>(rd, s0, nslices);
    return cudaGetLastError();
  }
  const int g = grid_for(E);
  if (mode == 0) k_root<0, double><<<g, kThreads, 0, st>>>(rd, s0, nslices);
  else if (mode == 2) k_root<2, u64><<<g, kThreads, 0, st>>>(rd, s0, nslices);
  else if (mode == 3) k_root<3, u64><<<g, kThreads, 0, st>>>(rd, s0, nslices);
  else k_root<1, float><<<g, kThreads, 0, st>>>(rd, s0, nslices);
  return cudaGetLastError();
}

cudaError_t launch_build_leaves(const LeafBuild* items, int n, double* v64, float* v32, float* v32lo,
                                cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_build_leaves<<<n, kThreads, 0, st>>>(items, v64, v32, v32lo);
  return cudaGetLastError();
}

cudaError_t launch_set_s0(int64_t* d_s0, int64_t value, cudaStream_t st) {
  k_set_s0<<<1, 1, 0, st>>>(d_s0, value);
  return cudaGetLastError();
}

cudaError_t launch_leaf_int(const double* v64, void* out, int64_t n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_leaf_int<<<grid_for(n), kThreads, 0, st>>>(v64, (u64*)out, n);
  return cudaGetLastError();
}

cudaError_t launch_leaf_mod(const double* v64, void* out, int64_t n, uint64_t p, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (p < 2 || p >= (1ull << 28)) return cudaErrorInvalidValue;
  k_leaf_mod<<<grid_for(n), kThreads, 0, st>>>(v64, (u64*)out, n, (long long)p);
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
  const int iters = kind == 0 ? 2048 : (kind == 1 ? 65536 : 8192);
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  for (int rep = 0; rep < 3; ++rep) {  // the first passes bring the clocks up
    cudaEventRecord(t0, st);
    if (kind == 0) k_probe<double><<<blocks, kThreads, 0, st>>>((double*)out, iters, 1.0);
    else if (kind == 1) k_probe<float><<<blocks, kThreads, 0, st>>>((float*)out, iters, 1.0f);
    else k_probe_dmma<<<blocks, kThreads, 0, st>>>((double*)out, iters);
    cudaEventRecord(t1, st);
  }
  e = cudaEventSynchronize(t1);
  float ms = 0;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(out);
  if (e != cudaSuccess) return e;
  const double threads = (double)blocks * kThreads;
  const double work = kind == 2 ? threads / 32.0 * 8.0 * iters * 512.0   // FLOP per warp-mma: 2*8*8*4
                                : threads * 2.0 * 64.0 * iters;
  *flops = work / (ms * 1e-3);
  return cudaGetLastError();
}

}  // namespace togb
