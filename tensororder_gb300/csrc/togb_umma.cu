// Split-form GEMM joins on the 5th-generation tensor cores (sm_103a).
//
// C[b][m,n] = sum_k A[b][m,k] * B[b][n,k] with FP32 operands, computed as
// 3xTF32: every operand value v (normalised to its slice maximum in [1,2)) is
// split into hi = tf32_rn(v) and lo = tf32_rn(v - hi), and
//
//     D_main += A_hi . B_hi          D_corr += A_hi . B_lo + A_lo . B_hi
//
// with the accumulators in tensor memory (FP32).  The dropped A_lo . B_lo term
// is ~2^-22 relative.  The tensor core rounds its FP32 accumulation toward
// zero, so a long-lived accumulator loses about one ulp per update, always in
// the same direction (measured: ~1.3e-6 low after 32 updates).  The main
// products of each 32-wide K chunk therefore go into fresh tensor-memory sets
// (two k-steps per set, sets ping-ponged by chunk parity) which the warps read
// with tcgen05.ld and add into round-to-nearest FP32 registers while the next
// chunk's MMAs run; only the ~2^-11 smaller correction products stay in one
// accumulator for the whole K range.
//
// One CTA (8 warps) owns a 128 x 64 output tile of one slice.  The A and B
// tiles of each 32-wide K chunk arrive in a 4-deep ring of raw FP32 stages, so
// three chunks of loads are always in flight.  When both operands are plain
// row-major K-major matrices (the layout planner asks producers for exactly
// that), one thread loads each tile with a TMA bulk tensor copy (128-byte
// swizzle, mbarrier transaction count); otherwise every thread gathers
// elements from their deposit layouts with cp.async.  A shared-to-shared pass then normalises each value, splits it
// into hi/lo and writes both in the canonical no-swizzle K-major UMMA layout
// (2 stages); one thread issues the 12 tcgen05.mma of the chunk and commits
// them to an mbarrier.  The epilogue adds the
// correction accumulator, stores C through its deposit layout and records the
// slice maximum and exponent like the other split-form kernels.
//
// Every wait on an mbarrier is bounded (about a second of clock64 time); on
// expiry the kernel raises the join's error word, waits a bounded time for its
// own MMAs, frees its tensor memory and returns.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstring>

#include "togb_device.cuh"
#include "togb_internal.h"
#include "togb_tcgen05.cuh"

namespace togb {
namespace {

template <int BN>
struct UmmaSmem {
  static constexpr int A_BYTES = kBM * kBK * 4;
  static constexpr int B_BYTES = BN * kBK * 4;
  static constexpr int STAGE = 2 * A_BYTES + 2 * B_BYTES;  // hi/lo, canonical layout
  static constexpr int RAW = A_BYTES + B_BYTES;             // raw FP32, [row][k]
  static constexpr int NRAW = 4;
  static constexpr int DYN = 2 * STAGE + NRAW * RAW + 1024;
};

// Tensor-memory columns: main sets [parity][half] at (2*parity + half) * BN,
// the correction accumulator at 4 * BN.
template <int BN, bool TMA>
__global__ void __launch_bounds__(kUmmaThreads, 1) k_umma(const __grid_constant__ JoinDesc jd,
                                                         const __grid_constant__ CUtensorMap tmA,
                                                         const __grid_constant__ CUtensorMap tmB,
                                                         const int64_t* __restrict__ d_s0, int nslices,
                                                         int tiles_n_bits) {
  using L = UmmaSmem<BN>;
  constexpr uint32_t kCols = 512;  // 5 * BN rounded up to a power of two
  static_assert(5 * BN <= (int)kCols, "tensor memory budget");
  extern __shared__ unsigned char dyn_raw[];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ __align__(8) uint64_t mbar_full[4];  // TMA: raw stage filled
  __shared__ uint32_t tmem_base_sh;
  __shared__ int timeout_sh;
  __shared__ int64_t tAm[kBM], tBn[BN], tCm[kBM], tCn[BN], tAk[kBK], tBk[kBK];
  __shared__ uint32_t red[kUmmaThreads / 32];

  const int b = blockIdx.y + blockIdx.z * gridDim.y;
  if (b >= nslices) return;
  // After one CTA's wait expired the result is void: later CTAs leave at once.
  if (jd.err && *(volatile int32_t*)jd.err) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  unsigned char* smem = (unsigned char*)(((uintptr_t)dyn_raw + 1023) & ~(uintptr_t)1023);
  const uint32_t smem_base = smem_u32(smem);

  const int64_t s = (d_s0 ? *d_s0 : 0) + b;
  const uint64_t tile = blockIdx.x;
  const uint64_t m0 = (tile >> tiles_n_bits) * kBM;
  const uint64_t n0 = (tile & ((1ull << tiles_n_bits) - 1)) * BN;
  const int64_t M = 1ll << jd.mb, N = 1ll << jd.nb, K = 1ll << jd.kb;
  const int mlim = (int)min((int64_t)kBM, M - (int64_t)m0);
  const int nlim = (int)min((int64_t)BN, N - (int64_t)n0);
  const int klim = (int)min((int64_t)kBK, K);
  const int nchunks = (int)((K + kBK - 1) / kBK);

  for (int i = tid; i < kBM; i += kUmmaThreads) {
    tAm[i] = deposit(jd.a.s_outer, i);
    tCm[i] = deposit(jd.c_s_m, i);
  }
  for (int i = tid; i < BN; i += kUmmaThreads) {
    tBn[i] = deposit(jd.b.s_outer, i);
    tCn[i] = deposit(jd.c_s_n, i);
  }
  if (tid < kBK) {
    tAk[tid] = deposit(jd.a.s_k, tid);
    tBk[tid] = deposit(jd.b.s_k, tid);
  }
  if (tid == 0) {
    mbar_init(smem_u32(&mbar[0]), 1);
    mbar_init(smem_u32(&mbar[1]), 1);
    for (int i = 0; i < 4; ++i) mbar_init(smem_u32(&mbar_full[i]), 1);
    fence_mbar_init();
    timeout_sh = 0;
  }
  if (warp == 0) {
    tmem_alloc(smem_u32(&tmem_base_sh), kCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_sh;
  const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);

  const float* __restrict__ A = (const float*)jd.a.ptr + slice_offset(jd.a, b, s) + deposit(jd.a.s_outer, m0);
  const float* __restrict__ B = (const float*)jd.b.ptr + slice_offset(jd.b, b, s) + deposit(jd.b.s_outer, n0);
  const int sa = op_shift(jd.a, b), sb = op_shift(jd.b, b);
  const float fa = pow2f(sa), fb = pow2f(sb);
  constexpr uint32_t kIdesc = idesc_tf32(kBM, BN);

  constexpr int HALF = BN / 2;  // TMEM columns read out per warp
  const int col0 = (warp >> 2) * HALF;
  unsigned char* raw = smem + 2 * L::STAGE;
  const uint32_t raw_base = smem_base + 2 * L::STAGE;

  // TMA: one thread loads chunk c's A and B boxes into raw stage c%4.
  auto issue_tma = [&](int c) {
    const int r = c % L::NRAW;
    const uint32_t dst = raw_base + r * L::RAW;
    const uint32_t full = smem_u32(&mbar_full[r]);
    mbar_expect_tx(full, (uint32_t)L::RAW);
    tma_load_3d(dst, &tmA, full, c * kBK, (int)m0, b);
    tma_load_3d(dst + L::A_BYTES, &tmB, full, c * kBK, (int)n0, b);
  };
  // Raw stage r holds A (128 x 32) then B (BN x 32), each already in the
  // canonical [k/4][row][4] order, so the split pass is element-wise.
  auto gather = [&](int c) {
    const int64_t k0 = (int64_t)c * kBK;
    const int64_t dak = deposit(jd.a.s_k, (uint64_t)k0), dbk = deposit(jd.b.s_k, (uint64_t)k0);
    const uint32_t dst = raw_base + (c % L::NRAW) * L::RAW;
#pragma unroll 4
    for (int e = tid; e < kBM * kBK; e += kUmmaThreads) {
      int row, kk;
      if (jd.a.k_fast) { kk = e & (kBK - 1); row = e >> 5; } else { row = e & (kBM - 1); kk = e >> 7; }
      const bool v = row < mlim && kk < klim && k0 + kk < K;
      cp_async4(dst + canon_off(row, kk, kBM), v ? (const void*)(A + dak + tAm[row] + tAk[kk]) : (const void*)A, v);
    }
#pragma unroll 4
    for (int e = tid; e < BN * kBK; e += kUmmaThreads) {
      int row, kk;
      if (jd.b.k_fast) { kk = e & (kBK - 1); row = e >> 5; } else { row = e % BN; kk = e / BN; }
      const bool v = row < nlim && kk < klim && k0 + kk < K;
      cp_async4(dst + L::A_BYTES + canon_off(row, kk, BN), v ? (const void*)(B + dbk + tBn[row] + tBk[kk]) : (const void*)B,
                v);
    }
  };
  auto split_store = [&](unsigned char* dst_hi, unsigned char* dst_lo, uint32_t off, float4 x4, float f) {
    float4 hi, lo;
    const float* x = &x4.x;
    float* h = &hi.x;
    float* l = &lo.x;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float v = x[q] * f;
      h[q] = tf32_rn(v);
      l[q] = tf32_rn(v - h[q]);
    }
    *reinterpret_cast<float4*>(dst_hi + off) = hi;
    *reinterpret_cast<float4*>(dst_lo + off) = lo;
  };

  float acc[HALF];
#pragma unroll
  for (int j = 0; j < HALF; ++j) acc[j] = 0.f;

  // Prologue: chunks 0..2 in flight (one commit group per chunk, empty ones too).
#pragma unroll
  for (int c = 0; c < L::NRAW - 1; ++c) {
    if constexpr (TMA) {
      if (tid == 0 && c < nchunks) issue_tma(c);
    } else {
      if (c < nchunks) gather(c);
      cp_async_commit();
    }
  }
  bool ok = true;
  for (int c = 0; c <= nchunks && ok; ++c) {
    if (c < nchunks) {
      // Raw stage (c+3)%4 last held chunk c-1, converted before the previous
      // iteration's barrier; hi/lo stage c&1 last fed chunk c-2, whose MMAs
      // completed before the read-out of chunk c-2 in the previous iteration.
      if constexpr (TMA) {
        if (tid == 0 && c + L::NRAW - 1 < nchunks) issue_tma(c + L::NRAW - 1);
        if (!mbar_wait_bounded(smem_u32(&mbar_full[c % L::NRAW]), (c / L::NRAW) & 1, jd.wait_cycles)) timeout_sh = 1;
        __syncthreads();
        if (timeout_sh) { ok = false; break; }
      } else {
        if (c + L::NRAW - 1 < nchunks) gather(c + L::NRAW - 1);
        cp_async_commit();
        cp_async_wait<L::NRAW - 1>();
        __syncthreads();
      }
      const int st = c & 1;
      unsigned char* stage = smem + st * L::STAGE;
      const unsigned char* r = raw + (c % L::NRAW) * L::RAW;
#pragma unroll
      for (int u = tid; u < kBM * 8; u += kUmmaThreads) {
        const float4 x = *reinterpret_cast<const float4*>(r + u * 16);
        split_store(stage, stage + L::A_BYTES, (uint32_t)u * 16, x, fa);
      }
#pragma unroll
      for (int u = tid; u < BN * 8; u += kUmmaThreads) {
        const float4 x = *reinterpret_cast<const float4*>(r + L::A_BYTES + u * 16);
        split_store(stage + 2 * L::A_BYTES, stage + 2 * L::A_BYTES + L::B_BYTES, (uint32_t)u * 16, x, fb);
      }
      fence_async_smem();
      tc_fence_before();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        const uint32_t sa_hi = smem_base + st * L::STAGE;
        const uint32_t sa_lo = sa_hi + L::A_BYTES;
        const uint32_t sb_hi = sa_hi + 2 * L::A_BYTES;
        const uint32_t sb_lo = sb_hi + L::B_BYTES;
        const uint32_t lbo_a = kBM * 16, lbo_b = BN * 16;
#pragma unroll
        for (int t = 0; t < kBK / 8; ++t) {
          uint64_t ah, al, bh, bl;
          if constexpr (TMA) {  // swizzled rows: advance 32 B (8 tf32) within the 128 B row
            ah = smem_desc_sw128(sa_hi + 32 * t);
            al = smem_desc_sw128(sa_lo + 32 * t);
            bh = smem_desc_sw128(sb_hi + 32 * t);
            bl = smem_desc_sw128(sb_lo + 32 * t);
          } else {
            ah = smem_desc(sa_hi + 2 * t * lbo_a, lbo_a, 128);
            al = smem_desc(sa_lo + 2 * t * lbo_a, lbo_a, 128);
            bh = smem_desc(sb_hi + 2 * t * lbo_b, lbo_b, 128);
            bl = smem_desc(sb_lo + 2 * t * lbo_b, lbo_b, 128);
          }
          const uint32_t main_set = tmem + (uint32_t)((2 * st + (t >> 1)) * BN);
          umma_tf32(main_set, ah, bh, kIdesc, (t & 1) ? 1u : 0u);
          const uint32_t corr = tmem + 4 * BN;
          umma_tf32(corr, ah, bl, kIdesc, (c > 0 || t > 0) ? 1u : 0u);
          umma_tf32(corr, al, bh, kIdesc, 1u);
        }
        umma_commit(smem_u32(&mbar[st]));
      }
    }
    if (c >= 1) {
      // Read out chunk c-1 once its MMAs completed.
      const int pc = c - 1, pst = pc & 1;
      if (tid == 0 && !mbar_wait_bounded(smem_u32(&mbar[pst]), (pc >> 1) & 1, jd.wait_cycles)) timeout_sh = 1;
      __syncthreads();
      if (timeout_sh) { ok = false; break; }
      tc_fence_after();
#pragma unroll
      for (int col = 0; col < HALF; col += 16) {
        float v0[16], v1[16];
        tmem_ld16(lane_base + (uint32_t)(2 * pst * BN + col0 + col), v0);
        tmem_ld16(lane_base + (uint32_t)((2 * pst + 1) * BN + col0 + col), v1);
        tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 16; ++j) acc[col + j] += v0[j] + v1[j];
      }
      tc_fence_before();
    }
  }
  if constexpr (!TMA) cp_async_wait<0>();

  uint32_t bits = 0;
  if (ok) {
    // The last commit covered every MMA, the correction products included.
    tc_fence_after();
    const int row = (warp & 3) * 32 + lane;
    float* __restrict__ C = (float*)jd.c_ptr + (int64_t)b * jd.c_batch_stride + deposit(jd.c_s_m, m0) +
                            deposit(jd.c_s_n, n0);
#pragma unroll
    for (int col = 0; col < HALF; col += 16) {
      float vc[16];
      tmem_ld16(lane_base + (uint32_t)(4 * BN + col0 + col), vc);
      tmem_ld_wait();
      if (row < mlim) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int n = col0 + col + j;
          if (n < nlim) {
            const float v = acc[col + j] + vc[j];
            C[tCm[row] + tCn[n]] = v;
            bits = max(bits, __float_as_uint(fmaxf(v, 0.f)));
          }
        }
      }
    }
  } else if (tid == 0 && jd.err) {
    atomicExch(jd.err, 1);
  }
  // Tear down: make sure no MMA of ours is still in flight, then free TMEM.
  if (!ok && tid == 0) {
    for (int st = 0; st < 2; ++st)
      for (int ph = 0; ph < 2; ++ph) mbar_wait_bounded(smem_u32(&mbar[st]), ph);
    if (TMA)
      for (int st = 0; st < 4; ++st)
        for (int ph = 0; ph < 2; ++ph) mbar_wait_bounded(smem_u32(&mbar_full[st]), ph);
  }
  for (int off = 16; off > 0; off >>= 1) bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, off));
  if (lane == 0) red[warp] = bits;
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kCols);
  if (ok && tid == 0) {
    uint32_t m = 0;
    for (int w = 0; w < kUmmaThreads / 32; ++w) m = max(m, red[w]);
    atomicMax(&jd.c_max[b], m);
    if (tile == 0) jd.c_exp[b] = op_exp(jd.a, b) + op_exp(jd.b, b) - sa - sb;
  }
}

template <int BN, bool TMA>
cudaError_t launch_bn(const JoinDesc& jd, const CUtensorMap& ta, const CUtensorMap& tb, const int64_t* s0,
                      int nslices, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(k_umma<BN, TMA>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       UmmaSmem<BN>::DYN);
  if (e != cudaSuccess) return e;
  const int tm_bits = jd.mb > 7 ? jd.mb - 7 : 0;
  const int tn_bits = jd.nb > 6 ? jd.nb - 6 : 0;
  const uint64_t tiles = 1ull << (tm_bits + tn_bits);
  if (tiles > 0x7fffffffull) return cudaErrorInvalidValue;
  const int gy = nslices < 65535 ? nslices : 65535;
  const int gz = (nslices + gy - 1) / gy;
  k_umma<BN, TMA><<<dim3((unsigned)tiles, gy, gz), kUmmaThreads, UmmaSmem<BN>::DYN, st>>>(jd, ta, tb, s0, nslices,
                                                                                           tn_bits);
  return cudaGetLastError();
}

// Tensor-pipe probe: one CTA per SM issues back-to-back kind::tf32 MMAs
// (M=128, N=256, K=8) from a zeroed shared-memory tile into tensor memory.
__global__ void __launch_bounds__(128, 1) k_probe_umma(int iters, int32_t* err) {
  extern __shared__ unsigned char dyn_raw[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_sh;
  unsigned char* smem = (unsigned char*)(((uintptr_t)dyn_raw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x;
  for (int i = tid; i < (16384 + 32768) / 16; i += blockDim.x) reinterpret_cast<float4*>(smem)[i] = make_float4(0, 0, 0, 0);
  if (tid == 0) {
    mbar_init(smem_u32(&mbar), 1);
    fence_mbar_init();
  }
  if (tid < 32) {
    tmem_alloc(smem_u32(&tmem_sh), 256);
    tmem_relinquish();
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_sh;
  bool ok = true;
  if (tid == 0) {
    const uint32_t a = smem_u32(smem), b = a + 16384;
    constexpr uint32_t idesc = idesc_tf32(128, 256);
    for (int it = 0; it < iters; ++it)
#pragma unroll
      for (int t = 0; t < 4; ++t)
        umma_tf32(tmem, smem_desc_sw128(a + 32 * t), smem_desc_sw128(b + 32 * t), idesc, (it | t) ? 1u : 0u);
    umma_commit(smem_u32(&mbar));
    ok = mbar_wait_bounded(smem_u32(&mbar), 0);
    if (!ok && err) atomicExch(err, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (tid < 32) tmem_dealloc(tmem, 256);
}

}  // namespace

cudaError_t probe_umma(cudaStream_t st, double* flops) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int dyn = 16384 + 32768 + 1024;
  cudaError_t e = cudaFuncSetAttribute(k_probe_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
  if (e != cudaSuccess) return e;
  int32_t* err = nullptr;
  if ((e = cudaMalloc(&err, 4)) != cudaSuccess) return e;
  cudaMemsetAsync(err, 0, 4, st);
  const int iters = 4096;
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  for (int rep = 0; rep < 2; ++rep) {
    cudaEventRecord(t0, st);
    k_probe_umma<<<sms, 128, dyn, st>>>(iters, err);
    cudaEventRecord(t1, st);
  }
  e = cudaEventSynchronize(t1);
  float ms = 0;
  cudaEventElapsedTime(&ms, t0, t1);
  int32_t herr = 0;
  cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(err);
  if (e != cudaSuccess) return e;
  if (herr) return cudaErrorLaunchTimeout;
  *flops = (double)sms * iters * 4 * 2.0 * 128 * 256 * 8 / (ms * 1e-3);
  return cudaGetLastError();
}

cudaError_t launch_umma(const JoinDesc& jd, const CUtensorMap* ta, const CUtensorMap* tb, const int64_t* s0,
                        int nslices, cudaStream_t st) {
  if (ta && tb) return launch_umma_ws(jd, *ta, *tb, nslices, st);
  CUtensorMap none;
  memset(&none, 0, sizeof(none));
  return launch_bn<64, false>(jd, none, none, s0, nslices, st);
}

}  // namespace togb
