// Split-form GEMM joins on the tensor cores, warp-specialised (sm_103a).
//
// C[b][m,n] = sum_k A[b][m,k] * B[b][n,k] with FP32 operands stored as plain
// K-major matrices (the layout the planner asks producers of GEMM operands to
// write), as 3xTF32: each operand value v, scaled to its slice maximum in
// [1, 2), is split into hi = tf32_rn(v) and lo = tf32_rn(v - hi), and every
// product is hi.hi + hi.lo + lo.hi (the dropped lo.lo term is ~2^-22).
//
// One CTA computes a 128 x BN output tile of one slice with four roles:
//   warp 0        TMA producer: loads the 32-wide K chunks of A and B (128-byte
//                 swizzle) into a ring of NST stages;
//   warps 4-7     converters: split each landed chunk in place into hi and a
//                 second, identically swizzled lo buffer;
//   warp 1        MMA issuer: one thread issues the tcgen05.mma of each chunk;
//   warps 8-15    read-out: drain the tensor-memory accumulators into FP32
//                 registers and run the epilogue.
// The tensor core truncates its FP32 accumulation, so one accumulator must not
// see many large updates.  The K range is therefore cut into windows of 16
// (two MMA k-steps); each window accumulates into a fresh tensor-memory set
// (two sets, alternating), correction products first while the set is still
// small, main products last, and the read-out warps add the window into
// round-to-nearest registers while the next window's MMAs run.
//
// The epilogue stages the tile in shared memory and writes it in the output's
// own address order (row-major float4 stores when the output's lowest address
// bits are the tile's n bits), then records the slice maximum and exponent
// like the other split-form kernels.
//
// Operands that do not vary with the slice (slice-invariant intermediates) use
// a tensor map with one slice and slice coordinate 0.  Every wait is bounded:
// on expiry the role raises a shared abort flag, the others leave their loops,
// the producer waits (bounded) for its loads in flight, the MMA thread for its
// MMAs, tensor memory is freed and the join's error word is set.
#include <cuda.h>
#include <cuda_runtime.h>

#include "togb_device.cuh"
#include "togb_internal.h"
#include "togb_tcgen05.cuh"

namespace togb {
namespace {

constexpr int kWsThreads = 512;  // 16 warps

template <int BN, int NST>
struct WsSmem {
  static constexpr int A_BYTES = kBM * kBK * 4;
  static constexpr int B_BYTES = BN * kBK * 4;
  static constexpr int RAW = A_BYTES + B_BYTES;  // TMA target, converted in place to hi
  static constexpr int STAGE = 2 * RAW;          // [hi: A | B][lo: A | B]
  static constexpr int CROW = BN + 4;            // staging row stride of the output tile (floats)
  static constexpr int DYN = NST * STAGE + 1024;
  static_assert(kBM * CROW * 4 <= NST * STAGE, "output staging tile fits in the stages");
  static_assert(DYN <= 227 * 1024, "shared memory budget");
};

__device__ __forceinline__ void split4(float4 x, float f, float4& hi, float4& lo) {
  const float* v = &x.x;
  float* h = &hi.x;
  float* l = &lo.x;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float s = v[q] * f;
    h[q] = tf32_rn(s);
    l[q] = tf32_rn(s - h[q]);
  }
}

template <int BN, int NST>
__global__ void __launch_bounds__(kWsThreads, 1) k_umma_ws(const __grid_constant__ JoinDesc jd,
                                                          const __grid_constant__ CUtensorMap tmA,
                                                          const __grid_constant__ CUtensorMap tmB,
                                                          int nslices, int tiles_n_bits) {
  using L = WsSmem<BN, NST>;
  constexpr int HALF = BN / 2;        // columns per read-out warp
  constexpr uint32_t kCols = 2 * BN;  // two accumulator sets
  constexpr int kConv = 128;          // converter threads
  constexpr int kRead = 256;          // read-out threads
  extern __shared__ unsigned char dyn_raw[];
  __shared__ __align__(8) uint64_t full[NST], conv[NST], empty[NST], accf[2], acce[2], fin;
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh;
  __shared__ int64_t tCm[kBM], tCn[BN];
  __shared__ uint32_t red[kRead / 32];

  const int b = blockIdx.y + blockIdx.z * gridDim.y;
  if (b >= nslices) return;
  // After one CTA's wait expired the result is void: later CTAs leave at once.
  if (jd.err && *(volatile int32_t*)jd.err) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  unsigned char* smem = (unsigned char*)(((uintptr_t)dyn_raw + 1023) & ~(uintptr_t)1023);
  const uint32_t sbase = smem_u32(smem);
  const uint64_t tile = blockIdx.x;
  const uint64_t m0 = (tile >> tiles_n_bits) * kBM;
  const uint64_t n0 = (tile & ((1ull << tiles_n_bits) - 1)) * BN;
  const int64_t M = 1ll << jd.mb, N = 1ll << jd.nb, K = 1ll << jd.kb;
  const int mlim = (int)min((int64_t)kBM, M - (int64_t)m0);
  const int nlim = (int)min((int64_t)BN, N - (int64_t)n0);
  const int ksteps = K >= 8 ? (int)(K / 8) : 1;  // MMA k-steps of 8
  const int nwin = (ksteps + 1) / 2;              // windows of two k-steps
  const int nchunks = (nwin + 1) / 2;             // TMA chunks of four k-steps

  for (int i = tid; i < kBM; i += kWsThreads) tCm[i] = deposit(jd.c_s_m, i);
  for (int i = tid; i < BN; i += kWsThreads) tCn[i] = deposit(jd.c_s_n, i);
  if (tid == 0) {
    for (int i = 0; i < NST; ++i) {
      mbar_init(smem_u32(&full[i]), 1);
      mbar_init(smem_u32(&conv[i]), kConv);
      mbar_init(smem_u32(&empty[i]), 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(smem_u32(&accf[i]), 1);
      mbar_init(smem_u32(&acce[i]), kRead);
    }
    mbar_init(smem_u32(&fin), 1);
    fence_mbar_init();
    abort_sh = 0;
  }
  if (warp == 1) {
    tmem_alloc(smem_u32(&tmem_sh), kCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_sh;
  volatile int* abort = &abort_sh;
  const int sa = op_shift(jd.a, b), sb = op_shift(jd.b, b);

  if (warp == 0) {
    // ---------------------------------------------------------------- producer
    if (lane == 0) {
      const int asl = jd.a.batch_stride ? b : 0, bsl = jd.b.batch_stride ? b : 0;
      int issued = 0;
      for (int c = 0; c < nchunks; ++c) {
        const int st = c % NST, u = c / NST;
        if (c >= NST && !mbar_wait_or_abort(smem_u32(&empty[st]), (u - 1) & 1, abort)) {
          *abort = 1;
          break;
        }
        const uint32_t dst = sbase + st * L::STAGE;
        const uint32_t bar = smem_u32(&full[st]);
        mbar_expect_tx(bar, (uint32_t)L::RAW);
        tma_load_3d(dst, &tmA, bar, c * kBK, (int)m0, asl);
        tma_load_3d(dst + L::A_BYTES, &tmB, bar, c * kBK, (int)n0, bsl);
        issued = c + 1;
      }
      if (*abort)  // loads still in flight must land before the CTA may exit
        for (int c = max(0, issued - NST); c < issued; ++c) mbar_wait_bounded(smem_u32(&full[c % NST]), (c / NST) & 1);
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------------- MMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_tf32(kBM, BN);
      bool ok = true;
      for (int c = 0; c < nchunks && ok; ++c) {
        const int st = c % NST, u = c / NST;
        if (!mbar_wait_or_abort(smem_u32(&conv[st]), u & 1, abort)) { ok = false; break; }
        tc_fence_after();
        const uint32_t a_hi = sbase + st * L::STAGE, b_hi = a_hi + L::A_BYTES;
        const uint32_t a_lo = a_hi + L::RAW, b_lo = a_lo + L::A_BYTES;
        for (int h = 0; h < 2; ++h) {
          const int w = 2 * c + h;
          if (w >= nwin) break;
          const int set = w & 1;
          if (w >= 2 && !mbar_wait_or_abort(smem_u32(&acce[set]), ((w >> 1) - 1) & 1, abort)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t d = tmem + (uint32_t)(set * BN);
          const int t0 = 2 * h, t1 = min(2 * h + 2, ksteps - 4 * c);
          uint32_t accum = 0;
          for (int t = t0; t < t1; ++t) {  // corrections while the set is small
            umma_tf32(d, smem_desc_sw128(a_hi + 32 * t), smem_desc_sw128(b_lo + 32 * t), idesc, accum);
            accum = 1;
            umma_tf32(d, smem_desc_sw128(a_lo + 32 * t), smem_desc_sw128(b_hi + 32 * t), idesc, 1u);
          }
          for (int t = t0; t < t1; ++t)
            umma_tf32(d, smem_desc_sw128(a_hi + 32 * t), smem_desc_sw128(b_hi + 32 * t), idesc, 1u);
          umma_commit(smem_u32(&accf[set]));
        }
        umma_commit(smem_u32(&empty[st]));
      }
      if (!ok) *abort = 1;
      // Every MMA of this thread completes before tensor memory is freed.
      umma_commit(smem_u32(&fin));
      mbar_wait_bounded(smem_u32(&fin), 0);
    }
    __syncwarp();
  } else if (warp >= 4 && warp < 8) {
    // ---------------------------------------------------------------- converters
    const int ct = tid - 128;
    const float fa = pow2f(sa), fb = pow2f(sb);
    for (int c = 0; c < nchunks; ++c) {
      const int st = c % NST, u = c / NST;
      if (!mbar_wait_or_abort(smem_u32(&full[st]), u & 1, abort)) {
        *abort = 1;
        break;
      }
      unsigned char* hi = smem + st * L::STAGE;
      unsigned char* lo = hi + L::RAW;
#pragma unroll 4
      for (int e = ct; e < L::RAW / 16; e += kConv) {
        const float4 x = *reinterpret_cast<const float4*>(hi + e * 16);
        float4 h, l;
        split4(x, e * 16 < L::A_BYTES ? fa : fb, h, l);
        *reinterpret_cast<float4*>(hi + e * 16) = h;
        *reinterpret_cast<float4*>(lo + e * 16) = l;
      }
      fence_async_smem();
      mbar_arrive(smem_u32(&conv[st]));
    }
  } else if (warp >= 8) {
    // ---------------------------------------------------------------- read-out + epilogue
    const int q = warp & 3, hf = (warp - 8) >> 2, rt = tid - 256;
    const int row = 32 * q + lane;
    const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(hf * HALF);
    float acc[HALF];
#pragma unroll
    for (int j = 0; j < HALF; ++j) acc[j] = 0.f;
    for (int w = 0; w < nwin; ++w) {
      const int set = w & 1;
      if (!mbar_wait_or_abort(smem_u32(&accf[set]), (w >> 1) & 1, abort)) {
        *abort = 1;
        break;
      }
      tc_fence_after();
#pragma unroll
      for (int col = 0; col < HALF; col += 32) {
        float v0[16], v1[16];
        tmem_ld16(tl + (uint32_t)(set * BN + col), v0);
        tmem_ld16(tl + (uint32_t)(set * BN + col + 16), v1);
        tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          acc[col + j] += v0[j];
          acc[col + 16 + j] += v1[j];
        }
      }
      tc_fence_before();
      mbar_arrive(smem_u32(&acce[set]));
    }
    named_bar(1, kRead);  // every read-out done: all MMAs and loads have finished
    uint32_t bits = 0;
    const bool ok = *abort == 0;
    float* cs = reinterpret_cast<float*>(smem);
    if (ok) {
#pragma unroll
      for (int j = 0; j < HALF; j += 4)
        *reinterpret_cast<float4*>(&cs[row * L::CROW + hf * HALF + j]) =
            make_float4(acc[j], acc[j + 1], acc[j + 2], acc[j + 3]);
      if (row < mlim) {
#pragma unroll
        for (int j = 0; j < HALF; ++j)
          if (hf * HALF + j < nlim) bits = max(bits, __float_as_uint(fmaxf(acc[j], 0.f)));
      }
    }
    named_bar(1, kRead);
    if (ok) {
      float* __restrict__ C = (float*)jd.c_ptr + (int64_t)b * jd.c_batch_stride + deposit(jd.c_s_m, m0) +
                              deposit(jd.c_s_n, n0);
      // Row-major float4 stores when the tile's n bits are the output's lowest address bits.
      bool rowmajor = (nlim & 3) == 0;
      for (int i = 0; (1 << i) < nlim; ++i) rowmajor = rowmajor && jd.c_s_n[i] == (1ll << i);
      if (rowmajor) {
        constexpr int V = BN / 4;
        for (int idx = rt; idx < kBM * V; idx += kRead) {
          const int r = idx / V, c4 = idx - r * V;
          if (r < mlim && 4 * c4 < nlim)
            *reinterpret_cast<float4*>(C + tCm[r] + 4 * c4) = *reinterpret_cast<const float4*>(&cs[r * L::CROW + 4 * c4]);
        }
      } else {
        for (int idx = rt; idx < kBM * BN; idx += kRead) {
          const int r = idx & (kBM - 1), c = idx >> 7;
          if (r < mlim && c < nlim) C[tCm[r] + tCn[c]] = cs[r * L::CROW + c];
        }
      }
    }
    for (int off = 16; off > 0; off >>= 1) bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, off));
    if (lane == 0) red[warp - 8] = bits;
    named_bar(1, kRead);
    if (rt == 0 && ok) {
      uint32_t m = 0;
      for (int i = 0; i < kRead / 32; ++i) m = max(m, red[i]);
      atomicMax(&jd.c_max[b], m);
      if (tile == 0) jd.c_exp[b] = op_exp(jd.a, b) + op_exp(jd.b, b) - sa - sb;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) tmem_dealloc(tmem, kCols);
  if (tid == 0 && abort_sh && jd.err) atomicExch(jd.err, 1);
}

template <int BN, int NST>
cudaError_t launch_ws(const JoinDesc& jd, const CUtensorMap& ta, const CUtensorMap& tb, int nslices,
                      cudaStream_t st) {
  using L = WsSmem<BN, NST>;
  cudaError_t e = cudaFuncSetAttribute(k_umma_ws<BN, NST>, cudaFuncAttributeMaxDynamicSharedMemorySize, L::DYN);
  if (e != cudaSuccess) return e;
  constexpr int bn_bits = BN == 128 ? 7 : 6;
  const int tm_bits = jd.mb > 7 ? jd.mb - 7 : 0;
  const int tn_bits = jd.nb > bn_bits ? jd.nb - bn_bits : 0;
  const uint64_t tiles = 1ull << (tm_bits + tn_bits);
  if (tiles > 0x7fffffffull) return cudaErrorInvalidValue;
  const int gy = nslices < 65535 ? nslices : 65535;
  const int gz = (nslices + gy - 1) / gy;
  k_umma_ws<BN, NST><<<dim3((unsigned)tiles, gy, gz), kWsThreads, L::DYN, st>>>(jd, ta, tb, nslices, tn_bits);
  return cudaGetLastError();
}

}  // namespace

int umma_ws_box_rows_b(int nb) { return nb >= 7 ? 128 : 64; }

cudaError_t launch_umma_ws(const JoinDesc& jd, const CUtensorMap& ta, const CUtensorMap& tb, int nslices,
                           cudaStream_t st) {
  if (jd.nb >= 7) return launch_ws<128, 3>(jd, ta, tb, nslices, st);
  return launch_ws<64, 4>(jd, ta, tb, nslices, st);
}

}  // namespace togb
