// Split-form GEMM joins on the tensor cores, warp-specialised (sm_103a).
//
// C[b][m,n] = sum_k A[b][m,k] * B[b][n,k] with FP32 operands stored as plain
// K-major matrices (the layout the planner asks producers of GEMM operands to
// write), as 3xTF32: each operand value v, scaled to its slice maximum in
// [1, 2), is split into hi = tf32_rn(v) and lo = tf32_rn(v - hi), and every
// product is hi.hi + hi.lo + lo.hi (the dropped lo.lo term is ~2^-22).
//
// One CTA computes a 128 x BN output tile of one slice with four roles, over a
// ring of NS stages, each a hi buffer and a lo buffer of [A | B] chunk rows:
//   warp 0        TMA producer: loads the 32-wide K chunks of A and B (128-byte
//                 swizzle) into a stage's hi buffer once the MMAs of the chunk
//                 it held have completed;
//   warps 2-7     converters: split each landed chunk in place -- hi over the
//                 loaded values, lo into the stage's lo buffer, same swizzled
//                 layout -- so a stage costs no separate raw buffer and three
//                 stages fit (the loads run up to two chunks ahead);
//   warp 1        MMA issuer: one thread issues the tcgen05.mma of each chunk;
//   warps 8-15    read-out: drain the tensor-memory accumulators into FP32
//                 registers and run the epilogue.
// The tensor core truncates its FP32 accumulation, so one accumulator must not
// see many large updates.  The K range is therefore cut into windows of 32
// (one TMA chunk, four MMA k-steps); each window accumulates into a fresh
// tensor-memory set (512 / BN sets used in rotation, so the MMAs run several
// windows ahead of the read-out), correction products first while the set is
// still small, main products last, and the read-out warps add the window into
// round-to-nearest registers while later windows' MMAs run.
//
// The kernel is persistent (one CTA per SM walking the tiles), so the next
// tile's loads, conversions and first MMAs overlap the current tile's
// epilogue.  Each read-out thread owns one output row.  When the tile's two
// lowest n bits are the output's two lowest address bits, every read-out warp
// transposes its 32 rows through a private shared-memory area and stores
// 16-byte vectors, four rows of eight per instruction (whole 128-byte row
// segments when the first five n bits are contiguous) -- or, when the host
// finds that consecutive rows lie close together in the output (c_direct),
// each lane stores its own row's vectors without the staging round trip;
// otherwise lanes store their rows' columns directly (coalesced when the m
// bits are lowest).  The
// layout planner orders a GEMM consumer's shared axes so that the larger of its
// GEMM-shaped producers gets such a layout.
// The slice maximum and exponent are recorded like in the other split-form
// kernels.
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

template <int BN, int NS>
struct WsSmem {
  static constexpr int A_BYTES = kBM * kBK * 4;
  static constexpr int B_BYTES = BN * kBK * 4;
  static constexpr int RAW = A_BYTES + B_BYTES;  // one chunk: [A | B]
  static constexpr int CONV = 2 * RAW;           // a stage: [hi: A | B] (the TMA target) [lo: A | B]
  static constexpr int STG = 8 * 32 * 32 * 4;   // per read-out warp: 32 rows x 32 columns of staging
  static constexpr int DYN = NS * CONV + STG + 1024;
  static_assert(DYN + 1536 <= 227 * 1024, "shared memory budget");
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

// Output tiles are numbered slice-major, n-tile fastest: consecutive tiles of
// a CTA's neighbours share their A rows in L2.
struct TileMap {
  int tps_bits, tn_bits;
  __device__ __forceinline__ void decode(int64_t t, int& b, uint64_t& m0, uint64_t& n0, int bn) const {
    b = (int)(t >> tps_bits);
    const uint64_t r = (uint64_t)t & ((1ull << tps_bits) - 1);
    m0 = (r >> tn_bits) * kBM;
    n0 = (r & ((1ull << tn_bits) - 1)) * (uint64_t)bn;
  }
};

// s[i] += x_i * y_i for the four lanes of a vector.
__device__ __forceinline__ void fma4(const float4 x, const float4 y, float* s) {
  s[0] = fmaf(x.x, y.x, s[0]);
  s[1] = fmaf(x.y, y.y, s[1]);
  s[2] = fmaf(x.z, y.z, s[2]);
  s[3] = fmaf(x.w, y.w, s[3]);
}

// Persistent: each CTA walks the tiles blockIdx.x, blockIdx.x + gridDim.x, ...
// The stage ring and the accumulator sets run continuously across tiles, so
// the next tile's loads, conversions and first MMAs overlap the current
// tile's epilogue.
template <int BN, int NS, bool PAIRS>
__global__ void __launch_bounds__(kWsThreads, 1) k_umma_ws(const __grid_constant__ JoinDesc jd,
                                                          const __grid_constant__ CUtensorMap tmA,
                                                          const __grid_constant__ CUtensorMap tmB,
                                                          int64_t ntiles, TileMap tm) {
  using L = WsSmem<BN, NS>;
  constexpr int HALF = BN / 2;         // columns per read-out warp
  constexpr uint32_t kCols = 512;      // all of tensor memory (one CTA per SM)
  constexpr int NSETS = kCols / BN;    // accumulator sets in rotation
  constexpr int kConv = 192;          // converter threads (warps 2-7)
  // Consumer barriers count warps: one elected lane arrives for its warp
  // after a __syncwarp, so a stage costs 6 (or 8) arrivals instead of one per
  // thread.
  constexpr int kConvWarps = kConv / 32;
  constexpr int kReadWarps = 8;
  extern __shared__ unsigned char dyn_raw[];
  __shared__ __align__(8) uint64_t full[NS], conv[NS], cfree[NS], accf[NSETS], acce[NSETS], fin;
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh;
  __shared__ int32_t tCm[kBM], tCn[BN];  // output offsets within a tile (< 2^31 per slice)

  // After one CTA's wait expired the result is void: later CTAs leave at once.
  if (jd.err && *(volatile int32_t*)jd.err) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  unsigned char* smem = (unsigned char*)(((uintptr_t)dyn_raw + 1023) & ~(uintptr_t)1023);
  const uint32_t sbase = smem_u32(smem);
  const int64_t M = 1ll << jd.mb, N = 1ll << jd.nb, K = 1ll << jd.kb;
  const int ksteps = K >= 8 ? (int)(K / 8) : 1;  // MMA k-steps of 8
  const int nchunks = (ksteps + 3) / 4;           // TMA chunks of four k-steps
  const int nwin = nchunks;                       // one accumulation window per chunk

  for (int i = tid; i < kBM; i += kWsThreads) tCm[i] = (int32_t)deposit(jd.c_s_m, i);
  for (int i = tid; i < BN; i += kWsThreads) tCn[i] = (int32_t)deposit(jd.c_s_n, i);
  if (tid == 0) {
    for (int i = 0; i < NS; ++i) {
      mbar_init(smem_u32(&full[i]), 1);
      mbar_init(smem_u32(&conv[i]), kConvWarps);
      mbar_init(smem_u32(&cfree[i]), 1);
    }
    for (int i = 0; i < NSETS; ++i) {
      mbar_init(smem_u32(&accf[i]), 1);
      mbar_init(smem_u32(&acce[i]), kReadWarps);
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

  if (warp == 0) {
    // ---------------------------------------------------------------- producer
    if (lane == 0) {
      int gc = 0;  // chunks issued by this CTA
      for (int64_t t = blockIdx.x; t < ntiles && !*abort; t += gridDim.x) {
        int b;
        uint64_t m0, n0;
        tm.decode(t, b, m0, n0, BN);
        const int asl = jd.a.batch_stride ? b : 0, bsl = jd.b.batch_stride ? b : 0;
        for (int c = 0; c < nchunks; ++c, ++gc) {
          const int st = gc % NS, u = gc / NS;
          // The stage is free once the MMAs of the chunk it held have completed.
          if (gc >= NS && !mbar_wait_or_abort(smem_u32(&cfree[st]), (u - 1) & 1, abort, jd.wait_cycles)) {
            *abort = 1;
            break;
          }
          const uint32_t dst = sbase + st * L::CONV;
          const uint32_t bar = smem_u32(&full[st]);
          mbar_expect_tx(bar, (uint32_t)L::RAW);
          tma_load_3d(dst, &tmA, bar, c * kBK, (int)m0, asl);
          tma_load_3d(dst + L::A_BYTES, &tmB, bar, c * kBK, (int)n0, bsl);
        }
      }
      if (*abort)  // loads still in flight must land before the CTA may exit
        for (int c = max(0, gc - NS); c < gc; ++c) mbar_wait_bounded(smem_u32(&full[c % NS]), (c / NS) & 1);
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------------- MMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_tf32(kBM, BN);
      bool ok = true;
      int gc = 0, gw = 0;  // chunks and windows consumed by this CTA
      for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        for (int c = 0; c < nchunks && ok; ++c, ++gc) {
          const int st = gc % NS, u = gc / NS;
          if (!mbar_wait_or_abort(smem_u32(&conv[st]), u & 1, abort, jd.wait_cycles)) { ok = false; break; }
          tc_fence_after();
          const uint32_t a_hi = sbase + st * L::CONV, b_hi = a_hi + L::A_BYTES;
          const uint32_t a_lo = a_hi + L::RAW, b_lo = a_lo + L::A_BYTES;
          {
            const int set = gw % NSETS;
            if (gw >= NSETS && !mbar_wait_or_abort(smem_u32(&acce[set]), (gw / NSETS - 1) & 1, abort, jd.wait_cycles)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t d = tmem + (uint32_t)(set * BN);
            const int ks = min(4, ksteps - 4 * c);  // k-steps in this chunk
            // Descriptors of the chunk's first k-step; a k-step of 8 FP32
            // values is 32 bytes, +2 in the descriptor's 16-byte address field.
            const uint64_t dah = smem_desc_sw128(a_hi), dal = smem_desc_sw128(a_lo);
            const uint64_t dbh = smem_desc_sw128(b_hi), dbl = smem_desc_sw128(b_lo);
            if (ks == 4) {  // full chunk: twelve MMAs, corrections first while the set is small
#pragma unroll
              for (int k = 0; k < 4; ++k) {
                umma_tf32(d, dah + 2 * k, dbl + 2 * k, idesc, k ? 1u : 0u);
                umma_tf32(d, dal + 2 * k, dbh + 2 * k, idesc, 1u);
              }
#pragma unroll
              for (int k = 0; k < 4; ++k) umma_tf32(d, dah + 2 * k, dbh + 2 * k, idesc, 1u);
            } else {  // short K or the tail chunk
              for (int k = 0; k < ks; ++k) {
                umma_tf32(d, dah + 2 * k, dbl + 2 * k, idesc, k ? 1u : 0u);
                umma_tf32(d, dal + 2 * k, dbh + 2 * k, idesc, 1u);
              }
              for (int k = 0; k < ks; ++k) umma_tf32(d, dah + 2 * k, dbh + 2 * k, idesc, 1u);
            }
            umma_commit(smem_u32(&accf[set]));
            ++gw;
          }
          umma_commit(smem_u32(&cfree[st]));
        }
      }
      if (!ok) *abort = 1;
      // Every MMA of this thread completes before tensor memory is freed.
      umma_commit(smem_u32(&fin));
      mbar_wait_bounded(smem_u32(&fin), 0);
    }
    __syncwarp();
  } else if (warp >= 2 && warp < 8) {
    // ---------------------------------------------------------------- converters
    const int ct = tid - 64;
    bool ok = true;
    int gc = 0;
    for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
      int b;
      uint64_t m0, n0;
      tm.decode(t, b, m0, n0, BN);
      const float fa = pow2f(op_shift(jd.a, b)), fb = pow2f(op_shift(jd.b, b));
      for (int c = 0; c < nchunks; ++c, ++gc) {
        const int cs = gc % NS, cu = gc / NS;
        const bool got = mbar_wait_or_abort(smem_u32(&full[cs]), cu & 1, abort, jd.wait_cycles);
        if (!__all_sync(0xffffffffu, got)) {  // warp-uniform exit
          *abort = 1;
          ok = false;
          break;
        }
        // In place: each thread reads its 16-byte pieces of the loaded chunk and
        // writes hi over them and lo into the stage's lo buffer.
        unsigned char* hi = smem + cs * L::CONV;
        unsigned char* lo = hi + L::RAW;
        // 16-byte pieces of a row the chunk's MMA k-steps read (two per k-step
        // of 8); the rest (K past the end) is neither read nor converted.
        const int live = 2 * min(4, ksteps - 4 * c);
#pragma unroll 4
        for (int e = ct; e < L::RAW / 16; e += kConv) {
          // 128-byte swizzle: piece p of row r holds logical piece p ^ (r % 8)
          if (live < 8 && (((e & 7) ^ ((e >> 3) & 7)) >= live)) continue;
          const float4 x = *reinterpret_cast<const float4*>(hi + e * 16);
          float4 h, l;
          split4(x, e * 16 < L::A_BYTES ? fa : fb, h, l);
          *reinterpret_cast<float4*>(hi + e * 16) = h;
          *reinterpret_cast<float4*>(lo + e * 16) = l;
        }
        fence_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&conv[cs]));
      }
    }
  } else if (warp >= 8) {
    // ---------------------------------------------------------------- read-out + epilogue
    const int q = warp & 3, hf = (warp - 8) >> 2, rt = tid - 256;
    const int row = 32 * q + lane;
    const int col0 = hf * HALF;
    const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)col0;
    // Staged float4 stores when the tile's two lowest n bits are the output's
    // two lowest address bits (four columns form one 16-byte vector); the
    // vectors of a row are then placed through the column offset table.
    const bool rowmajor = jd.nb >= 2 && jd.c_s_n[0] == 1 && jd.c_s_n[1] == 2;
    float4* wst = reinterpret_cast<float4*>(smem + NS * L::CONV) + (warp - 8) * 256;  // 32 rows x 8 float4
    int gw = 0;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
      int b;
      uint64_t m0, n0;
      tm.decode(t, b, m0, n0, BN);
      float acc[HALF];
#pragma unroll
      for (int j = 0; j < HALF; ++j) acc[j] = 0.f;
      if constexpr (PAIRS) {
        // Long K: windows are read in pairs and added to each other before
        // they are added into the running sum, halving the rounding steps of
        // the long FP32 accumulation.
        for (int w = 0; w < nwin;) {
          const bool two = w + 1 < nwin;
          const int set0 = gw % NSETS, set1 = (gw + 1) % NSETS;
          const bool got = mbar_wait_or_abort(smem_u32(&accf[set0]), (gw / NSETS) & 1, abort, jd.wait_cycles) &&
                           (!two || mbar_wait_or_abort(smem_u32(&accf[set1]), ((gw + 1) / NSETS) & 1, abort, jd.wait_cycles));
          if (!__all_sync(0xffffffffu, got)) {
            *abort = 1;
            break;
          }
          tc_fence_after();
#pragma unroll
          for (int col = 0; col < HALF; col += 16) {
            float v0[16], v1[16];
            tmem_ld16(tl + (uint32_t)(set0 * BN + col), v0);
            if (two) tmem_ld16(tl + (uint32_t)(set1 * BN + col), v1);
            tmem_ld_wait();
#pragma unroll
            for (int j = 0; j < 16; ++j) acc[col + j] += two ? v0[j] + v1[j] : v0[j];
          }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) {
            mbar_arrive(smem_u32(&acce[set0]));
            if (two) mbar_arrive(smem_u32(&acce[set1]));
          }
          w += two ? 2 : 1;
          gw += two ? 2 : 1;
        }
      } else {
        for (int w = 0; w < nwin; ++w, ++gw) {
          const int set = gw % NSETS;
          if (!__all_sync(0xffffffffu, mbar_wait_or_abort(smem_u32(&accf[set]), (gw / NSETS) & 1, abort, jd.wait_cycles))) {
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
          __syncwarp();
          if (lane == 0) mbar_arrive(smem_u32(&acce[set]));
        }
      }
      if (__any_sync(0xffffffffu, *abort != 0)) break;  // warp-uniform
      const int mlim = (int)min((int64_t)kBM, M - (int64_t)m0);
      const int nlim = (int)min((int64_t)BN, N - (int64_t)n0);
      // Fused root (dot): this join's output is consumed only by the count's
      // final dot product with Y, stored at the same addresses.  Instead of
      // storing, the epilogue reads Y at those addresses and forms the products
      // in four FP32 chains per lane; the warp adds the lanes' sums in FP64 in
      // a fixed order and writes one partial per warp and tile (the root kernel
      // adds them in order: the same bits every run).
      const bool dot = jd.dot_y != nullptr;
      const int64_t at = (int64_t)b * (dot ? jd.dot_y_bs : jd.c_batch_stride) + deposit(jd.c_s_m, m0) +
                         deposit(jd.c_s_n, n0);
      float* __restrict__ C = (float*)jd.c_ptr + at;
      const float* __restrict__ Y = jd.dot_y + at;
      if (dot) {
        // Y is read along the lane's own row, a batch of vectors at a time:
        // every load of a batch is issued before the first product, so their
        // latencies overlap (each 128-byte line is read whole by one lane).
        float s4[4] = {0.f, 0.f, 0.f, 0.f};
        if (row < mlim) {
          const float* __restrict__ Yr = Y + tCm[row];
          if (rowmajor) {
#pragma unroll
            for (int h = 0; h < HALF; h += 32) {
              float4 y[8];
#pragma unroll
              for (int i = 0; i < 8; ++i)
                y[i] = col0 + h + 4 * i < nlim ? __ldg(reinterpret_cast<const float4*>(Yr + tCn[col0 + h + 4 * i]))
                                               : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
              for (int i = 0; i < 8; ++i)
                fma4(make_float4(acc[h + 4 * i], acc[h + 4 * i + 1], acc[h + 4 * i + 2], acc[h + 4 * i + 3]), y[i], s4);
            }
          } else {
#pragma unroll
            for (int h = 0; h < HALF; h += 16) {
              float y[16];
#pragma unroll
              for (int i = 0; i < 16; ++i) y[i] = col0 + h + i < nlim ? __ldg(Yr + tCn[col0 + h + i]) : 0.f;
#pragma unroll
              for (int i = 0; i < 16; ++i) s4[i & 3] = fmaf(acc[h + i], y[i], s4[i & 3]);
            }
          }
        }
        double d = ((double)s4[0] + (double)s4[1]) + ((double)s4[2] + (double)s4[3]);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) d += __shfl_xor_sync(0xffffffffu, d, off);
        const int64_t tis = t & ((1ll << tm.tps_bits) - 1);  // tile within the slice
        if (lane == 0) jd.dot_part[(int64_t)b * jd.dot_part_bs + tis * kReadWarps + (warp - 8)] = d;
        if (m0 == 0 && n0 == 0 && rt == 0)
          jd.c_exp[b] = op_exp(jd.a, b) + op_exp(jd.b, b) - op_shift(jd.a, b) - op_shift(jd.b, b);
        continue;
      }
      // Slice maximum of the row's entries: a running fmaxf from +0 (negative
      // and NaN entries count as 0), whose IEEE bits order like its value.
      float mx = 0.f;
      if (row < mlim) {
        if (col0 + HALF <= nlim) {
#pragma unroll
          for (int j = 0; j < HALF; ++j) mx = fmaxf(mx, acc[j]);
        } else {
#pragma unroll
          for (int j = 0; j < HALF; ++j)
            if (col0 + j < nlim) mx = fmaxf(mx, acc[j]);
        }
      }
      uint32_t bits = __float_as_uint(mx);
      if (rowmajor && jd.c_direct) {
        // Each lane stores its own row's 16-byte vectors: the host chose this
        // when consecutive rows lie close together in the output, so one
        // instruction's 32 vectors fall in a few lines.
        if (row < mlim) {
          const int64_t crow = tCm[row];
#pragma unroll
          for (int j = 0; j < HALF; j += 4)
            if (col0 + j < nlim)
              *reinterpret_cast<float4*>(C + crow + tCn[col0 + j]) =
                  make_float4(acc[j], acc[j + 1], acc[j + 2], acc[j + 3]);
        }
      } else if (rowmajor) {
        // 32 columns at a time through this warp's staging area: each lane
        // writes its row's eight float4, then one store instruction covers four
        // rows of eight vectors -- whole 128-byte segments when the first five
        // n bits are contiguous (float4 slots XOR-swizzled by the row).
#pragma unroll
        for (int p = 0; p < HALF; p += 32) {
#pragma unroll
          for (int j = 0; j < 8; ++j)
            wst[lane * 8 + (j ^ (lane & 7))] =
                make_float4(acc[p + 4 * j], acc[p + 4 * j + 1], acc[p + 4 * j + 2], acc[p + 4 * j + 3]);
          __syncwarp();
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            const int r = (lane >> 3) + 4 * k, c = lane & 7, gr = 32 * q + r;
            if (gr < mlim && col0 + p + 4 * c < nlim)
              *reinterpret_cast<float4*>(C + tCm[gr] + tCn[col0 + p + 4 * c]) = wst[r * 8 + (c ^ (r & 7))];
          }
          __syncwarp();
        }
      } else if (row < mlim) {
        const int64_t crow = tCm[row];
#pragma unroll
        for (int j = 0; j < HALF; ++j)
          if (col0 + j < nlim) C[crow + tCn[col0 + j]] = acc[j];
      }
      for (int off = 16; off > 0; off >>= 1) bits = max(bits, __shfl_xor_sync(0xffffffffu, bits, off));
      if (lane == 0 && bits) atomicMax(&jd.c_max[b], bits);
      if (m0 == 0 && n0 == 0 && rt == 0)
        jd.c_exp[b] = op_exp(jd.a, b) + op_exp(jd.b, b) - op_shift(jd.a, b) - op_shift(jd.b, b);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) tmem_dealloc(tmem, kCols);
  if (tid == 0 && abort_sh && jd.err) atomicExch(jd.err, 1);
}

template <int BN, int NS, bool PAIRS>
cudaError_t launch_ws(const JoinDesc& jd, const CUtensorMap& ta, const CUtensorMap& tb, int nslices,
                      cudaStream_t st) {
  using L = WsSmem<BN, NS>;
  cudaError_t e = cudaFuncSetAttribute(k_umma_ws<BN, NS, PAIRS>, cudaFuncAttributeMaxDynamicSharedMemorySize, L::DYN);
  if (e != cudaSuccess) return e;
  constexpr int bn_bits = BN == 128 ? 7 : 6;
  TileMap tm;
  const int tm_bits = jd.mb > 7 ? jd.mb - 7 : 0;
  tm.tn_bits = jd.nb > bn_bits ? jd.nb - bn_bits : 0;
  tm.tps_bits = tm_bits + tm.tn_bits;
  if (tm.tps_bits != umma_ws_tile_bits(jd.mb, jd.nb)) return cudaErrorInvalidValue;
  if (tm.tps_bits > 40) return cudaErrorInvalidValue;
  const int64_t ntiles = (int64_t)nslices << tm.tps_bits;
  const int64_t grid = ntiles < sm_count() ? ntiles : sm_count();
  k_umma_ws<BN, NS, PAIRS><<<(unsigned)grid, kWsThreads, L::DYN, st>>>(jd, ta, tb, ntiles, tm);
  return cudaGetLastError();
}

}  // namespace

int umma_ws_box_rows_b(int nb) { return nb >= 7 ? 128 : 64; }

int umma_ws_tile_bits(int mb, int nb) {
  const int bn_bits = nb >= 7 ? 7 : 6;
  return (mb > 7 ? mb - 7 : 0) + (nb > bn_bits ? nb - bn_bits : 0);
}

cudaError_t launch_umma_ws(const JoinDesc& jd, const CUtensorMap& ta, const CUtensorMap& tb, int nslices,
                           cudaStream_t st) {
  // More than 32 windows of 32 (K > 1024): the paired read-out.
  const bool pairs = jd.kb > 10;
  // Three stages of 64 KB (BN = 128) or four of 48 KB (BN = 64).
  if (jd.nb >= 7)
    return pairs ? launch_ws<128, 3, true>(jd, ta, tb, nslices, st) : launch_ws<128, 3, false>(jd, ta, tb, nslices, st);
  return pairs ? launch_ws<64, 4, true>(jd, ta, tb, nslices, st) : launch_ws<64, 4, false>(jd, ta, tb, nslices, st);
}

}  // namespace togb
