// Internal descriptors shared by the host runtime and the CUDA kernels.
//
// A join of the flattened plan is one batched "deposit GEMM":
//
//     C[b][m, n] = sum_k A[b][m, k] * B[b][n, k]
//
// over the slices b of a chunk.  Every index is binary, so the element of an
// operand at GEMM coordinates (outer, k) lives at
//
//     ptr + slice_offset(b) + sum_i bit_i(outer) * s_outer[i] + sum_i bit_i(k) * s_k[i]
//
// ("deposit" addressing).  That covers any axis permutation of either operand
// without materialising a transpose (the TTGT transposes np.tensordot performs
// in numpy_apis.py:42-43), and leaves are read straight from their unsliced
// parent tensors: a sliced axis contributes `slice_stride` when its group's bit
// of the global slice index is set (SlicedTensor.build, tensor.py:66-68).
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

#define TOGB_MAXBITS 32

// A deposit as bit-field moves: every stride is a power of two, so
// dep(x) = sum_r ((x >> src[r]) & (2^len[r] - 1)) << dst[r] over maximal runs of
// consecutive index bits that land on consecutive address bits.
struct Runs {
  int32_t n;
  int8_t src[TOGB_MAXBITS];
  int8_t len[TOGB_MAXBITS];
  int8_t dst[TOGB_MAXBITS];
};

struct OpDesc {
  const void* ptr;        // device address of element (0,...,0) of slice 0
  int64_t batch_stride;   // elements between consecutive slices in a chunk (0 for leaves)
  int32_t outer_bits;     // log2 of the outer extent (M for A, N for B)
  int32_t k_bits;         // log2 K
  int32_t n_slice_terms;  // leaves: number of sliced axes
  int32_t k_fast;         // loader hint: the operand's smallest stride lies on a k bit
  int32_t leaf_shift;     // split mode, leaves: power-of-two normaliser
  int32_t meta_step;      // split mode: 1 = per-slice exponent/max entries, 0 = one entry for every slice
  int64_t s_outer[TOGB_MAXBITS];
  int64_t s_k[TOGB_MAXBITS];
  int64_t dk[TOGB_MAXBITS];            // dep_k(k+1) - dep_k(k) when bit t is the lowest zero of k
  int32_t slice_shift[TOGB_MAXBITS];   // bit of the global slice index for sliced axis j
  int64_t slice_stride[TOGB_MAXBITS];
  const int32_t* exp_ptr;    // split mode, intermediates: exponent, entry b * meta_step for slice b
  const uint32_t* max_ptr;   // split mode, intermediates: max bits, entry b * meta_step for slice b
  const void* ptr_lo;        // split mode, leaves: FP32 residual (value - hi), same layout
  Runs r_outer;              // run form of s_outer
  Runs r_k;                  // run form of s_k
  int32_t ktab[16];          // dep_k(k) for k < min(K, 16)
};

struct JoinDesc {
  OpDesc a, b;
  int32_t mb, nb, kb;  // log2 M, N, K
  int32_t join;        // index of this join in post-order
  void* c_ptr;
  int64_t c_batch_stride;
  int64_t c_s_m[TOGB_MAXBITS];
  int64_t c_s_n[TOGB_MAXBITS];
  int32_t* c_exp;      // split mode: per-slice exponent of the output
  uint32_t* c_max;     // split mode: per-slice max bits of the output (zeroed before the join)
  Runs r_cm, r_cn;     // run forms of c_s_m / c_s_n
  int32_t c_natural;   // output stored C[m][n] row-major, slices contiguous: address = linear index
  Runs r_inv_m, r_inv_n;  // output address bits -> m / n bits (inverse deposit of c_s_m / c_s_n)
  int32_t* err;        // device error word: set to 1 when a bounded wait gives up (may be null)
  int64_t wait_cycles; // SM clock cycles a pipeline wait may last before the kernel gives up
  int32_t c_direct;    // tensor-core epilogue: store each row's 16-byte vectors straight from
                       // registers instead of through shared-memory staging (host's choice)
  int32_t pad_;
  // Root fused into this tensor-core join (split form): instead of storing its
  // output C, the epilogue forms sum C[a] * Y[a] over its tile (Y: the root's
  // other operand, stored at the same addresses) and writes one FP64 partial
  // per read-out warp and tile.  Null dot_y: the ordinary epilogue.
  const float* dot_y;  // Y of slice 0 of the chunk
  int64_t dot_y_bs;    // elements of Y between slices (0 when Y is shared by every slice)
  double* dot_part;    // slice b's partials at dot_part + b * dot_part_bs, tile t's warp w at t * 8 + w
  int64_t dot_part_bs;
  // Residue form: words are residues modulo mod_p (below 2^28);
  // mod_m = floor((2^64 - 1) / mod_p) for Barrett reduction.  Zero otherwise.
  uint64_t mod_p, mod_m;
};

// Root reduction: adds every slice's root tensor into the compensated FP64
// accumulator, entry e of the result in the reference's axis order.
struct RootDesc {
  OpDesc r;            // outer bits = root entries in reference order
  double* acc_sum;
  double* acc_comp;
  // Fused root (a count whose dot product was formed in the epilogue of the
  // tensor-core join producing its right operand): slice b's value is
  // 2^(px_exp[b] + py_exp[b * py_step]) times the sum of the npart FP64
  // partials at part + b * part_stride, which the root kernel then writes over
  // the slice's first partial.  `done` counts the root kernel's finished CTAs
  // (zero between launches).  Null part: read the root tensor.
  double* part;
  uint32_t* done;
  int64_t part_stride;
  const int32_t* px_exp;
  const int32_t* py_exp;
  int32_t npart;
  int32_t py_step;
  uint64_t mod_p, mod_m;  // residue form: the modulus and its Barrett constant
};

namespace togb {

// Default limit of a device-side wait: about one second at 2 GHz.
constexpr int64_t kDefaultWaitCycles = 2000000000ll;

enum Kernel { K_DIRECT = 0, K_TILED = 1, K_REDUCE = 2, K_UMMA = 3 };

// Host helper: run form of a stride table (strides must be powers of two).
void make_runs(const int64_t* s, int nbits, Runs* out);
// Host helper: runs mapping the output address bits owned by one GEMM index
// (strides s[0..nbits)) back to that index's bits.
void make_inverse_runs(const int64_t* s, int nbits, Runs* out);

// Fused slice-invariant joins: one launch runs a topologically ordered list
// of thread-per-output joins.  Each join's outputs are cut into tiles of
// kOnceTile; CTAs claim tiles in list order from a global counter and, before
// computing a tile, wait (bounded) until every tile of the joins it reads has
// been published.  A CTA only ever waits for tiles claimed before its own, by
// CTAs that are running, so the launch needs no co-residency.
constexpr int kOnceTile = 1024;  // outputs per tile (256 threads x 4)
// The fields of a JoinDesc a fused join needs (slice-invariant joins read no
// slice offsets), small enough to be copied to shared memory per tile.
struct OnceJoin {
  const void* a;
  const void* b;
  const float* a_lo;         // split form, leaves: residual planes (or null)
  const float* b_lo;
  void* c;
  const uint32_t* a_max;     // split form, intermediates: max bits (null for leaves)
  const uint32_t* b_max;
  const int32_t* a_exp;
  const int32_t* b_exp;
  int32_t* c_exp;
  uint32_t* c_max;
  int32_t a_shift, b_shift;  // split form, leaves: power-of-two normaliser
  int32_t mb, nb, kb, natural;
  int32_t a_ktab[16], b_ktab[16];
  Runs a_outer, b_outer, a_k, b_k, inv_m, inv_n;
  uint64_t mod_p, mod_m;     // residue form: the modulus and its Barrett constant
};
struct OnceList {
  const OnceJoin* joins;     // device [n]
  const int32_t* tile_join;  // device [total_tiles]: list index of each tile's join
  const int32_t* tile_first; // device [n + 1]: first tile of each join
  const int32_t* deps;       // device [2n]: list index of the A / B producer within the list, or -1
  int32_t n;
  int32_t total_tiles;
  uint32_t* counters;        // device [1 + n]: next tile, then published tiles per join (zero before the launch)
  int32_t* err;              // set when a wait expires
  int64_t wait_cycles;       // SM clock cycles a producer wait may last before the CTA gives up
};
cudaError_t launch_once_list(int mode, const OnceList& ol, cudaStream_t st);

// Streaming multiprocessors of the current device (cached per device).
constexpr int kMaxDevices = 256;
int sm_count();
// Which thread-per-output variant a K_DIRECT join runs: 0 k_direct,
// 1 k_direct_staged, 2 k_stream (m-fast A), 3 k_stream (k-fast A).
int direct_variant(int mode, const JoinDesc& jd);
// Launchers (togb_kernels.cu).  `s0` points at the global index of the first
// slice of the chunk; `nslices` is the number of slices in the chunk.
cudaError_t launch_join(int mode, int kernel, const JoinDesc& jd, const int64_t* s0, int nslices,
                        cudaStream_t st);
cudaError_t launch_root(int mode, const RootDesc& rd, const int64_t* s0, int nslices, cudaStream_t st);
// Split-form GEMM on the tensor cores (togb_umma.cu): 3xTF32, TMEM accumulators.
// `ta`/`tb` are TMA maps of plain K-major operands (k, row, slice), or null to
// gather through the deposit layouts.
cudaError_t launch_umma(const JoinDesc& jd, const CUtensorMap* ta, const CUtensorMap* tb, const int64_t* s0,
                        int nslices, cudaStream_t st);
// Warp-specialised tensor-core GEMM over TMA-loaded operands (togb_umma_ws.cu).
cudaError_t launch_umma_ws(const JoinDesc& jd, const CUtensorMap& ta, const CUtensorMap& tb, int nslices,
                           cudaStream_t st);
// Rows of the B-operand TMA box of launch_umma_ws for an N of 2^nb.
int umma_ws_box_rows_b(int nb);
// log2 of the output tiles per slice launch_umma_ws cuts a 2^mb x 2^nb join into.
int umma_ws_tile_bits(int mb, int nb);
cudaError_t launch_set_s0(int64_t* d_s0, int64_t value, cudaStream_t st);
// One leaf to materialise on the device (togb_program_create_compact).
struct LeafBuild {
  int64_t off;         // element offset of the leaf in the leaf arrays
  int32_t rank;
  int32_t kind;        // togb_leaf_kind
  int32_t out_pos;     // clause: index bit of the gate output axis, -1 if none
  uint32_t false_idx;  // clause: index of the all-false corner
  double w_neg, w_pos; // variable weights
};
// Fill the FP64 values and the FP32 hi/lo split of every listed leaf.
cudaError_t launch_build_leaves(const LeafBuild* items, int n, double* v64, float* v32, float* v32lo,
                                cudaStream_t st);
// The int form's leaf words: out[i] = the int64 value of v64[i] rounded toward zero.
cudaError_t launch_leaf_int(const double* v64, void* out, int64_t n, cudaStream_t st);
// The residue form's leaf words: that int64 value modulo p, in [0, p).
cudaError_t launch_leaf_mod(const double* v64, void* out, int64_t n, uint64_t p, cudaStream_t st);
// out[e] = acc[e] + acc[E + e]: the compensated sum of a root accumulator.
cudaError_t launch_finalize(const double* acc, int64_t E, double* out, cudaStream_t st);
cudaError_t probe_peak(int kind, cudaStream_t st, double* flops);
// Tensor-pipe throughput of tcgen05 kind::tf32 MMAs (togb_umma.cu).
cudaError_t probe_umma(cudaStream_t st, double* flops);

}  // namespace togb

#include "togb.h"

namespace togb {

// FP64 contraction of a whole program inside `scratch` (togb_runtime.cpp).
togb_status static_contract_f64(const togb_program_desc* d, const double* d_leaf, char* scratch,
                                size_t scratch_bytes, double* d_out, cudaStream_t st);
// Record `msg` as the calling thread's last error and return `st`.
togb_status report(togb_status st, const char* msg);

}  // namespace togb
