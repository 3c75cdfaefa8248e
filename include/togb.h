/*
 * togb.h -- C ABI of the GB300 contraction backend for TensorOrder.
 *
 * The entry points replace the Execution stage of a TensorOrder plan:
 *
 *   togb_program_create / togb_program_run / togb_program_result
 *       replace BaseTensorAPI.contract_sliced
 *       (src/tensor_network/tensor_apis/base_api.py:17-28), which loops over
 *       slices (TensorNetwork.slice_groups, src/tensor_network/tensor_network.pyx:363-401),
 *       contracts each slice with TensorNetwork.identify
 *       (src/tensor_network/tensor_network.pyx:142-156) and sums result[()]
 *       in FP64.  The caller passes the plan flattened by the host side
 *       (leaves, post-order tokens, slice groups); the library does the rest.
 *   togb_tensordot_f64
 *       replaces NumpyAPI.tensordot (src/tensor_network/tensor_apis/numpy_apis.py:42-43)
 *       and TensorFlowAPI.tensordot (src/tensor_network/tensor_apis/tensorflow_apis.py:99-102)
 *       for binary-index tensors already resident on the device.
 *
 * All pointers are plain host or device pointers; no framework types cross
 * this boundary.  Every call returns a togb_status; togb_last_error() gives a
 * message for the calling thread's most recent failure.  TOGB_ERR_OOM maps to
 * the reference's OutOfMemoryError (base_api.py:4), whose handler re-slices
 * the plan and retries (src/execution.py:134-142).
 */
#ifndef TOGB_H
#define TOGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  TOGB_OK = 0,
  TOGB_ERR_INVALID = 1,     /* malformed program or argument            */
  TOGB_ERR_OOM = 2,         /* device allocation failed / workspace too small */
  TOGB_ERR_CUDA = 3,        /* CUDA runtime error                         */
  TOGB_ERR_UNSUPPORTED = 4, /* valid input outside what the kernels cover */
  TOGB_ERR_TIMEOUT = 5      /* a device-side wait ran out of its budget   */
} togb_status;

typedef enum {
  TOGB_MODE_F64 = 0,   /* plain form: FP64 storage and arithmetic          */
  TOGB_MODE_SPLIT = 1, /* chosen form: FP32 storage with a per-slice power-of-two
                          exponent per tensor; FP64 only in the slice sum  */
  TOGB_MODE_INT64 = 2, /* int form: 64-bit integer storage and arithmetic
                          modulo 2^64, the reference's "int" and "uint"
                          entry types (numpy int64 / uint64,
                          src/tensor_network/tensor_apis/numpy_apis.py:15-22).
                          Leaf values are converted toward zero.  Read the
                          result with togb_program_result_u64.        */
  TOGB_MODE_MOD = 3    /* residue form: the int form's integers modulo the
                          program's modulus (togb_program_set_modulus, below
                          2^28), for exact counts by the Chinese remainder
                          theorem (the reference's "bigint" entry type).
                          Read the result with togb_program_result_u64. */
} togb_mode;

typedef struct togb_program togb_program;

/* A flattened plan.  Leaf i has leaf_rank[i] axes whose edge ids follow in
 * leaf_axes (the tensor's index_list order); its values are the 2^rank FP64
 * entries of the unsliced tensor, row-major in that axis order, concatenated
 * in leaf_values.  postorder holds a leaf index (push) or -1 (pop right, pop
 * left, push their tensordot).  Slice group g lists group_size[g] edge ids in
 * group_edges; slice s fixes the edges of group g to bit (num_groups-1-g) of s,
 * which is itertools.product order over the groups. */
typedef struct {
  int32_t num_leaves;
  const int32_t* leaf_rank;
  const int32_t* leaf_axes;
  const double* leaf_values;
  int32_t num_tokens;
  const int32_t* postorder;
  int32_t num_groups;
  const int32_t* group_size;
  const int32_t* group_edges;
} togb_program_desc;

/* Joins whose subtree reads no sliced edge compute the same tensor for every
 * slice; they run once per togb_program_run call ("once" joins) and every
 * slice reads their output.  The other joins run for every slice. */
typedef struct {
  int64_t num_slices;
  int32_t num_joins;
  int32_t max_rank;              /* largest tensor rank over unsliced axes     */
  int32_t root_rank;             /* rank of the final tensor (0 for a count)   */
  int32_t num_launches;          /* kernel launches per chunk of slices        */
  double flops_per_slice;        /* per-slice joins: sum of 2*M*N*K            */
  double bytes_per_slice_f64;    /* per-slice joins: sum of 8*(M*K + K*N + M*N) */
  int64_t workspace_per_slice[4];/* workspace bytes per slice, by togb_mode    */
  int64_t workspace_fixed[4];    /* workspace bytes independent of slice count */
  int32_t num_joins_once;        /* slice-invariant joins                      */
  int32_t pad_;
  double flops_once;             /* slice-invariant joins: sum of 2*M*N*K      */
  double bytes_once_f64;         /* slice-invariant joins: sum of 8*(M*K+K*N+M*N) */
} togb_program_info;

/* Lower and plan a program for `device`; copies the leaves to the device. */
togb_status togb_program_create(const togb_program_desc* desc, int device, togb_program** out);

/* Leaves of the two CNF tensor kinds described by their parameters, so the
 * library builds their values on the device instead of receiving them:
 *   TOGB_LEAF_CLAUSE    OrTensor.build (tensor_network_constructions.py:69-99):
 *                       all ones except 0 at the all-false corner; with a
 *                       factored gate output axis (output_index >= 0) the
 *                       output axis's false value is 0 except at the
 *                       all-false corner, whose output-flipped neighbour is 0;
 *   TOGB_LEAF_VARIABLE  VariableTensor.build (:144-152): w_neg at all-zeros,
 *                       w_pos at all-ones, 0 elsewhere (rank 0: w_neg + w_pos);
 *   TOGB_LEAF_DENSE     values given in desc->leaf_values.
 * `positive` has bit a set when axis a's literal is positive. */
typedef enum { TOGB_LEAF_DENSE = 0, TOGB_LEAF_CLAUSE = 1, TOGB_LEAF_VARIABLE = 2 } togb_leaf_kind;
typedef struct {
  int32_t kind;
  int32_t output_index;
  uint32_t positive;
  int32_t pad_;
  double w_neg, w_pos;
} togb_leaf_spec;

/* togb_program_create with compact leaves: specs[i] describes leaf i;
 * desc->leaf_values holds only the dense leaves' values, concatenated in leaf
 * order (may be NULL when no leaf is dense).  Clause and variable leaves are
 * materialised by a kernel on `device`. */
togb_status togb_program_create_compact(const togb_program_desc* desc, const togb_leaf_spec* specs, int device,
                                        togb_program** out);

/* New leaf values for a program made by togb_program_create_compact, for
 * counting the same network again with other weights: specs[i] describes
 * leaf i (same kind as at creation; clause polarities and variable weights may
 * change) and dense_values the dense leaves' values in leaf order
 * (num_dense_values of them).  The copies and the device build of clause and
 * variable leaves are queued on `stream`; runs queued after them on that
 * stream see the new leaves.  The lowering, layouts and workspaces are kept;
 * when a leaf's power-of-two normaliser changes, the descriptors and captured
 * graphs are rebuilt at the next run.  Validation as at creation:
 * TOGB_ERR_INVALID for a changed kind or a wrong value count,
 * TOGB_ERR_UNSUPPORTED for negative or non-finite values.  No counterpart in
 * the reference, which rebuilds its tensors for every count
 * (tensor_network_constructions.py:69-152). */
togb_status togb_program_set_leaves(togb_program* prog, const togb_leaf_spec* specs, const double* dense_values,
                                    int64_t num_dense_values, void* stream);

togb_status togb_program_info_get(const togb_program* prog, togb_program_info* info);

/* Lower and plan a program on the host only (no device, no leaf values
 * needed), for inspecting the plan: togb_program_info_get,
 * togb_program_joins, togb_program_kernel_allowed and togb_program_describe
 * work on it; running it does not.  Destroy with togb_program_destroy. */
togb_status togb_program_create_host(const togb_program_desc* desc, togb_program** out);
/* Text description of join `join` in `mode`: GEMM extents, kernel, operand
 * and output strides and their bit runs.  A host-only program is lowered for
 * `mode` on demand; a device program is described as its last run in `mode`
 * lowered it (TOGB_ERR_UNSUPPORTED before such a run), including whether the
 * root's dot product is formed in its operand's epilogue. */
togb_status togb_program_describe(togb_program* prog, int mode, int32_t join, char* buf, size_t n);

/* Zero the device-side slice accumulator (compensated FP64 sum, or the int
 * forms' words).  Runs between two resets must use forms of one kind: FP64
 * and split runs add FP64 sums, int-form runs add 64-bit words, residue-form
 * runs add residues of one modulus (TOGB_ERR_INVALID otherwise). */
togb_status togb_program_reset(togb_program* prog, void* stream);

/* Contract slices [slice_begin, slice_end) in `mode` and add them into the
 * accumulator.  `workspace` is device memory of `workspace_bytes`; when NULL
 * the program allocates (and keeps) its own.  Slices are processed in chunks
 * that fit the workspace.  Work is queued on `stream` (a cudaStream_t, NULL =
 * legacy default stream); the call returns without waiting for it. */
togb_status togb_program_run(togb_program* prog, int mode, int64_t slice_begin, int64_t slice_end,
                             void* workspace, size_t workspace_bytes, void* stream);

/* Wait for `stream` and copy the accumulated root tensor (2^root_rank
 * entries, row-major in the reference's output axis order) to host `out`,
 * together with the compensation terms (`comp`, may be NULL). */
togb_status togb_program_result(togb_program* prog, void* stream, double* out, double* comp, int64_t n);

/* The int forms' result: wait for `stream` and copy the accumulated root
 * tensor (2^root_rank 64-bit words: the sums modulo 2^64, to be read as int64
 * or uint64, or their residues modulo the program's modulus) to host `out`.
 * TOGB_ERR_INVALID when the accumulator holds FP64 sums. */
togb_status togb_program_result_u64(togb_program* prog, void* stream, uint64_t* out, int64_t n);

/* The residue form's modulus, in [2, 2^28).  Runs in TOGB_MODE_MOD compute
 * modulo it; changing it rebuilds that form's descriptors at its next run.
 * Between two resets every residue-form run must use the same modulus. */
togb_status togb_program_set_modulus(togb_program* prog, uint64_t modulus);

/* Per join in post-order, five int32: log2 M, log2 N, log2 K over unsliced
 * axes, the kernel used in `mode` (0 thread-per-output, 1 tiled SIMT GEMM,
 * 2 CTA-per-output reduction, 3 tensor-core GEMM), and 1 when the join runs
 * for every slice or 0 when it runs once per call.  n = num_joins. */
togb_status togb_program_joins(const togb_program* prog, int mode, int32_t* out, int32_t n);

/* Kernel launches of one count in `mode` with the descriptors of the last
 * togb_program_run: the slice-invariant phase (one per fused list of
 * thread-per-output joins and one per other join), then per chunk of slices
 * the slice-base update, every per-slice join and the root reduction.  Before
 * any run (and for host-only programs) the phase as a run would queue it, with
 * all slices in one chunk.  No counterpart in the reference. */
togb_status togb_program_launch_count(const togb_program* prog, int mode, int64_t* launches);

/* Choose the kernel of join `join` in `mode` (kernel ids as in
 * togb_program_joins; -1 restores the default).  A kernel that cannot run the
 * join in that form -- the split form's leaf residuals are applied only by the
 * thread-per-output and reduction kernels, the tensor-core kernel needs
 * M, N >= 32 and K >= 4 -- is rejected with TOGB_ERR_UNSUPPORTED.  The count
 * does not depend on the choice beyond the form's tolerance; only the speed
 * does.  No counterpart in the reference (numpy_apis.py:42-43 always calls
 * np.tensordot). */
togb_status togb_program_set_kernel(togb_program* prog, int mode, int32_t join, int32_t kernel);
/* *allowed = 1 when togb_program_set_kernel would accept the choice. */
togb_status togb_program_kernel_allowed(const togb_program* prog, int mode, int32_t join, int32_t kernel,
                                        int32_t* allowed);

/* Limit, in SM clock cycles, of every device-side wait of this program's
 * kernels: a fused slice-invariant list waiting for a producer tile published
 * by another CTA of the same launch, and the tensor-core joins' load / MMA /
 * read-out pipeline waits.  A wait that runs out sets the program's error
 * word and its kernel returns; togb_program_result then reports
 * TOGB_ERR_TIMEOUT (and clears the word, so the next run starts clean).
 * cycles <= 0 restores the default, 2e9 (about one second at 2 GHz).  The
 * reference has no device waits; its only timeout is the host-side SIGALRM of
 * util.TimeoutTimer (src/util/util.py:13-122). */
togb_status togb_program_set_wait_limit(togb_program* prog, int64_t cycles);

/* Per-join device time of the last run with togb_program_set_timing(prog, 1):
 * `ms[j]` for each join in post-order (n = num_joins). */
togb_status togb_program_set_timing(togb_program* prog, int enable);
togb_status togb_program_join_times(togb_program* prog, float* ms, int32_t n);

void togb_program_destroy(togb_program* prog);

/* out = np.tensordot(a, b, (axes_a, axes_b)) for binary-index FP64 tensors on
 * the device (every dimension 2).  `out` must hold 2^(rank_a+rank_b-2*n_axes)
 * doubles; its axes are a's free axes in order, then b's.  Asynchronous on
 * `stream`. */
togb_status togb_tensordot_f64(const double* a, int32_t rank_a, const double* b, int32_t rank_b,
                               int32_t n_axes, const int32_t* axes_a, const int32_t* axes_b,
                               double* out, void* stream);

/* The same contraction of int64 tensors with sums and products modulo 2^64,
 * as np.tensordot computes int64 (and, bit for bit, uint64) tensors. */
togb_status togb_tensordot_i64(const int64_t* a, int32_t rank_a, const int64_t* b, int32_t rank_b,
                               int32_t n_axes, const int32_t* axes_a, const int32_t* axes_b,
                               int64_t* out, void* stream);

/* Device throughput probe used for roofline denominators: runs `kind` on
 * every SM (0 = FP64 FMA chains, 1 = FP32 FMA chains, 2 = FP64 mma.sync
 * m8n8k4, 3 = tcgen05.mma kind::tf32 128x256x8) and returns the achieved
 * FLOP/s measured with CUDA events on `stream`. */
togb_status togb_probe_peak(int kind, void* stream, double* flops_per_second);

/* Size of the device scratch array behind togb_contract_static_f64. */
#define TOGB_STATIC_SCRATCH_BYTES (32u << 20)

/* Contract a whole program in FP64 without allocating device memory.  This
 * entry point has no counterpart in the reference.  It serves callers that
 * cannot call cudaMalloc -- processes whose device memory all belongs to their
 * own allocator, or pipelines that cannot afford the device synchronisation
 * cudaMalloc/cudaFree imply.  The caller passes the program (host arrays;
 * desc->leaf_values may be NULL), the leaf values already on the current
 * device (same concatenated layout as desc->leaf_values), and `d_out`, device
 * memory for the 2^root_rank compensated sums over all slices.  Intermediates
 * live in one file-scope device array of TOGB_STATIC_SCRATCH_BYTES (32 MiB),
 * held by every GPU that loads the library until exit; a program that needs
 * more than that for a single slice is rejected with TOGB_ERR_OOM and a message
 * giving both sizes.  The first call in each CUDA context (per device, and
 * again after a cudaDeviceReset) looks up the array's address: make it before
 * any stream capture.  All calls share the array: calls whose work overlaps on
 * the GPU race, so serialise them.  Queued on `stream`. */
togb_status togb_contract_static_f64(const togb_program_desc* desc, const double* d_leaf_values,
                                     double* d_out, void* stream);

/* A batch of programs (instances of uneven size, each with its own plan,
 * slice count and workspace) contracted by one CUDA graph: every program's
 * complete count -- accumulator reset, slice-invariant joins, all chunks of
 * slices -- runs on internal stream i % nstreams, forked from and joined back
 * into the caller's stream.  The programs' kernels (togb_program_set_kernel)
 * and workspaces are fixed when the batch is created; a program may belong
 * to one live batch at a time and must not be run on its own meanwhile.  The
 * reference contracts instances one after another (execution.py:122-152).
 * `mode` is TOGB_MODE_F64 or TOGB_MODE_SPLIT. */
typedef struct togb_batch togb_batch;
togb_status togb_batch_create(togb_program* const* progs, int32_t n, int mode, void* const* workspaces,
                              const size_t* workspace_bytes, int32_t nstreams, togb_batch** out);
/* One step: every program's count, queued on `stream`. */
togb_status togb_batch_run(togb_batch* batch, void* stream);
/* Wait for `stream`; out[i] = count of program i (scalar roots only). */
togb_status togb_batch_results(togb_batch* batch, void* stream, double* out, int32_t n);
void togb_batch_destroy(togb_batch* batch);

/* The learned cost model's network: an MLP F -> H -> H -> 1 (ReLU hidden
 * layers, FP32) on the device.  No counterpart in the reference, whose only
 * cost model is the FLOP/memory estimate of contraction_tree.pyx:382-496.
 * `params` holds togb_mlp_param_count(F, H) floats laid out
 * W1[F][H] b1[H] W2[H][H] b2[H] W3[H] b3; `scratch` holds
 * togb_mlp_scratch_floats(B, H) floats.  All pointers are device memory;
 * every call is queued on `stream`. */
int64_t togb_mlp_param_count(int F, int H);
int64_t togb_mlp_scratch_floats(int B, int H);
/* y[B] = network(x[B][F]). */
togb_status togb_mlp_forward(const float* params, int F, int H, const float* x, int B, float* y, float* scratch,
                             void* stream);
/* grads (same layout as params) of the mean squared error against target[B];
 * *loss (device, may be NULL) receives that error. */
togb_status togb_mlp_loss_grad(const float* params, int F, int H, const float* x, const float* target, int B,
                               float* grads, float* loss, float* scratch, void* stream);
/* One Adam step (bias-corrected, step >= 1) over n parameters. */
togb_status togb_mlp_adam(float* params, const float* grads, float* m, float* v, int64_t n, float lr, float beta1,
                          float beta2, float eps, int32_t step, void* stream);

const char* togb_last_error(void);
int togb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* TOGB_H */
