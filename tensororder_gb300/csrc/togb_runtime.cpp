// Host runtime of the contraction path: lowers a flattened TensorOrder plan,
// plans tensor layouts and a device arena, and queues the per-chunk kernel
// sequence (optionally as a CUDA graph).  Implements include/togb.h.
//
// Lowering follows the reference's execution exactly:
//  * the post-order stack walk of TensorNetwork.identify
//    (src/tensor_network/tensor_network.pyx:142-156);
//  * shared edges / output edge order of compute_join_properties
//    (src/contraction_methods/contraction_tree.pyx:248-288): left unshared
//    edges in order, then right unshared edges in order;
//  * slicing by edge groups in itertools.product order
//    (src/tensor_network/tensor_network.pyx:363-401), with every sliced axis
//    removed from the tensors it touches (it is a size-1 axis in the
//    reference, src/tensor_network/tensor.py:66-68);
//  * the FP64 slice sum of BaseTensorAPI.contract_sliced
//    (src/tensor_network/tensor_apis/base_api.py:21-28), done here with a
//    compensated sum on the device.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "togb.h"
#include "togb_internal.h"

namespace {

thread_local std::string g_err;

togb_status fail(togb_status st, const std::string& msg) {
  g_err = msg;
  return st;
}

togb_status cuda_fail(cudaError_t e, const char* what) {
  cudaGetLastError();
  const togb_status st = (e == cudaErrorMemoryAllocation) ? TOGB_ERR_OOM : TOGB_ERR_CUDA;
  return fail(st, std::string(what) + ": " + cudaGetErrorString(e));
}

#define TOGB_CUDA(x)                                  \
  do {                                                \
    cudaError_t e_ = (x);                             \
    if (e_ != cudaSuccess) return cuda_fail(e_, #x);  \
  } while (0)

constexpr int64_t kAlignElems = 32;  // arena offsets aligned to 32 elements

struct Node {
  int leaf = -1;                 // leaf index, or -1 for a join
  int left = -1, right = -1;     // operand nodes of a join
  int join = -1;                 // post-order index among joins
  std::vector<int> ref;          // unsliced edges in the reference's axis order
  std::unordered_map<int, int64_t> stride;  // unsliced edge -> element stride
  int rank = 0;                  // number of unsliced axes
  std::vector<int> m_lsb, n_lsb, k_lsb;     // GEMM bit order, least significant first
  int64_t off = -1;              // arena offset (elements), joins only
  int kernel = togb::K_DIRECT;
  int kernel_set[4] = {-1, -1, -1, -1}; // per-form kernel chosen by the caller (togb_program_set_kernel), -1 = default
  bool dep = true;               // depends on the slice (reads a sliced leaf, directly or below)
  int slot = -1;                 // joins: index among the joins of its phase (metadata row)
};

int64_t pow2(int r) { return int64_t(1) << r; }

int log2_exact(int64_t v) {
  int l = 0;
  while ((int64_t(1) << l) < v) ++l;
  return l;
}

// Kernel for a join in a given form.  Long-K joins with few outputs get the
// CTA-per-output reduction; GEMM-sized joins (M, N >= 32, K >= 16) the tiled
// kernel, with K-major operands requested from their producers; the rest the
// thread-per-output kernel.  M or N of 32 leaves part of a tile empty, which
// costs little: such joins are bound by their operand and output bytes, while
// a thread-per-output kernel reading operands whose K and free bits are
// interleaved wastes most of every sector it loads.
int choose_kernel(int mb, int nb, int kb) {
  if (kb >= 12 && mb + nb <= 6) return togb::K_REDUCE;
  if (mb >= 5 && nb >= 5 && kb >= 4) return togb::K_TILED;
  return togb::K_DIRECT;
}

}  // namespace

void togb::make_runs(const int64_t* s, int nbits, Runs* out) {
  std::memset(out, 0, sizeof(*out));
  int i = 0;
  while (i < nbits) {
    const int d = log2_exact(s[i]);
    int len = 1;
    while (i + len < nbits && s[i + len] == (s[i] << len)) ++len;
    out->src[out->n] = (int8_t)i;
    out->len[out->n] = (int8_t)len;
    out->dst[out->n] = (int8_t)d;
    ++out->n;
    i += len;
  }
}

void togb::make_inverse_runs(const int64_t* s, int nbits, Runs* out) {
  // (address bit, index bit) pairs sorted by address bit, then merged into runs.
  std::vector<std::pair<int, int>> bits;
  for (int i = 0; i < nbits; ++i) bits.push_back({log2_exact(s[i]), i});
  std::sort(bits.begin(), bits.end());
  std::memset(out, 0, sizeof(*out));
  size_t i = 0;
  while (i < bits.size()) {
    int len = 1;
    while (i + len < bits.size() && bits[i + len].first == bits[i].first + len &&
           bits[i + len].second == bits[i].second + len)
      ++len;
    out->src[out->n] = (int8_t)bits[i].first;
    out->len[out->n] = (int8_t)len;
    out->dst[out->n] = (int8_t)bits[i].second;
    ++out->n;
    i += len;
  }
}

// One step of the slice-invariant phase: a fused OnceList of joins, or one join.
struct OnceSeg {
  bool fused = false;
  std::vector<int> js;  // indices into joins, in execution order
  togb::OnceList ol{};
};

struct togb_program {
  int device = 0;
  int G = 0;
  int64_t num_slices = 1;
  std::vector<Node> nodes;
  int root = -1;
  std::vector<int> joins;  // node ids in execution (post-)order
  // Joins by phase, as indices into `joins`: slice-invariant joins run once per
  // togb_program_run call (their subtrees read no sliced edge, so every slice
  // would compute the same tensor); the rest run for every slice of a chunk.
  std::vector<int> once, per;
  std::unordered_map<int, int> group_of_edge;
  // leaves
  std::vector<int> leaf_rank;
  std::vector<std::vector<int>> leaf_axes;
  std::vector<int64_t> leaf_off;
  std::vector<int> leaf_shift;  // split mode normaliser per leaf
  std::vector<int> leaf_kind;   // togb_leaf_kind of each leaf as created
  double* d_leaf64 = nullptr;
  float* d_leaf32 = nullptr;    // split mode: FP32 rounding of each leaf value
  float* d_leaf32lo = nullptr;  // split mode: value - hi, rounded to FP32
  int64_t num_leaf_values = 0;  // entries of every leaf array
  // Int form: the FP64 leaf values converted toward zero, made from d_leaf64
  // by the first int-form run after the leaves were created or replaced.
  void* d_leaf_int = nullptr;
  bool leaf_int_current = false;
  // Residue form: the same integers modulo `modulus` (togb_program_set_modulus),
  // converted for the modulus in `leaf_mod_p` (0 = not converted).
  void* d_leaf_mod = nullptr;
  uint64_t leaf_mod_p = 0;
  uint64_t modulus = 0;
  // planning
  int64_t arena = 0;       // per-slice elements (slice-dependent joins)
  int64_t arena_once = 0;  // elements of the slice-invariant joins, shared by all slices
  double flops = 0, bytes64 = 0;            // per slice, slice-dependent joins
  double flops_once = 0, bytes64_once = 0;  // once per run, slice-invariant joins
  int max_rank = 0;
  // device state
  double* d_acc = nullptr;  // [2 * 2^root_rank]: sum then compensation (int form: wrapping words, then zeros)
  int acc_kind = 0;         // what the accumulator holds since the last reset: 0 nothing, 1 FP64 sums,
                            // 2 int words, 3 residues modulo acc_modulus
  uint64_t acc_modulus = 0;
  int64_t* d_s0 = nullptr;
  int32_t* d_err = nullptr; // set by a kernel whose bounded wait expired
  int64_t wait_cycles = togb::kDefaultWaitCycles;  // limit of every device-side pipeline wait
  int root_fused = -1;     // index into joins of a root dot product formed in its operand's epilogue
  void* own_ws = nullptr;
  size_t own_ws_bytes = 0;
  // togb_program_set_leaves: device build records and host staging, kept
  // with the program so the copies queued on the caller's stream outlive it.
  togb::LeafBuild* d_items = nullptr;
  size_t d_items_cap = 0;
  std::vector<togb::LeafBuild> h_items;
  std::vector<float> h_hi, h_lo;
  cudaStream_t cap_stream = nullptr;
  // descriptors for the current (mode, chunk, workspace)
  int cur_mode = -1;
  int cur_B = 0;
  const void* cur_ws = nullptr;
  std::vector<JoinDesc> jds;
  std::vector<CUtensorMap> tmaps;  // per join: TMA maps of A and B (tensor-core joins with plain operands)
  std::vector<char> use_tma;
  RootDesc rd{};
  uint32_t* d_max = nullptr;  // split mode max bits [per-slice joins][B] inside the workspace
  size_t max_bytes = 0;
  uint32_t* d_max_once = nullptr;  // split mode max bits [slice-invariant joins]
  size_t max_once_bytes = 0;
  // Fused slice-invariant phase: runs of consecutive thread-per-output joins
  // of `once` become one OnceList launch each (the other joins stay single
  // launches).  Possible when the slice-invariant arena is planned without
  // reuse (no join overwrites an operand another join may still read).
  bool allow_fused_once = true;  // false for the allocation-free entry point
  bool once_no_reuse = false;
  std::vector<OnceSeg> once_segs;
  int once_segs_mode = -1;          // form the segments were built for, -1 = none
  uint32_t* d_once_ctr = nullptr;   // tile counters of every fused segment
  size_t once_ctr_bytes = 0;
  std::vector<void*> once_bufs;     // device copies of the segments' tables (freed with the program)
  std::map<int, cudaGraphExec_t> graphs;  // by chunk slice count
  std::map<int, int> phase_runs;          // launches of each phase key since the last clear
  bool use_graphs = true;
  bool timing = false;
  bool host_only = false;  // lowered for inspection only; owns no device memory
  std::vector<float> join_ms;
};

namespace {

size_t elem_size(int mode) { return mode == TOGB_MODE_SPLIT ? 4 : 8; }

bool known_mode(int mode) {
  return mode == TOGB_MODE_F64 || mode == TOGB_MODE_SPLIT || mode == TOGB_MODE_INT64 || mode == TOGB_MODE_MOD;
}

int64_t round256(int64_t x) { return (x + 255) / 256 * 256; }

// Workspace layout, from a 256-byte aligned base:
//   [slice-invariant arena][slice-invariant exponent + max bits]   (fixed part)
//   [per-slice arena x B][per-slice exponent x B][per-slice max bits x B]
int64_t ws_per_slice(const togb_program* p, int mode) {
  int64_t b = p->arena * (int64_t)elem_size(mode);
  if (mode == TOGB_MODE_SPLIT) b += 8 * (int64_t)p->per.size();  // exponent + max bits
  return b;
}

int64_t ws_once(const togb_program* p, int mode) {
  int64_t b = round256(p->arena_once * (int64_t)elem_size(mode));
  if (mode == TOGB_MODE_SPLIT) b += round256(8 * (int64_t)p->once.size());
  return b;
}

const int64_t kWsSlack = 256;  // alignment slack

int64_t ws_fixed(const togb_program* p, int mode) { return kWsSlack + ws_once(p, mode); }

void clear_graphs(togb_program* p) {
  for (auto& kv : p->graphs) cudaGraphExecDestroy(kv.second);
  p->graphs.clear();
  p->phase_runs.clear();
}

// Bottom-up part of a join's plan: edge sets, reference output order, kernel,
// cost, and a natural layout -- GEMM bit orders following the operands'
// strides (monotone reads) and the output stored C[m][n].  plan_layouts may
// later replace the layout of joins that feed a GEMM-shaped consumer.
void plan_join(togb_program* p, Node& J) {
  const Node& L = p->nodes[J.left];
  const Node& R = p->nodes[J.right];
  std::vector<int> shared, lfree, rfree;
  for (int e : L.ref) {
    if (std::find(R.ref.begin(), R.ref.end(), e) != R.ref.end()) shared.push_back(e);
    else lfree.push_back(e);
  }
  for (int e : R.ref)
    if (std::find(L.ref.begin(), L.ref.end(), e) == L.ref.end()) rfree.push_back(e);
  J.ref = lfree;
  J.ref.insert(J.ref.end(), rfree.begin(), rfree.end());
  J.rank = (int)J.ref.size();
  auto by_stride = [](const Node& X) {
    return [&X](int a, int b) { return X.stride.at(a) < X.stride.at(b); };
  };
  J.m_lsb = lfree;
  std::sort(J.m_lsb.begin(), J.m_lsb.end(), by_stride(L));
  J.n_lsb = rfree;
  std::sort(J.n_lsb.begin(), J.n_lsb.end(), by_stride(R));
  J.k_lsb = shared;
  const Node& big = (L.rank >= R.rank) ? L : R;
  std::sort(J.k_lsb.begin(), J.k_lsb.end(), by_stride(big));
  const int nb = (int)J.n_lsb.size();
  for (int i = 0; i < nb; ++i) J.stride[J.n_lsb[i]] = pow2(i);
  for (size_t i = 0; i < J.m_lsb.size(); ++i) J.stride[J.m_lsb[i]] = pow2(nb + (int)i);
  const int mb = (int)J.m_lsb.size(), kb = (int)J.k_lsb.size();
  J.kernel = choose_kernel(mb, nb, kb);
}

// Top-down layout requests.  A GEMM-shaped join (tiled / tensor-core kernels)
// or a long-K reduction asks for its intermediate operands in [free][shared]
// order with one shared-axis order on both sides, so it reads two row-major
// K-major matrices; the producers then write their outputs in that order (a
// producer's free axes keep their significance from the requested order, so
// its stores follow its loads).  Every other join keeps the natural layout of
// plan_join, which favours the thread-per-output kernel's reads.  A leaf
// operand's layout is its parent tensor's, so it fixes the shared-axis order.
void plan_layouts(togb_program* p) {
  std::vector<std::vector<int>> req(p->nodes.size());  // requested order, most significant first
  std::vector<char> requested(p->nodes.size(), 0);
  auto in = [](const std::vector<int>& v, int e) { return std::find(v.begin(), v.end(), e) != v.end(); };
  for (auto it = p->joins.rbegin(); it != p->joins.rend(); ++it) {
    Node& J = p->nodes[*it];
    std::vector<int> mu, nu;  // most significant first
    if (requested[*it]) {
      const std::vector<int>& sigma = req[*it];
      const int r = (int)sigma.size();
      for (int q = 0; q < r; ++q) J.stride[sigma[q]] = pow2(r - 1 - q);
      for (int e : sigma) {
        if (in(J.m_lsb, e)) mu.push_back(e);
        else nu.push_back(e);
      }
    } else {
      mu.assign(J.m_lsb.rbegin(), J.m_lsb.rend());
      nu.assign(J.n_lsb.rbegin(), J.n_lsb.rend());
    }
    J.m_lsb.assign(mu.rbegin(), mu.rend());
    J.n_lsb.assign(nu.rbegin(), nu.rend());
    if (J.kernel != togb::K_TILED && J.kernel != togb::K_REDUCE) continue;
    const Node& L = p->nodes[J.left];
    const Node& R = p->nodes[J.right];
    std::vector<int> kappa = J.k_lsb;
    const Node* leaf = L.leaf >= 0 ? &L : (R.leaf >= 0 ? &R : nullptr);
    // A GEMM-shaped operand producer writes its tile rows fastest when its
    // column axes are its output's lowest address bits (row-major tiles).  The
    // shared axes sit at the bottom of both operands, so order them for the
    // larger such producer: its column axes first (in its own order), then the
    // rest by its natural strides.
    const Node* fav = nullptr;
    for (const Node* X : {&L, &R})
      if (X->leaf < 0 && X->kernel == togb::K_TILED && (!fav || X->rank > fav->rank)) fav = X;
    if (fav) {
      const bool swapped = fav->m_lsb.size() < 7 && fav->n_lsb.size() > fav->m_lsb.size();
      const std::vector<int>& cols = swapped ? fav->m_lsb : fav->n_lsb;
      std::vector<int> lsb;
      for (int e : cols)
        if (in(kappa, e)) lsb.push_back(e);
      std::vector<int> rest;
      for (int e : kappa)
        if (!in(lsb, e)) rest.push_back(e);
      std::sort(rest.begin(), rest.end(), [fav](int a, int b) { return fav->stride.at(a) < fav->stride.at(b); });
      lsb.insert(lsb.end(), rest.begin(), rest.end());
      kappa.assign(lsb.rbegin(), lsb.rend());  // most significant first
    } else if (leaf) {
      std::sort(kappa.begin(), kappa.end(), [leaf](int a, int b) { return leaf->stride.at(a) > leaf->stride.at(b); });
    } else {
      std::sort(kappa.begin(), kappa.end());
    }
    if (L.leaf < 0) {
      req[J.left] = mu;
      req[J.left].insert(req[J.left].end(), kappa.begin(), kappa.end());
      requested[J.left] = 1;
    }
    if (R.leaf < 0) {
      req[J.right] = nu;
      req[J.right].insert(req[J.right].end(), kappa.begin(), kappa.end());
      requested[J.right] = 1;
    }
    J.k_lsb.assign(kappa.rbegin(), kappa.rend());
  }
}

// First-fit arena over the outputs of one phase's joins, freeing an operand
// after its consumer when both belong to the phase.  A slice-invariant output
// read by a per-slice join stays live for the whole run.
int64_t plan_phase_arena(togb_program* p, bool dep) {
  std::vector<std::pair<int64_t, int64_t>> live;  // (offset, size), sorted by offset
  int64_t top = 0;
  auto alloc = [&](int64_t size) {
    int64_t cur = 0;
    size_t pos = 0;
    for (; pos < live.size(); ++pos) {
      if (live[pos].first - cur >= size) break;
      cur = live[pos].first + live[pos].second;
    }
    live.insert(live.begin() + pos, {cur, size});
    top = std::max(top, cur + size);
    return cur;
  };
  auto release = [&](int64_t off) {
    for (size_t i = 0; i < live.size(); ++i)
      if (live[i].first == off) { live.erase(live.begin() + i); return; }
  };
  for (int id : p->joins) {
    Node& J = p->nodes[id];
    if (J.dep != dep) continue;
    const int64_t size = (pow2(J.rank) + kAlignElems - 1) / kAlignElems * kAlignElems;
    J.off = alloc(size);
    if (!dep && p->once_no_reuse) continue;  // fused slice-invariant phase: every output keeps its place
    for (int opnd : {J.left, J.right}) {
      const Node& O = p->nodes[opnd];
      if (O.leaf < 0 && O.dep == dep) release(O.off);
    }
  }
  return top;
}

void plan_arena(togb_program* p) {
  p->once.clear();
  p->per.clear();
  p->flops = p->bytes64 = p->flops_once = p->bytes64_once = 0;
  for (size_t j = 0; j < p->joins.size(); ++j) {
    Node& J = p->nodes[p->joins[j]];
    std::vector<int>& phase = J.dep ? p->per : p->once;
    J.slot = (int)phase.size();
    phase.push_back((int)j);
    const Node& L = p->nodes[J.left];
    const Node& R = p->nodes[J.right];
    const int kb = (int)J.k_lsb.size();
    const double M = std::ldexp(1.0, L.rank - kb), N = std::ldexp(1.0, R.rank - kb), K = std::ldexp(1.0, kb);
    (J.dep ? p->flops : p->flops_once) += 2.0 * M * N * K;
    (J.dep ? p->bytes64 : p->bytes64_once) += 8.0 * (M * K + K * N + M * N);
  }
  // The slice-invariant outputs keep their places (so the phase can run as
  // fused lists) unless that needs more than 2^24 elements.
  int64_t once_total = 0;
  for (int j : p->once) once_total += (pow2(p->nodes[p->joins[j]].rank) + kAlignElems - 1) / kAlignElems * kAlignElems;
  p->once_no_reuse = p->allow_fused_once && once_total <= (int64_t(1) << 24);
  p->arena = std::max<int64_t>(plan_phase_arena(p, true), kAlignElems);
  p->arena_once = plan_phase_arena(p, false);
}

// dep_k(k) for the first 16 values of k (the unrolled small-K kernels).
void fill_ktab(OpDesc& od) {
  for (int k = 0; k < 16; ++k) {
    int64_t off = 0;
    for (int i = 0; i < od.k_bits; ++i)
      if ((k >> i) & 1) off += od.s_k[i];
    od.ktab[k] = (k < (1 << std::min(od.k_bits, 4))) ? (int32_t)off : 0;
  }
}

// True when C is stored [slice][m][n] row-major, i.e. address = linear index.
int is_natural(const JoinDesc& jd) {
  for (int i = 0; i < jd.nb; ++i)
    if (jd.c_s_n[i] != pow2(i)) return 0;
  for (int i = 0; i < jd.mb; ++i)
    if (jd.c_s_m[i] != pow2(jd.nb + i)) return 0;
  return jd.c_batch_stride == pow2(jd.mb + jd.nb) ? 1 : 0;
}

// Workspace regions for a chunk of B slices (see ws_per_slice / ws_once).
struct WsLayout {
  char* once;             // slice-invariant arena
  int32_t* once_exp;      // [once joins]
  uint32_t* once_max;     // [once joins]
  char* per;              // per-slice arena, node j at per + off * B * es
  int32_t* per_exp;       // [per joins][B]
  uint32_t* per_max;      // [per joins][B]
};

WsLayout ws_layout(const togb_program* p, int mode, char* ws, int B) {
  const int64_t es = (int64_t)elem_size(mode);
  WsLayout w{};
  w.once = ws;
  char* meta = ws + round256(p->arena_once * es);
  w.once_exp = (int32_t*)meta;
  w.once_max = (uint32_t*)(meta + 4 * (int64_t)p->once.size());
  w.per = ws + ws_once(p, mode);
  char* pmeta = w.per + p->arena * (int64_t)B * es;
  w.per_exp = (int32_t*)pmeta;
  w.per_max = (uint32_t*)(pmeta + 4 * (int64_t)p->per.size() * B);
  return w;
}

void fill_operand(const togb_program* p, const Node& X, const std::vector<int>& outer,
                  const std::vector<int>& k, int mode, char* ws, int B, OpDesc& od) {
  std::memset(&od, 0, sizeof(od));
  const size_t es = elem_size(mode);
  const WsLayout w = ws_layout(p, mode, ws, B);
  if (X.leaf >= 0) {
    const char* base = mode == TOGB_MODE_F64     ? (const char*)p->d_leaf64
                       : mode == TOGB_MODE_INT64 ? (const char*)p->d_leaf_int
                       : mode == TOGB_MODE_MOD   ? (const char*)p->d_leaf_mod
                                                 : (const char*)p->d_leaf32;
    od.ptr = base + p->leaf_off[X.leaf] * es;
    od.batch_stride = 0;
    const std::vector<int>& axes = p->leaf_axes[X.leaf];
    const int R = (int)axes.size();
    int nt = 0;
    for (int a = 0; a < R; ++a) {
      auto it = p->group_of_edge.find(axes[a]);
      if (it == p->group_of_edge.end()) continue;
      od.slice_shift[nt] = p->G - 1 - it->second;
      od.slice_stride[nt] = pow2(R - 1 - a);
      ++nt;
    }
    od.n_slice_terms = nt;
    od.leaf_shift = p->leaf_shift[X.leaf];
    if (mode == TOGB_MODE_SPLIT) od.ptr_lo = p->d_leaf32lo + p->leaf_off[X.leaf];
  } else if (X.dep) {
    od.ptr = w.per + X.off * (int64_t)B * es;
    od.batch_stride = pow2(X.rank);
    if (mode == TOGB_MODE_SPLIT) {
      od.exp_ptr = w.per_exp + (int64_t)X.slot * B;
      od.max_ptr = w.per_max + (int64_t)X.slot * B;
      od.meta_step = 1;
    }
  } else {
    // Slice-invariant intermediate: one tensor read by every slice.
    od.ptr = w.once + X.off * (int64_t)es;
    od.batch_stride = 0;
    if (mode == TOGB_MODE_SPLIT) {
      od.exp_ptr = w.once_exp + X.slot;
      od.max_ptr = w.once_max + X.slot;
      od.meta_step = 0;
    }
  }
  od.outer_bits = (int)outer.size();
  od.k_bits = (int)k.size();
  int64_t min_outer = INT64_MAX, min_k = INT64_MAX;
  for (size_t i = 0; i < outer.size(); ++i) {
    od.s_outer[i] = X.stride.at(outer[i]);
    min_outer = std::min(min_outer, od.s_outer[i]);
  }
  int64_t prefix = 0;
  for (size_t i = 0; i < k.size(); ++i) {
    od.s_k[i] = X.stride.at(k[i]);
    min_k = std::min(min_k, od.s_k[i]);
    od.dk[i] = od.s_k[i] - prefix;
    prefix += od.s_k[i];
  }
  od.k_fast = min_k < min_outer ? 1 : 0;
  togb::make_runs(od.s_outer, od.outer_bits, &od.r_outer);
  togb::make_runs(od.s_k, od.k_bits, &od.r_k);
  fill_ktab(od);
}

// Kernel for a join in the split form: GEMM-sized joins of two intermediates
// go to the tensor cores; leaf operands need their FP32 residual, which only
// the CUDA-core kernels apply.
int default_split_kernel(const togb_program* p, const Node& J) {
  const bool leaf = p->nodes[J.left].leaf >= 0 || p->nodes[J.right].leaf >= 0;
  if (J.kernel == togb::K_TILED) return leaf ? togb::K_DIRECT : togb::K_UMMA;
  return J.kernel;
}

// Kernel of a join in a form: the caller's choice if set, else the default.
int join_kernel(const togb_program* p, const Node& J, int mode) {
  if (known_mode(mode) && J.kernel_set[mode] >= 0) return J.kernel_set[mode];
  return mode == TOGB_MODE_SPLIT ? default_split_kernel(p, J) : J.kernel;
}

int split_kernel(const togb_program* p, const Node& J) { return join_kernel(p, J, TOGB_MODE_SPLIT); }

// Kernels a join may run in a form.  Every kernel reads any layout; the
// limits are numerical (the split form's leaf residuals are applied only by
// the thread-per-output and reduction kernels) and launch-size limits.
bool kernel_allowed(const togb_program* p, const Node& J, int mode, int kernel) {
  const int mb = (int)J.m_lsb.size(), nb = (int)J.n_lsb.size(), kb = (int)J.k_lsb.size();
  const bool leaf = p->nodes[J.left].leaf >= 0 || p->nodes[J.right].leaf >= 0;
  switch (kernel) {
    case togb::K_DIRECT: return true;
    case togb::K_REDUCE: return mb + nb <= 20;  // one CTA per output entry and slice
    case togb::K_TILED: return mode != TOGB_MODE_SPLIT || !leaf;
    case togb::K_UMMA: return mode == TOGB_MODE_SPLIT && !leaf && mb >= 5 && nb >= 5 && kb >= 2;
    default: return false;
  }
}

// A split-form intermediate operand stored as a row-major [rows][K] matrix,
// one per slice or one shared by all slices (slice-invariant).  Leaves (read
// from their parent tensors) carry no exponent table and never qualify.
bool plain_k_major(const OpDesc& o) {
  if (!o.exp_ptr) return false;
  for (int i = 0; i < o.k_bits; ++i)
    if (o.s_k[i] != pow2(i)) return false;
  for (int i = 0; i < o.outer_bits; ++i)
    if (o.s_outer[i] != pow2(o.k_bits + i)) return false;
  return o.batch_stride == 0 || o.batch_stride == pow2(o.k_bits + o.outer_bits);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)f;
    cudaGetLastError();
  }
  return fn;
}

// TMA map of a plain FP32 operand: dims (k, row, slice), box (32, box_rows, 1),
// 128-byte swizzle (the K-major SWIZZLE_128B operand layout of tcgen05.mma).
bool make_tmap(const OpDesc& o, int nslices, uint32_t box_rows, CUtensorMap* out) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn) return false;
  const cuuint64_t K = (cuuint64_t)pow2(o.k_bits), R = (cuuint64_t)pow2(o.outer_bits);
  const cuuint64_t dims[3] = {K, R, (cuuint64_t)nslices};
  const cuuint64_t strides[2] = {K * 4, K * R * 4};
  const cuuint32_t box[3] = {32, box_rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  if ((K * 4) % 16 != 0 || ((uintptr_t)o.ptr % 16) != 0) return false;
  return fn(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(o.ptr), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor-core epilogue of a row-major tile (the output's two lowest n bits are
// its two lowest address bits): 1 when each lane should store its own row's
// 16-byte vectors rather than transposing through shared memory.  Counts the
// 128-byte lines one warp's stores of rows 0..31 x columns 0..31 touch both
// ways; the staged path costs about four times the instructions, so the direct
// path is taken while it touches at most twice the lines.
int choose_direct_epilogue(const JoinDesc& jd) {
  if (jd.nb < 2 || jd.c_s_n[0] != 1 || jd.c_s_n[1] != 2) return 0;
  auto dep_bits = [](const int64_t* s, int nbits, int x) {
    int64_t off = 0;
    for (int i = 0; i < nbits; ++i)
      if ((x >> i) & 1) off += s[i];
    return off;
  };
  const int rows = std::min(32, 1 << jd.mb), cols = std::min(32, 1 << jd.nb);
  int64_t direct = 0, staged = 0;
  for (int j = 0; j < cols; j += 4) {  // direct: instruction j stores column group j of every row
    std::vector<int64_t> lines;
    for (int r = 0; r < rows; ++r) lines.push_back((dep_bits(jd.c_s_m, jd.mb, r) + dep_bits(jd.c_s_n, jd.nb, j)) / 32);
    std::sort(lines.begin(), lines.end());
    direct += std::unique(lines.begin(), lines.end()) - lines.begin();
  }
  for (int k = 0; k < rows / 4; ++k) {  // staged: instruction k stores four rows of eight vectors
    std::vector<int64_t> lines;
    for (int l = 0; l < 32; ++l) {
      const int r = (l >> 3) + 4 * k, c = 4 * (l & 7);
      if (r < rows && c < cols) lines.push_back((dep_bits(jd.c_s_m, jd.mb, r) + dep_bits(jd.c_s_n, jd.nb, c)) / 32);
    }
    std::sort(lines.begin(), lines.end());
    staged += std::unique(lines.begin(), lines.end()) - lines.begin();
  }
  return direct <= 2 * staged ? 1 : 0;
}

// C = A.B^T computed as (B.A^T)^T: exchange the operands and the output's m/n strides.
void swap_operands(JoinDesc& jd) {
  std::swap(jd.a, jd.b);
  std::swap(jd.mb, jd.nb);
  for (int i = 0; i < TOGB_MAXBITS; ++i) std::swap(jd.c_s_m[i], jd.c_s_n[i]);
  std::swap(jd.r_cm, jd.r_cn);
  std::swap(jd.r_inv_m, jd.r_inv_n);
  jd.c_natural = 0;
}

// A count whose final join R = Y . X is a full dot product (scalar root), where
// X -- the right operand, the join queued just before R -- runs on the
// warp-specialised tensor-core kernel and both operands are stored in R's
// k order (address = k): X's epilogue forms the dot product with Y instead of
// storing X, R is not launched, and the root kernel sums X's per-tile
// partials.  This saves writing X and reading X and Y again (split form).
void fuse_root(togb_program* p, int mode) {
  p->root_fused = -1;
  if (mode != TOGB_MODE_SPLIT || p->host_only) return;
  const Node& R = p->nodes[p->root];
  if (R.leaf >= 0 || R.rank != 0) return;
  const Node& X = p->nodes[R.right];
  const Node& Y = p->nodes[R.left];
  if (X.leaf >= 0 || Y.leaf >= 0 || !X.dep) return;
  const int jr = R.join, jx = X.join;
  if (split_kernel(p, X) != togb::K_UMMA || !p->use_tma[jx]) return;
  const JoinDesc& dr = p->jds[jr];
  if (dr.a.outer_bits != 0 || dr.b.outer_bits != 0 || dr.kb != X.rank || !dr.a.exp_ptr) return;
  for (int i = 0; i < dr.kb; ++i)
    if (dr.a.s_k[i] != pow2(i) || dr.b.s_k[i] != pow2(i)) return;
  JoinDesc& dx = p->jds[jx];
  dx.dot_y = (const float*)dr.a.ptr;
  dx.dot_y_bs = dr.a.batch_stride;
  dx.dot_part = (double*)dx.c_ptr;  // X's own slot (2^rank floats per slice) holds its partials
  dx.dot_part_bs = dx.c_batch_stride / 2;
  p->rd.part = dx.dot_part;
  p->rd.done = reinterpret_cast<uint32_t*>(p->d_err + 1);
  p->rd.part_stride = dx.dot_part_bs;
  p->rd.npart = 8 << togb::umma_ws_tile_bits(dx.mb, dx.nb);  // tiles per slice x read-out warps
  p->rd.px_exp = dx.c_exp;
  p->rd.py_exp = dr.a.exp_ptr;
  p->rd.py_step = dr.a.meta_step;
  p->root_fused = jr;
}

void build_descs(togb_program* p, int mode, void* ws_v, int B) {
  p->once_segs_mode = -1;  // fused slice-invariant lists follow the descriptors
  p->once_segs.clear();
  char* ws = (char*)ws_v;
  const size_t es = elem_size(mode);
  p->jds.assign(p->joins.size(), JoinDesc{});
  p->tmaps.assign(2 * p->joins.size(), CUtensorMap{});
  p->use_tma.assign(p->joins.size(), 0);
  for (size_t j = 0; j < p->joins.size(); ++j) {
    const Node& J = p->nodes[p->joins[j]];
    JoinDesc& jd = p->jds[j];
    std::memset(&jd, 0, sizeof(jd));
    fill_operand(p, p->nodes[J.left], J.m_lsb, J.k_lsb, mode, ws, B, jd.a);
    fill_operand(p, p->nodes[J.right], J.n_lsb, J.k_lsb, mode, ws, B, jd.b);
    jd.mb = (int)J.m_lsb.size();
    jd.nb = (int)J.n_lsb.size();
    jd.kb = (int)J.k_lsb.size();
    jd.join = (int)j;
    const WsLayout w = ws_layout(p, mode, ws, B);
    // A slice-invariant join runs once (one slice in its launch), into the shared arena.
    jd.c_ptr = J.dep ? w.per + J.off * (int64_t)B * es : w.once + J.off * (int64_t)es;
    jd.c_batch_stride = pow2(J.rank);
    for (int i = 0; i < jd.mb; ++i) jd.c_s_m[i] = J.stride.at(J.m_lsb[i]);
    for (int i = 0; i < jd.nb; ++i) jd.c_s_n[i] = J.stride.at(J.n_lsb[i]);
    togb::make_runs(jd.c_s_m, jd.mb, &jd.r_cm);
    togb::make_runs(jd.c_s_n, jd.nb, &jd.r_cn);
    togb::make_inverse_runs(jd.c_s_m, jd.mb, &jd.r_inv_m);
    togb::make_inverse_runs(jd.c_s_n, jd.nb, &jd.r_inv_n);
    jd.c_natural = is_natural(jd);
    jd.err = p->d_err;
    jd.wait_cycles = p->wait_cycles;
    if (mode == TOGB_MODE_MOD && p->modulus >= 2) {  // runs require a modulus; describe may lack one
      jd.mod_p = p->modulus;
      jd.mod_m = ~0ull / p->modulus;
    }
    if (mode == TOGB_MODE_SPLIT) {
      jd.c_exp = J.dep ? w.per_exp + (int64_t)J.slot * B : w.once_exp + J.slot;
      jd.c_max = J.dep ? w.per_max + (int64_t)J.slot * B : w.once_max + J.slot;
      // The tensor-core kernel tiles 128 rows of M: put the larger extent there.
      if (split_kernel(p, J) == togb::K_UMMA) {
        if (jd.mb < 7 && jd.nb > jd.mb) swap_operands(jd);
        jd.c_direct = choose_direct_epilogue(jd);
        const int sl_a = jd.a.batch_stride ? B : 1, sl_b = jd.b.batch_stride ? B : 1;
        p->use_tma[j] = plain_k_major(jd.a) && plain_k_major(jd.b) && jd.kb >= 2 &&
                        make_tmap(jd.a, sl_a, 128, &p->tmaps[2 * j]) &&
                        make_tmap(jd.b, sl_b, togb::umma_ws_box_rows_b(jd.nb), &p->tmaps[2 * j + 1]);
      }
    }
  }
  // Root: outer bits enumerate the reference axis order, last axis lowest.
  const Node& Rn = p->nodes[p->root];
  std::vector<int> ref_lsb(Rn.ref.rbegin(), Rn.ref.rend());
  p->rd = RootDesc{};
  fill_operand(p, Rn, ref_lsb, {}, mode, ws, B, p->rd.r);
  p->rd.acc_sum = p->d_acc;
  p->rd.acc_comp = p->d_acc + pow2(Rn.rank);
  if (mode == TOGB_MODE_MOD && p->modulus >= 2) {
    p->rd.mod_p = p->modulus;
    p->rd.mod_m = ~0ull / p->modulus;
  }
  fuse_root(p, mode);
  if (mode == TOGB_MODE_SPLIT) {
    const WsLayout w = ws_layout(p, mode, ws, B);
    p->d_max = w.per_max;
    p->max_bytes = 4 * p->per.size() * (size_t)B;
    p->d_max_once = w.once_max;
    p->max_once_bytes = 4 * p->once.size();
  } else {
    p->d_max = p->d_max_once = nullptr;
    p->max_bytes = p->max_once_bytes = 0;
  }
}

// Splits the slice-invariant joins of the current descriptors into fused
// lists (runs of consecutive thread-per-output joins) and single launches, and
// copies each list's tables to the device.  Tables of earlier builds stay
// allocated until the program is destroyed: a batch graph captured from them
// may still be launched.
// The steps of the slice-invariant phase in `mode`: fused lists of
// thread-per-output joins and single launches of the other joins.  Every join
// goes as early as its producers allow, in the order F0 N0 F1 N1 ... (F: fused
// lists, N: the other joins, one launch each).  A thread-per-output join goes
// to the first F after all of its producers, any other join to the first N
// after them.  Inside an F the joins are ordered by depth, so a claimed tile
// waits only for joins whose tiles were claimed (and mostly finished) well
// before it.  Host-only: the device tables are built by prepare_once_fused.
std::vector<OnceSeg> once_segments(const togb_program* p, int mode) {
  std::vector<OnceSeg> segs;
  std::unordered_map<int, int> place, depth;  // join -> step index (F_s = 2s, N_t = 2t + 1), depth in its F
  int steps = 0;
  for (int j : p->once) {
    const Node& J = p->nodes[p->joins[j]];
    const bool direct = join_kernel(p, J, mode) == togb::K_DIRECT;
    int at = direct ? 0 : 1, d = 0;
    for (int opnd : {J.left, J.right}) {
      const Node& O = p->nodes[opnd];
      if (O.leaf >= 0 || O.dep) continue;
      const int pi = place.at(O.join);
      // an F join may share its producer's F (the list waits) and follows an
      // N producer in the next F; an N join follows an F producer in the
      // next N and may share an N producer's step (launched after it)
      const int need = direct ? (pi % 2 == 0 ? pi : pi + 1) : (pi % 2 == 0 ? pi + 1 : pi);
      at = std::max(at, need);
      if (direct && need == pi) d = std::max(d, depth.at(O.join) + 1);
    }
    place[j] = at;
    depth[j] = d;
    steps = std::max(steps, at + 1);
  }
  for (int st = 0; st < steps; ++st) {
    std::vector<std::pair<int, int>> members;  // (depth, position in once) of the joins of this step
    for (size_t i = 0; i < p->once.size(); ++i)
      if (place[p->once[i]] == st) members.push_back({st % 2 == 0 ? depth[p->once[i]] : 0, (int)i});
    if (members.empty()) continue;
    std::stable_sort(members.begin(), members.end());
    if (st % 2 == 0) {
      segs.emplace_back();
      segs.back().fused = true;
      for (auto& m : members) segs.back().js.push_back(p->once[m.second]);
    } else {
      for (auto& m : members) {
        segs.emplace_back();
        segs.back().fused = false;
        segs.back().js.push_back(p->once[m.second]);
      }
    }
  }
  return segs;
}

togb_status prepare_once_fused(togb_program* p, int mode) {
  if (p->once_segs_mode == mode) return TOGB_OK;
  p->once_segs.clear();
  p->once_segs_mode = -1;
  if (!p->once_no_reuse || p->once.empty()) {
    p->once_segs_mode = mode;
    return TOGB_OK;
  }
  p->once_segs = once_segments(p, mode);
  // Host images of the tables: [OnceJoin x n][tile_first x (n + 1)][deps x 2n][tile_join x tiles],
  // 256-byte aligned pieces.
  std::vector<char> img;
  size_t ctr = 0;
  auto put = [&img](const void* src, size_t bytes) {
    const size_t off = (img.size() + 255) / 256 * 256;
    img.resize(off + bytes);
    std::memcpy(img.data() + off, src, bytes);
    return off;
  };
  const size_t G = p->once_segs.size();
  std::vector<size_t> off_j(G), off_tf(G), off_dep(G), off_tj(G), off_ctr(G);
  for (size_t g = 0; g < G; ++g) {
    OnceSeg& S = p->once_segs[g];
    if (!S.fused) continue;
    const int n = (int)S.js.size();
    std::unordered_map<int, int> local;
    for (int i = 0; i < n; ++i) local[S.js[i]] = i;
    std::vector<togb::OnceJoin> oj(n);
    std::vector<int32_t> tf(n + 1, 0), deps(2 * n, -1), tj;
    for (int i = 0; i < n; ++i) {
      const Node& J = p->nodes[p->joins[S.js[i]]];
      const JoinDesc& jd = p->jds[S.js[i]];
      togb::OnceJoin& o = oj[i];
      std::memset(&o, 0, sizeof(o));
      o.a = jd.a.ptr;
      o.b = jd.b.ptr;
      o.a_lo = (const float*)jd.a.ptr_lo;
      o.b_lo = (const float*)jd.b.ptr_lo;
      o.c = jd.c_ptr;
      o.a_max = jd.a.max_ptr;
      o.b_max = jd.b.max_ptr;
      o.a_exp = jd.a.exp_ptr;
      o.b_exp = jd.b.exp_ptr;
      o.c_exp = jd.c_exp;
      o.c_max = jd.c_max;
      o.a_shift = jd.a.leaf_shift;
      o.b_shift = jd.b.leaf_shift;
      o.mb = jd.mb;
      o.nb = jd.nb;
      o.kb = jd.kb;
      o.natural = jd.c_natural;
      std::memcpy(o.a_ktab, jd.a.ktab, sizeof(o.a_ktab));
      std::memcpy(o.b_ktab, jd.b.ktab, sizeof(o.b_ktab));
      o.a_outer = jd.a.r_outer;
      o.b_outer = jd.b.r_outer;
      o.a_k = jd.a.r_k;
      o.b_k = jd.b.r_k;
      o.inv_m = jd.r_inv_m;
      o.inv_n = jd.r_inv_n;
      o.mod_p = jd.mod_p;
      o.mod_m = jd.mod_m;
      const int64_t outs = pow2(jd.mb + jd.nb);
      const int64_t tiles = (outs + togb::kOnceTile - 1) / togb::kOnceTile;
      if ((int64_t)tf[i] + tiles > INT32_MAX / 2) return fail(TOGB_ERR_UNSUPPORTED, "slice-invariant phase too large to fuse");
      tf[i + 1] = tf[i] + (int32_t)tiles;
      for (int64_t t = 0; t < tiles; ++t) tj.push_back(i);
      int w = 0;
      for (int opnd : {J.left, J.right}) {
        const Node& O = p->nodes[opnd];
        if (O.leaf < 0) {
          auto it = local.find(O.join);
          if (it != local.end()) deps[2 * i + w] = it->second;
        }
        ++w;
      }
    }
    off_j[g] = put(oj.data(), sizeof(togb::OnceJoin) * n);
    off_tf[g] = put(tf.data(), sizeof(int32_t) * (n + 1));
    off_dep[g] = put(deps.data(), sizeof(int32_t) * 2 * n);
    off_tj[g] = put(tj.data(), sizeof(int32_t) * tj.size());
    off_ctr[g] = ctr;
    ctr += 1 + (size_t)n;
    S.ol.n = n;
    S.ol.total_tiles = tf[n];
  }
  if (img.empty()) {
    p->once_segs_mode = mode;
    return TOGB_OK;
  }
  char* d = nullptr;
  cudaError_t e = cudaMalloc(&d, img.size());
  if (e != cudaSuccess) return cuda_fail(e, "fused slice-invariant tables");
  p->once_bufs.push_back(d);
  if ((e = cudaMemcpy(d, img.data(), img.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_fail(e, "fused slice-invariant tables");
  if (ctr * 4 > p->once_ctr_bytes) {
    uint32_t* c = nullptr;
    if ((e = cudaMalloc(&c, ctr * 4)) != cudaSuccess) return cuda_fail(e, "fused slice-invariant counters");
    p->once_bufs.push_back(c);
    p->d_once_ctr = c;
    p->once_ctr_bytes = ctr * 4;
  }
  for (size_t g = 0; g < G; ++g) {
    OnceSeg& S = p->once_segs[g];
    if (!S.fused) continue;
    S.ol.joins = (const togb::OnceJoin*)(d + off_j[g]);
    S.ol.tile_first = (const int32_t*)(d + off_tf[g]);
    S.ol.deps = (const int32_t*)(d + off_dep[g]);
    S.ol.tile_join = (const int32_t*)(d + off_tj[g]);
    S.ol.counters = p->d_once_ctr + off_ctr[g];
    S.ol.err = p->d_err;
    S.ol.wait_cycles = p->wait_cycles;
  }
  p->once_segs_mode = mode;
  return TOGB_OK;
}

// Queue one phase: the slice-invariant joins once (`once`, one slice per
// launch), or the per-slice joins and the root reduction for a chunk of `nb`
// slices.  With `ev`, event i is recorded before the phase's join i and one
// more after its last join.
togb_status enqueue_phase(togb_program* p, int mode, bool once, int nb, cudaStream_t st,
                          std::vector<cudaEvent_t>* ev) {
  const std::vector<int>& js = once ? p->once : p->per;
  // Split mode: every output's maximum starts at +0 (atomicMax target).
  uint32_t* mx = once ? p->d_max_once : p->d_max;
  const size_t mx_bytes = once ? p->max_once_bytes : p->max_bytes;
  if (mx_bytes) TOGB_CUDA(cudaMemsetAsync(mx, 0, mx_bytes, st));
  const int launch_slices = once ? 1 : nb;
  if (once && !ev && p->once_segs_mode == mode && !p->once_segs.empty()) {
    // Fused form of the slice-invariant phase (not while timing join by join).
    if (p->once_ctr_bytes) TOGB_CUDA(cudaMemsetAsync(p->d_once_ctr, 0, p->once_ctr_bytes, st));
    for (const OnceSeg& S : p->once_segs) {
      cudaError_t e;
      if (S.fused) {
        e = togb::launch_once_list(mode, S.ol, st);
      } else {
        const int j = S.js[0];
        const int kernel = join_kernel(p, p->nodes[p->joins[j]], mode);
        if (kernel == togb::K_UMMA && mode == TOGB_MODE_SPLIT && p->use_tma[j])
          e = togb::launch_umma(p->jds[j], &p->tmaps[2 * j], &p->tmaps[2 * j + 1], p->d_s0, 1, st);
        else
          e = togb::launch_join(mode, kernel, p->jds[j], p->d_s0, 1, st);
      }
      if (e != cudaSuccess) return cuda_fail(e, "join kernel launch");
    }
    return TOGB_OK;
  }
  for (size_t i = 0; i < js.size(); ++i) {
    const int j = js[i];
    if (ev) TOGB_CUDA(cudaEventRecord((*ev)[i], st));
    if (!once && j == p->root_fused) continue;  // formed in its right operand's epilogue
    const Node& J = p->nodes[p->joins[j]];
    const int kernel = join_kernel(p, J, mode);
    cudaError_t e;
    if (kernel == togb::K_UMMA && mode == TOGB_MODE_SPLIT && p->use_tma[j])
      e = togb::launch_umma(p->jds[j], &p->tmaps[2 * j], &p->tmaps[2 * j + 1], p->d_s0, launch_slices, st);
    else
      e = togb::launch_join(mode, kernel, p->jds[j], p->d_s0, launch_slices, st);
    if (e != cudaSuccess) return cuda_fail(e, "join kernel launch");
  }
  if (ev) TOGB_CUDA(cudaEventRecord((*ev)[js.size()], st));
  if (once) return TOGB_OK;
  cudaError_t e = togb::launch_root(mode, p->rd, p->d_s0, nb, st);
  if (e != cudaSuccess) return cuda_fail(e, "root kernel launch");
  return TOGB_OK;
}

// Queue a phase on `st`: timed launch by launch when timing is on (adding
// each join's device time to join_ms), else as a CUDA graph captured once per
// (phase, chunk size) and replayed.
togb_status run_phase(togb_program* p, int mode, bool once, int nb, cudaStream_t st) {
  const std::vector<int>& js = once ? p->once : p->per;
  if (once && js.empty()) return TOGB_OK;
  if (p->timing) {
    std::vector<cudaEvent_t> ev(js.size() + 1, nullptr);
    togb_status r = TOGB_OK;
    for (auto& x : ev)
      if (cudaEventCreate(&x) != cudaSuccess) { x = nullptr; r = fail(TOGB_ERR_CUDA, "event create"); }
    if (r == TOGB_OK) r = enqueue_phase(p, mode, once, nb, st, &ev);
    if (r == TOGB_OK) {
      cudaError_t e = cudaEventSynchronize(ev.back());
      for (size_t i = 0; e == cudaSuccess && i < js.size(); ++i) {
        float ms = 0;
        e = cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
        p->join_ms[js[i]] += ms;
      }
      if (e != cudaSuccess) r = cuda_fail(e, "join timing");
    }
    for (auto& x : ev)
      if (x) cudaEventDestroy(x);
    return r;
  }
  if (!p->use_graphs) return enqueue_phase(p, mode, once, nb, st, nullptr);
  const int key = once ? -1 : nb;
  auto it = p->graphs.find(key);
  // A phase's first run is queued launch by launch: a program contracted once
  // (the plugin's contract_sliced call) pays no capture or instantiation.
  // From the second run on it is captured once and replayed.
  if (it == p->graphs.end() && p->phase_runs[key]++ == 0) return enqueue_phase(p, mode, once, nb, st, nullptr);
  if (it == p->graphs.end()) {
    cudaGraph_t g = nullptr;
    TOGB_CUDA(cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal));
    togb_status r = enqueue_phase(p, mode, once, nb, p->cap_stream, nullptr);
    cudaError_t ce = cudaStreamEndCapture(p->cap_stream, &g);
    if (r != TOGB_OK) { if (g) cudaGraphDestroy(g); return r; }
    if (ce != cudaSuccess) return cuda_fail(ce, "graph capture");
    cudaGraphExec_t ex = nullptr;
    ce = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return cuda_fail(ce, "graph instantiate");
    it = p->graphs.emplace(key, ex).first;
  }
  TOGB_CUDA(cudaGraphLaunch(it->second, st));
  return TOGB_OK;
}

}  // namespace

extern "C" {

int togb_version(void) { return 1; }

const char* togb_last_error(void) { return g_err.c_str(); }

}  // extern "C"

namespace {

// Host half of togb_program_create: validation, lowering and planning.  No
// device memory is touched.  Leaf values are validated only when present.
// Split-form normaliser of one leaf: the power of two that brings its largest
// entry into [1, 2) (0 for an all-zero leaf).  `vals` holds a dense leaf's
// 2^r entries.  Returns an error message for values the forms cannot take.
const char* leaf_normaliser(int kind, const togb_leaf_spec* spec, const double* vals, int r, int* shift) {
  double mx = 0;
  if (kind == TOGB_LEAF_VARIABLE) {
    const double wn = spec->w_neg, wp = spec->w_pos;
    if (!(wn >= 0) || !(wp >= 0) || std::isinf(wn) || std::isinf(wp))
      return "variable weights must be finite and non-negative";
    mx = r == 0 ? wn + wp : std::max(wn, wp);
  } else if (kind == TOGB_LEAF_CLAUSE) {
    if (spec->output_index >= r) return "clause output axis out of range";
    mx = 1.0;
  } else if (kind == TOGB_LEAF_DENSE) {
    for (int64_t i = 0; vals && i < pow2(r); ++i) {
      const double v = vals[i];
      if (!(v >= 0) || std::isinf(v)) return "leaf entries must be finite and non-negative";
      mx = std::max(mx, v);
    }
  } else {
    return "unknown leaf kind";
  }
  int e2 = 0;
  if (mx > 0) std::frexp(mx, &e2);  // mx in [2^(e2-1), 2^e2)
  *shift = mx > 0 ? 1 - e2 : 0;
  return nullptr;
}

togb_status lower_host(const togb_program_desc* d, int device, togb_program** out, int64_t* num_values,
                       const togb_leaf_spec* specs = nullptr) {
  if (!d || !out) return fail(TOGB_ERR_INVALID, "null argument");
  *out = nullptr;
  if (d->num_leaves <= 0 || d->num_tokens <= 0) return fail(TOGB_ERR_INVALID, "empty program");
  if (d->num_groups < 0 || d->num_groups > 40) return fail(TOGB_ERR_UNSUPPORTED, "at most 40 slice groups");
  togb_program* p = new togb_program();
  p->device = device;
  p->G = d->num_groups;
  p->num_slices = pow2(p->G);
  // Slice groups.
  int64_t ge = 0;
  for (int g = 0; g < d->num_groups; ++g) {
    if (d->group_size[g] <= 0) { delete p; return fail(TOGB_ERR_INVALID, "empty slice group"); }
    for (int i = 0; i < d->group_size[g]; ++i) {
      const int e = d->group_edges[ge++];
      if (!p->group_of_edge.emplace(e, g).second) {
        delete p;
        return fail(TOGB_ERR_INVALID, "edge listed in two slice groups");
      }
    }
  }
  // Leaves.
  p->leaf_rank.assign(d->leaf_rank, d->leaf_rank + d->num_leaves);
  p->leaf_axes.resize(d->num_leaves);
  p->leaf_off.resize(d->num_leaves);
  p->leaf_shift.resize(d->num_leaves);
  p->leaf_kind.resize(d->num_leaves);
  int64_t ax = 0, voff = 0, dense_off = 0;
  for (int l = 0; l < d->num_leaves; ++l) {
    const int r = d->leaf_rank[l];
    if (r < 0 || r > 30) { delete p; return fail(TOGB_ERR_UNSUPPORTED, "leaf rank outside [0, 30]"); }
    p->leaf_axes[l].assign(d->leaf_axes + ax, d->leaf_axes + ax + r);
    ax += r;
    p->leaf_off[l] = voff;
    const int kind = specs ? specs[l].kind : TOGB_LEAF_DENSE;
    p->leaf_kind[l] = kind;
    const double* vals = nullptr;
    if (kind == TOGB_LEAF_DENSE) {
      vals = d->leaf_values ? d->leaf_values + (specs ? dense_off : voff) : nullptr;
      if (specs && !vals) { delete p; return fail(TOGB_ERR_INVALID, "dense leaf without values"); }
      dense_off += pow2(r);
    }
    if (const char* why = leaf_normaliser(kind, specs ? &specs[l] : nullptr, vals, r, &p->leaf_shift[l])) {
      delete p;
      const bool bad = kind == TOGB_LEAF_CLAUSE || kind < 0 || kind > TOGB_LEAF_VARIABLE;
      return fail(bad ? TOGB_ERR_INVALID : TOGB_ERR_UNSUPPORTED, why);
    }
    voff += pow2(r);
  }
  // Post-order walk (TensorNetwork.identify).
  std::vector<int> stack;
  std::vector<char> used(d->num_leaves, 0);
  for (int t = 0; t < d->num_tokens; ++t) {
    const int tok = d->postorder[t];
    if (tok >= 0) {
      if (tok >= d->num_leaves || used[tok]) { delete p; return fail(TOGB_ERR_INVALID, "bad leaf token"); }
      used[tok] = 1;
      Node n;
      n.leaf = tok;
      n.dep = false;
      const std::vector<int>& axes = p->leaf_axes[tok];
      const int R = (int)axes.size();
      for (int a = 0; a < R; ++a) {
        if (p->group_of_edge.count(axes[a])) { n.dep = true; continue; }
        if (n.stride.count(axes[a])) { delete p; return fail(TOGB_ERR_INVALID, "repeated edge in a leaf"); }
        n.ref.push_back(axes[a]);
        n.stride[axes[a]] = pow2(R - 1 - a);
      }
      n.rank = (int)n.ref.size();
      p->nodes.push_back(std::move(n));
      stack.push_back((int)p->nodes.size() - 1);
    } else {
      if (stack.size() < 2) { delete p; return fail(TOGB_ERR_INVALID, "join without two operands"); }
      Node n;
      n.right = stack.back(); stack.pop_back();
      n.left = stack.back(); stack.pop_back();
      n.join = (int)p->joins.size();
      n.dep = p->nodes[n.left].dep || p->nodes[n.right].dep;
      p->nodes.push_back(std::move(n));
      const int id = (int)p->nodes.size() - 1;
      plan_join(p, p->nodes[id]);
      if (p->nodes[id].rank > 30) { delete p; return fail(TOGB_ERR_UNSUPPORTED, "intermediate rank above 30"); }
      p->joins.push_back(id);
      stack.push_back(id);
    }
  }
  if (stack.size() != 1) { delete p; return fail(TOGB_ERR_INVALID, "post-order does not reduce to one tensor"); }
  for (int l = 0; l < d->num_leaves; ++l)
    if (!used[l]) { delete p; return fail(TOGB_ERR_INVALID, "leaf never pushed"); }
  p->root = stack[0];
  // Unsliced programs have one slice: nothing to hoist.  The root always runs
  // per slice (it feeds the slice sum).
  if (p->G == 0)
    for (Node& n : p->nodes) n.dep = true;
  p->nodes[p->root].dep = true;
  for (const Node& n : p->nodes) p->max_rank = std::max(p->max_rank, n.rank);
  plan_layouts(p);
  plan_arena(p);
  p->num_leaf_values = voff;
  *num_values = voff;
  *out = p;
  return TOGB_OK;
}

}  // namespace

extern "C" {

togb_status togb_program_create(const togb_program_desc* d, int device, togb_program** out) {
  if (!d || !out) return fail(TOGB_ERR_INVALID, "null argument");
  *out = nullptr;
  if (!d->leaf_values) return fail(TOGB_ERR_INVALID, "null leaf values");
  togb_program* p = nullptr;
  int64_t voff = 0;
  togb_status st = lower_host(d, device, &p, &voff);
  if (st != TOGB_OK) return st;

  // Device side.
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) { delete p; return cuda_fail(e, "cudaSetDevice"); }
  std::vector<float> v32(voff), v32lo(voff);
  for (int64_t i = 0; i < voff; ++i) {
    v32[i] = (float)d->leaf_values[i];
    v32lo[i] = (float)(d->leaf_values[i] - (double)v32[i]);
  }
  const int64_t E = pow2(p->nodes[p->root].rank);
  if ((e = cudaMalloc(&p->d_leaf64, std::max<int64_t>(voff, 1) * 8)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_leaf32, std::max<int64_t>(voff, 1) * 4)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_leaf32lo, std::max<int64_t>(voff, 1) * 4)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_acc, 2 * E * 8)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_s0, 8)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_err, 8)) != cudaSuccess ||  // error word, root kernel's CTA counter
      (e = cudaMemset(p->d_err, 0, 8)) != cudaSuccess ||
      (e = cudaMemcpy(p->d_leaf64, d->leaf_values, voff * 8, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(p->d_leaf32, v32.data(), voff * 4, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(p->d_leaf32lo, v32lo.data(), voff * 4, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemset(p->d_acc, 0, 2 * E * 8)) != cudaSuccess ||
      (e = cudaMemset(p->d_s0, 0, 8)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking)) != cudaSuccess) {
    togb_program_destroy(p);
    return cuda_fail(e, "program allocation");
  }
  *out = p;
  return TOGB_OK;
}

togb_status togb_program_create_compact(const togb_program_desc* d, const togb_leaf_spec* specs, int device,
                                        togb_program** out) {
  if (!d || !out || !specs) return fail(TOGB_ERR_INVALID, "null argument");
  *out = nullptr;
  togb_program* p = nullptr;
  int64_t voff = 0;
  togb_status st = lower_host(d, device, &p, &voff, specs);
  if (st != TOGB_OK) return st;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) { delete p; return cuda_fail(e, "cudaSetDevice"); }
  const int64_t E = pow2(p->nodes[p->root].rank);
  std::vector<togb::LeafBuild> items;
  for (int l = 0; l < d->num_leaves; ++l) {
    if (specs[l].kind == TOGB_LEAF_DENSE) continue;
    togb::LeafBuild it{};
    const int r = p->leaf_rank[l];
    it.off = p->leaf_off[l];
    it.rank = r;
    it.kind = specs[l].kind;
    it.out_pos = specs[l].output_index >= 0 ? r - 1 - specs[l].output_index : -1;
    for (int a = 0; a < r; ++a)
      if (!((specs[l].positive >> a) & 1)) it.false_idx |= 1u << (r - 1 - a);
    it.w_neg = specs[l].w_neg;
    it.w_pos = specs[l].w_pos;
    items.push_back(it);
  }
  togb::LeafBuild* d_items = nullptr;
  if ((e = cudaMalloc(&p->d_leaf64, std::max<int64_t>(voff, 1) * 8)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_leaf32, std::max<int64_t>(voff, 1) * 4)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_leaf32lo, std::max<int64_t>(voff, 1) * 4)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_acc, 2 * E * 8)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_s0, 8)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_err, 8)) != cudaSuccess ||  // error word, root kernel's CTA counter
      (e = cudaMemset(p->d_err, 0, 8)) != cudaSuccess ||
      (e = cudaMemset(p->d_acc, 0, 2 * E * 8)) != cudaSuccess ||
      (e = cudaMemset(p->d_s0, 0, 8)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (!items.empty() && (e = cudaMalloc(&d_items, items.size() * sizeof(togb::LeafBuild))) != cudaSuccess)) {
    togb_program_destroy(p);
    return cuda_fail(e, "program allocation");
  }
  // Dense leaves: their values, and the FP32 split, copied leaf by leaf.
  int64_t dense_off = 0;
  for (int l = 0; e == cudaSuccess && l < d->num_leaves; ++l) {
    if (specs[l].kind != TOGB_LEAF_DENSE) continue;
    const int64_t n = pow2(p->leaf_rank[l]);
    const double* v = d->leaf_values + dense_off;
    std::vector<float> hi(n), lo(n);
    for (int64_t i = 0; i < n; ++i) {
      hi[i] = (float)v[i];
      lo[i] = (float)(v[i] - (double)hi[i]);
    }
    const int64_t o = p->leaf_off[l];
    if ((e = cudaMemcpy(p->d_leaf64 + o, v, n * 8, cudaMemcpyHostToDevice)) == cudaSuccess &&
        (e = cudaMemcpy(p->d_leaf32 + o, hi.data(), n * 4, cudaMemcpyHostToDevice)) == cudaSuccess)
      e = cudaMemcpy(p->d_leaf32lo + o, lo.data(), n * 4, cudaMemcpyHostToDevice);
    dense_off += n;
  }
  if (e == cudaSuccess && !items.empty() &&
      (e = cudaMemcpy(d_items, items.data(), items.size() * sizeof(togb::LeafBuild), cudaMemcpyHostToDevice)) ==
          cudaSuccess &&
      (e = togb::launch_build_leaves(d_items, (int)items.size(), p->d_leaf64, p->d_leaf32, p->d_leaf32lo, nullptr)) ==
          cudaSuccess)
    e = cudaDeviceSynchronize();
  if (d_items) cudaFree(d_items);
  if (e != cudaSuccess) {
    togb_program_destroy(p);
    return cuda_fail(e, "leaf build");
  }
  *out = p;
  return TOGB_OK;
}

togb_status togb_program_set_leaves(togb_program* p, const togb_leaf_spec* specs, const double* dense_values,
                                    int64_t num_dense_values, void* stream) {
  if (!p || !specs) return fail(TOGB_ERR_INVALID, "null argument");
  if (p->host_only) return fail(TOGB_ERR_UNSUPPORTED, "host-only program: it has no leaves on a device");
  const int n = (int)p->leaf_rank.size();
  int64_t want = 0;
  for (int l = 0; l < n; ++l) {
    if (specs[l].kind != p->leaf_kind[l]) return fail(TOGB_ERR_INVALID, "leaf " + std::to_string(l) + " changed kind");
    if (specs[l].kind == TOGB_LEAF_DENSE) want += pow2(p->leaf_rank[l]);
  }
  if (num_dense_values != want || (want > 0 && !dense_values))
    return fail(TOGB_ERR_INVALID, "dense leaf values: expected " + std::to_string(want));
  // Validate everything and compute the normalisers before touching the device.
  std::vector<int> shift(n);
  int64_t dense_off = 0;
  for (int l = 0; l < n; ++l) {
    const int r = p->leaf_rank[l];
    const double* vals = specs[l].kind == TOGB_LEAF_DENSE ? dense_values + dense_off : nullptr;
    if (const char* why = leaf_normaliser(specs[l].kind, &specs[l], vals, r, &shift[l]))
      return fail(specs[l].kind == TOGB_LEAF_CLAUSE ? TOGB_ERR_INVALID : TOGB_ERR_UNSUPPORTED, why);
    if (vals) dense_off += pow2(r);
  }
  TOGB_CUDA(cudaSetDevice(p->device));
  cudaStream_t st = (cudaStream_t)stream;
  // Dense leaves: FP64 values and their FP32 hi/lo split, staged in the program.
  p->h_hi.resize((size_t)want);
  p->h_lo.resize((size_t)want);
  p->h_items.clear();
  dense_off = 0;
  for (int l = 0; l < n; ++l) {
    const int r = p->leaf_rank[l];
    if (specs[l].kind != TOGB_LEAF_DENSE) {
      togb::LeafBuild it{};
      it.off = p->leaf_off[l];
      it.rank = r;
      it.kind = specs[l].kind;
      it.out_pos = specs[l].output_index >= 0 ? r - 1 - specs[l].output_index : -1;
      for (int a = 0; a < r; ++a)
        if (!((specs[l].positive >> a) & 1)) it.false_idx |= 1u << (r - 1 - a);
      it.w_neg = specs[l].w_neg;
      it.w_pos = specs[l].w_pos;
      p->h_items.push_back(it);
      continue;
    }
    const int64_t m = pow2(r), o = p->leaf_off[l];
    const double* v = dense_values + dense_off;
    for (int64_t i = 0; i < m; ++i) {
      p->h_hi[dense_off + i] = (float)v[i];
      p->h_lo[dense_off + i] = (float)(v[i] - (double)p->h_hi[dense_off + i]);
    }
    TOGB_CUDA(cudaMemcpyAsync(p->d_leaf64 + o, v, m * 8, cudaMemcpyHostToDevice, st));
    TOGB_CUDA(cudaMemcpyAsync(p->d_leaf32 + o, p->h_hi.data() + dense_off, m * 4, cudaMemcpyHostToDevice, st));
    TOGB_CUDA(cudaMemcpyAsync(p->d_leaf32lo + o, p->h_lo.data() + dense_off, m * 4, cudaMemcpyHostToDevice, st));
    dense_off += m;
  }
  if (!p->h_items.empty()) {
    if (p->h_items.size() > p->d_items_cap) {
      if (p->d_items) {
        TOGB_CUDA(cudaStreamSynchronize(st));  // an earlier build may still read the records
        cudaFree(p->d_items);
        p->d_items = nullptr;
        p->d_items_cap = 0;
      }
      TOGB_CUDA(cudaMalloc(&p->d_items, p->h_items.size() * sizeof(togb::LeafBuild)));
      p->d_items_cap = p->h_items.size();
    }
    TOGB_CUDA(cudaMemcpyAsync(p->d_items, p->h_items.data(), p->h_items.size() * sizeof(togb::LeafBuild),
                              cudaMemcpyHostToDevice, st));
    const cudaError_t e =
        togb::launch_build_leaves(p->d_items, (int)p->h_items.size(), p->d_leaf64, p->d_leaf32, p->d_leaf32lo, st);
    if (e != cudaSuccess) return cuda_fail(e, "leaf build");
  }
  p->leaf_int_current = false;  // the int forms convert the new values at their next run
  p->leaf_mod_p = 0;
  if (shift != p->leaf_shift) {  // the normalisers are part of the descriptors: rebuild them
    p->leaf_shift = shift;
    clear_graphs(p);
    p->cur_mode = -1;
  }
  return TOGB_OK;
}

togb_status togb_program_create_host(const togb_program_desc* d, togb_program** out) {
  if (!d || !out) return fail(TOGB_ERR_INVALID, "null argument");
  int64_t voff = 0;
  togb_program* p = nullptr;
  togb_status st = lower_host(d, -1, &p, &voff);
  if (st != TOGB_OK) return st;
  p->host_only = true;
  *out = p;
  return TOGB_OK;
}

togb_status togb_program_describe(togb_program* p, int mode, int32_t join, char* buf, size_t n) {
  if (!p || !buf || n == 0) return fail(TOGB_ERR_INVALID, "null argument");
  if (!known_mode(mode)) return fail(TOGB_ERR_INVALID, "unknown mode");
  if (join < 0 || join >= (int32_t)p->joins.size()) return fail(TOGB_ERR_INVALID, "join index out of range");
  if (p->cur_mode != mode) {
    if (!p->host_only) return fail(TOGB_ERR_UNSUPPORTED, "describe a device program after a run in this mode");
    // Descriptors against a null workspace: offsets are what matters here.
    build_descs(p, mode, nullptr, 1);
    p->cur_mode = mode;
  }
  const JoinDesc& jd = p->jds[join];
  const Node& J = p->nodes[p->joins[join]];
  std::string s = "join " + std::to_string(join) + " mnk " + std::to_string(jd.mb) + " " + std::to_string(jd.nb) +
                  " " + std::to_string(jd.kb) + " kernel " + std::to_string(join_kernel(p, J, mode)) +
                  " per_slice " + std::to_string(J.dep ? 1 : 0) + " c_natural " + std::to_string(jd.c_natural);
  if (join_kernel(p, J, mode) == togb::K_DIRECT) {
    static const char* names[] = {"direct", "staged", "stream", "stream_kfast"};
    s += std::string(" variant ") + names[togb::direct_variant(mode, jd)];
  }
  if (join_kernel(p, J, mode) == togb::K_UMMA && mode == TOGB_MODE_SPLIT) {
    s += std::string(" epilogue ") + (jd.dot_y ? "root_dot" : (jd.c_direct ? "direct" : "staged"));
    if (!p->host_only) s += p->use_tma[join] ? " loads tma" : " loads gather";
  }
  if (join == p->root_fused) s += " fused_into_operand";
  s += "\n";
  auto strides = [&](const char* name, const int64_t* v, int nb) {
    s += name;
    for (int i = 0; i < nb; ++i) s += " " + std::to_string(v[i]);
    s += "\n";
  };
  for (int w = 0; w < 2; ++w) {
    const OpDesc& o = w ? jd.b : jd.a;
    s += w ? "B" : "A";
    s += std::string(" leaf ") + (o.exp_ptr || o.batch_stride ? "0" : "1") + " batch_stride " +
         std::to_string(o.batch_stride) + " k_fast " + std::to_string(o.k_fast) + " runs_outer " +
         std::to_string(o.r_outer.n) + " runs_k " + std::to_string(o.r_k.n) + "\n";
    strides(w ? "  B s_outer" : "  A s_outer", o.s_outer, o.outer_bits);
    strides(w ? "  B s_k" : "  A s_k", o.s_k, o.k_bits);
  }
  strides("C s_m", jd.c_s_m, jd.mb);
  strides("C s_n", jd.c_s_n, jd.nb);
  s += "C runs_inv_m " + std::to_string(jd.r_inv_m.n) + " runs_inv_n " + std::to_string(jd.r_inv_n.n) + "\n";
  std::snprintf(buf, n, "%s", s.c_str());
  return TOGB_OK;
}

togb_status togb_program_info_get(const togb_program* p, togb_program_info* info) {
  if (!p || !info) return fail(TOGB_ERR_INVALID, "null argument");
  info->num_slices = p->num_slices;
  info->num_joins = (int32_t)p->joins.size();
  info->max_rank = p->max_rank;
  info->root_rank = p->nodes[p->root].rank;
  info->num_launches = (int32_t)p->per.size() + 1;
  info->flops_per_slice = p->flops;
  info->bytes_per_slice_f64 = p->bytes64;
  for (int m = 0; m < 4; ++m) {
    info->workspace_per_slice[m] = ws_per_slice(p, m);
    info->workspace_fixed[m] = ws_fixed(p, m);
  }
  info->num_joins_once = (int32_t)p->once.size();
  info->flops_once = p->flops_once;
  info->bytes_once_f64 = p->bytes64_once;
  return TOGB_OK;
}

togb_status togb_program_reset(togb_program* p, void* stream) {
  if (!p) return fail(TOGB_ERR_INVALID, "null program");
  if (p->host_only) return fail(TOGB_ERR_UNSUPPORTED, "host-only program: create it with togb_program_create to run it");
  TOGB_CUDA(cudaSetDevice(p->device));
  const int64_t E = pow2(p->nodes[p->root].rank);
  TOGB_CUDA(cudaMemsetAsync(p->d_acc, 0, 2 * E * 8, (cudaStream_t)stream));
  p->acc_kind = 0;
  return TOGB_OK;
}

togb_status togb_program_joins(const togb_program* p, int mode, int32_t* out, int32_t n) {
  if (!p || !out) return fail(TOGB_ERR_INVALID, "null argument");
  if (!known_mode(mode)) return fail(TOGB_ERR_INVALID, "unknown mode");
  if (n != (int32_t)p->joins.size()) return fail(TOGB_ERR_INVALID, "n must equal the number of joins");
  for (size_t j = 0; j < p->joins.size(); ++j) {
    const Node& J = p->nodes[p->joins[j]];
    out[5 * j + 0] = (int32_t)J.m_lsb.size();
    out[5 * j + 1] = (int32_t)J.n_lsb.size();
    out[5 * j + 2] = (int32_t)J.k_lsb.size();
    out[5 * j + 3] = join_kernel(p, J, mode);
    out[5 * j + 4] = J.dep ? 1 : 0;
  }
  return TOGB_OK;
}

togb_status togb_program_launch_count(const togb_program* p, int mode, int64_t* launches) {
  if (!p || !launches) return fail(TOGB_ERR_INVALID, "null argument");
  if (!known_mode(mode)) return fail(TOGB_ERR_INVALID, "unknown mode");
  int64_t once = (int64_t)p->once.size();
  if (p->once_segs_mode == mode) {
    if (!p->once_segs.empty()) once = (int64_t)p->once_segs.size();
  } else if (p->once_no_reuse && !p->once.empty()) {
    once = (int64_t)once_segments(p, mode).size();  // as a run in this form would queue them
  }
  const int64_t B = p->cur_mode == mode && p->cur_B > 0 ? p->cur_B : p->num_slices;
  const int64_t chunks = (p->num_slices + B - 1) / B;
  const int64_t fused = p->cur_mode == mode && p->root_fused >= 0 ? 1 : 0;
  *launches = once + chunks * ((int64_t)p->per.size() - fused + 2);
  return TOGB_OK;
}

togb_status togb_program_set_kernel(togb_program* p, int mode, int32_t join, int32_t kernel) {
  if (!p) return fail(TOGB_ERR_INVALID, "null program");
  if (!known_mode(mode)) return fail(TOGB_ERR_INVALID, "unknown mode");
  if (join < 0 || join >= (int32_t)p->joins.size()) return fail(TOGB_ERR_INVALID, "join index out of range");
  Node& J = p->nodes[p->joins[join]];
  if (kernel >= 0 && !kernel_allowed(p, J, mode, kernel))
    return fail(TOGB_ERR_UNSUPPORTED, "kernel " + std::to_string(kernel) + " cannot run join " + std::to_string(join));
  if (J.kernel_set[mode] != kernel) {
    J.kernel_set[mode] = kernel < 0 ? -1 : kernel;
    if (p->cur_mode == mode) {  // descriptors (TMA maps, operand order) follow the kernel choice
      clear_graphs(p);
      p->cur_mode = -1;
    }
  }
  return TOGB_OK;
}

togb_status togb_program_kernel_allowed(const togb_program* p, int mode, int32_t join, int32_t kernel,
                                        int32_t* allowed) {
  if (!p || !allowed) return fail(TOGB_ERR_INVALID, "null argument");
  if (!known_mode(mode)) return fail(TOGB_ERR_INVALID, "unknown mode");
  if (join < 0 || join >= (int32_t)p->joins.size()) return fail(TOGB_ERR_INVALID, "join index out of range");
  *allowed = kernel_allowed(p, p->nodes[p->joins[join]], mode, kernel) ? 1 : 0;
  return TOGB_OK;
}

togb_status togb_program_set_wait_limit(togb_program* p, int64_t cycles) {
  if (!p) return fail(TOGB_ERR_INVALID, "null program");
  const int64_t c = cycles > 0 ? cycles : togb::kDefaultWaitCycles;
  if (c != p->wait_cycles) {
    p->wait_cycles = c;
    clear_graphs(p);      // captured launches carry the old limit
    p->cur_mode = -1;     // descriptors are rebuilt on the next run
    p->once_segs_mode = -1;
  }
  return TOGB_OK;
}

togb_status togb_program_set_timing(togb_program* p, int enable) {
  if (!p) return fail(TOGB_ERR_INVALID, "null program");
  p->timing = enable != 0;
  return TOGB_OK;
}

togb_status togb_program_join_times(togb_program* p, float* ms, int32_t n) {
  if (!p || !ms) return fail(TOGB_ERR_INVALID, "null argument");
  if (n != (int32_t)p->joins.size() || p->join_ms.size() != p->joins.size())
    return fail(TOGB_ERR_INVALID, "no timing recorded for this program (enable timing, then run)");
  std::copy(p->join_ms.begin(), p->join_ms.end(), ms);
  return TOGB_OK;
}

togb_status togb_program_run(togb_program* p, int mode, int64_t begin, int64_t end, void* workspace,
                             size_t ws_bytes, void* stream_v) {
  if (!p) return fail(TOGB_ERR_INVALID, "null program");
  if (p->host_only) return fail(TOGB_ERR_UNSUPPORTED, "host-only program: create it with togb_program_create to run it");
  if (!known_mode(mode)) return fail(TOGB_ERR_INVALID, "unknown mode");
  if (begin < 0 || end > p->num_slices || begin > end) return fail(TOGB_ERR_INVALID, "slice range out of bounds");
  const int kind = mode == TOGB_MODE_INT64 ? 2 : mode == TOGB_MODE_MOD ? 3 : 1;
  if (kind == 3 && p->modulus < 2) return fail(TOGB_ERR_INVALID, "set a modulus (togb_program_set_modulus) first");
  if (p->acc_kind != 0 && (p->acc_kind != kind || (kind == 3 && p->acc_modulus != p->modulus))) {
    const std::string holds = p->acc_kind == 1   ? "FP64 sums"
                              : p->acc_kind == 2 ? "int-form words"
                                                 : "residues modulo " + std::to_string(p->acc_modulus);
    return fail(TOGB_ERR_INVALID, "the accumulator holds " + holds + ": reset it first");
  }
  if (begin == end) return TOGB_OK;
  cudaStream_t st = (cudaStream_t)stream_v;
  TOGB_CUDA(cudaSetDevice(p->device));
  if (kind >= 2) {
    // The int forms' leaves, made from the FP64 values on this stream.  Each
    // buffer is allocated once, so descriptors keep its address.
    const bool mod = kind == 3;
    void*& buf = mod ? p->d_leaf_mod : p->d_leaf_int;
    if (mod ? p->leaf_mod_p != p->modulus : !p->leaf_int_current) {
      if (!buf) {
        cudaError_t e = cudaMalloc(&buf, std::max<int64_t>(p->num_leaf_values, 1) * 8);
        if (e != cudaSuccess) {
          buf = nullptr;
          return cuda_fail(e, "int-form leaf allocation");
        }
      }
      cudaError_t e = mod ? togb::launch_leaf_mod(p->d_leaf64, buf, p->num_leaf_values, p->modulus, st)
                          : togb::launch_leaf_int(p->d_leaf64, buf, p->num_leaf_values, st);
      if (e != cudaSuccess) return cuda_fail(e, "int-form leaf conversion");
      if (mod) p->leaf_mod_p = p->modulus;
      else p->leaf_int_current = true;
    }
  }
  p->acc_kind = kind;
  p->acc_modulus = kind == 3 ? p->modulus : 0;
  const int64_t per = ws_per_slice(p, mode);
  const int64_t fixed = ws_fixed(p, mode);
  const int64_t want = end - begin;
  if (!workspace) {
    // Own workspace: as many slices per chunk as fit a quarter of free memory.
    size_t freeb = 0, totalb = 0;
    TOGB_CUDA(cudaMemGetInfo(&freeb, &totalb));
    int64_t fit = ((int64_t)(freeb / 4 + p->own_ws_bytes) - fixed) / per;
    int64_t B = std::max<int64_t>(1, std::min<int64_t>(want, std::min<int64_t>(fit, 65535)));
    const size_t need = (size_t)(B * per + fixed);
    if (p->own_ws_bytes < need) {
      if (p->own_ws) { cudaFree(p->own_ws); p->own_ws = nullptr; p->own_ws_bytes = 0; }
      cudaError_t e = cudaMalloc(&p->own_ws, need);
      if (e != cudaSuccess) return cuda_fail(e, "workspace allocation");
      p->own_ws_bytes = need;
    }
    workspace = p->own_ws;
    ws_bytes = p->own_ws_bytes;
  }
  char* ws = (char*)(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
  const int64_t usable = (int64_t)ws_bytes - (int64_t)(ws - (char*)workspace) - ws_once(p, mode);
  // Slices per chunk: what the workspace holds, independent of this call's
  // range, so a count queued as several calls over consecutive ranges keeps
  // one set of descriptors and graphs.
  int64_t B = usable > 0 ? usable / per : 0;
  B = std::min<int64_t>(B, std::min<int64_t>(p->num_slices, 65535));
  if (B < 1) return fail(TOGB_ERR_OOM, "workspace smaller than one slice");
  if (mode != p->cur_mode || B != p->cur_B || ws != p->cur_ws) {
    clear_graphs(p);
    build_descs(p, mode, ws, (int)B);
    p->cur_mode = mode;
    p->cur_B = (int)B;
    p->cur_ws = ws;
  }
  if (p->timing) p->join_ms.assign(p->joins.size(), 0.f);
  togb_status r = prepare_once_fused(p, mode);
  if (r != TOGB_OK) return r;
  // The slice-invariant joins first (once per call), then every chunk.
  r = run_phase(p, mode, true, 1, st);
  for (int64_t s = begin; r == TOGB_OK && s < end; s += B) {
    const int nb = (int)std::min<int64_t>(B, end - s);
    cudaError_t e = togb::launch_set_s0(p->d_s0, s, st);
    if (e != cudaSuccess) return cuda_fail(e, "slice base update");
    r = run_phase(p, mode, false, nb, st);
  }
  return r;
}

namespace {

// Checks shared by the result entry points, then a wait for `stream` and the
// device error word.
togb_status result_ready(togb_program* p, void* stream, const void* out, int64_t n, int kind) {
  if (!p || !out) return fail(TOGB_ERR_INVALID, "null argument");
  if (p->host_only) return fail(TOGB_ERR_UNSUPPORTED, "host-only program has no result");
  const int64_t E = pow2(p->nodes[p->root].rank);
  if (n != E) return fail(TOGB_ERR_INVALID, "result size does not match the root tensor");
  if (p->acc_kind != 0 && (p->acc_kind == 1) != (kind == 1))
    return fail(TOGB_ERR_INVALID, kind != 1 ? "the accumulator holds FP64 sums: read it with togb_program_result"
                                            : "the accumulator holds int-form words: read it with togb_program_result_u64");
  TOGB_CUDA(cudaSetDevice(p->device));
  TOGB_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  int32_t err = 0;
  TOGB_CUDA(cudaMemcpy(&err, p->d_err, 4, cudaMemcpyDeviceToHost));
  if (err) {
    TOGB_CUDA(cudaMemset(p->d_err, 0, 4));
    return fail(TOGB_ERR_TIMEOUT,
                "a device-side wait ran out of its limit (a fused slice-invariant list waiting for a producer "
                "tile, or a tensor-core join waiting in its load/MMA/read-out pipeline); the result is invalid");
  }
  return TOGB_OK;
}

}  // namespace

togb_status togb_program_set_modulus(togb_program* p, uint64_t modulus) {
  if (!p) return fail(TOGB_ERR_INVALID, "null program");
  if (modulus < 2 || modulus >= (1ull << 28)) return fail(TOGB_ERR_INVALID, "the modulus must lie in [2, 2^28)");
  if (modulus != p->modulus) {
    p->modulus = modulus;
    if (p->cur_mode == TOGB_MODE_MOD) {  // descriptors and graphs carry the modulus
      clear_graphs(p);
      p->cur_mode = -1;
    }
  }
  return TOGB_OK;
}

togb_status togb_program_result_u64(togb_program* p, void* stream, uint64_t* out, int64_t n) {
  togb_status r = result_ready(p, stream, out, n, 2);
  if (r != TOGB_OK) return r;
  TOGB_CUDA(cudaMemcpy(out, p->d_acc, n * 8, cudaMemcpyDeviceToHost));
  return TOGB_OK;
}

togb_status togb_program_result(togb_program* p, void* stream, double* out, double* comp, int64_t n) {
  togb_status r = result_ready(p, stream, out, n, 1);
  if (r != TOGB_OK) return r;
  const int64_t E = n;
  std::vector<double> h(2 * E);
  TOGB_CUDA(cudaMemcpy(h.data(), p->d_acc, 2 * E * 8, cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < E; ++i) {
    out[i] = h[i] + h[E + i];
    if (comp) comp[i] = h[E + i];
  }
  return TOGB_OK;
}

void togb_program_destroy(togb_program* p) {
  if (!p) return;
  if (p->host_only) {
    delete p;
    return;
  }
  cudaSetDevice(p->device);
  clear_graphs(p);
  cudaFree(p->d_leaf64);
  cudaFree(p->d_leaf32);
  cudaFree(p->d_leaf32lo);
  cudaFree(p->d_leaf_int);
  cudaFree(p->d_leaf_mod);
  cudaFree(p->d_acc);
  cudaFree(p->d_s0);
  cudaFree(p->d_err);
  for (void* b : p->once_bufs) cudaFree(b);
  if (p->d_items) cudaFree(p->d_items);
  if (p->own_ws) cudaFree(p->own_ws);
  if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
  delete p;
}

// ---------------------------------------------------------------------------
// Batches: many programs (instances of uneven size, each with its own plan and
// slice count) contracted by one CUDA graph.  Program i runs on internal
// stream i % nstreams, so independent instances overlap on the GPU; the graph
// forks from the caller's stream and joins back into it.
struct togb_batch {
  std::vector<togb_program*> progs;
  std::vector<char*> ws;
  std::vector<int64_t> B;
  int mode = 0;
  std::vector<cudaStream_t> streams;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  cudaStream_t cap = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

void batch_free(togb_batch* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (auto s : b->streams) cudaStreamDestroy(s);
  for (auto e : b->joins) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->cap) cudaStreamDestroy(b->cap);
  delete b;
}

// All of program p's work for one count, queued on st: accumulator reset,
// slice-invariant joins, then every chunk of slices.
togb_status enqueue_count(togb_program* p, int mode, int64_t B, cudaStream_t st) {
  const int64_t E = pow2(p->nodes[p->root].rank);
  TOGB_CUDA(cudaMemsetAsync(p->d_acc, 0, 2 * E * 8, st));
  p->acc_kind = 1;  // batches run the FP64 and split forms
  togb_status r = enqueue_phase(p, mode, true, 1, st, nullptr);
  for (int64_t s = 0; r == TOGB_OK && s < p->num_slices; s += B) {
    const int nb = (int)std::min<int64_t>(B, p->num_slices - s);
    cudaError_t e = togb::launch_set_s0(p->d_s0, s, st);
    if (e != cudaSuccess) return cuda_fail(e, "slice base update");
    r = enqueue_phase(p, mode, false, nb, st, nullptr);
  }
  return r;
}

}  // namespace

extern "C" {

togb_status togb_batch_create(togb_program* const* progs, int32_t n, int mode, void* const* workspaces,
                              const size_t* ws_bytes, int32_t nstreams, togb_batch** out) {
  if (!progs || !workspaces || !ws_bytes || !out || n <= 0 || nstreams <= 0 || nstreams > 64)
    return fail(TOGB_ERR_INVALID, "bad batch arguments");
  if (mode != TOGB_MODE_F64 && mode != TOGB_MODE_SPLIT)
    return fail(TOGB_ERR_INVALID, "batches run the FP64 and split forms");
  *out = nullptr;
  togb_batch* b = new togb_batch();
  b->mode = mode;
  const int dev = progs[0]->device;
  cudaError_t e = cudaSetDevice(dev);
  if (e != cudaSuccess) { batch_free(b); return cuda_fail(e, "cudaSetDevice"); }
  for (int32_t i = 0; i < n; ++i) {
    togb_program* p = progs[i];
    if (!p || p->device != dev || !workspaces[i]) { batch_free(b); return fail(TOGB_ERR_INVALID, "bad batch member"); }
    for (int32_t k = 0; k < i; ++k)
      if (progs[k] == p) { batch_free(b); return fail(TOGB_ERR_INVALID, "a program appears twice in a batch"); }
    char* ws = (char*)(((uintptr_t)workspaces[i] + 255) & ~(uintptr_t)255);
    const int64_t usable = (int64_t)ws_bytes[i] - (int64_t)(ws - (char*)workspaces[i]) - ws_once(p, mode);
    const int64_t per = ws_per_slice(p, mode);
    const int64_t B = std::min<int64_t>(usable > 0 ? usable / per : 0, std::min<int64_t>(p->num_slices, 65535));
    if (B < 1) { batch_free(b); return fail(TOGB_ERR_OOM, "workspace of batch member " + std::to_string(i) + " smaller than one slice"); }
    if (mode != p->cur_mode || B != p->cur_B || ws != p->cur_ws) {
      clear_graphs(p);
      build_descs(p, mode, ws, (int)B);
      p->cur_mode = mode;
      p->cur_B = (int)B;
      p->cur_ws = ws;
    }
    togb_status pr = prepare_once_fused(p, mode);
    if (pr != TOGB_OK) { batch_free(b); return pr; }
    b->progs.push_back(p);
    b->ws.push_back(ws);
    b->B.push_back(B);
  }
  const int K = std::min<int32_t>(nstreams, n);
  b->streams.resize(K, nullptr);
  b->joins.resize(K, nullptr);
  if ((e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess) {
    batch_free(b);
    return cuda_fail(e, "batch streams");
  }
  for (int k = 0; k < K; ++k)
    if ((e = cudaStreamCreateWithFlags(&b->streams[k], cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->joins[k], cudaEventDisableTiming)) != cudaSuccess) {
      batch_free(b);
      return cuda_fail(e, "batch streams");
    }
  // Capture: fork to K streams, each program's count on its stream, join back.
  cudaGraph_t g = nullptr;
  togb_status r = TOGB_OK;
  if ((e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
    batch_free(b);
    return cuda_fail(e, "batch capture");
  }
  e = cudaEventRecord(b->fork, b->cap);
  for (int k = 0; e == cudaSuccess && k < K; ++k) e = cudaStreamWaitEvent(b->streams[k], b->fork, 0);
  for (int32_t i = 0; e == cudaSuccess && r == TOGB_OK && i < n; ++i)
    r = enqueue_count(b->progs[i], mode, b->B[i], b->streams[i % K]);
  for (int k = 0; e == cudaSuccess && k < K; ++k) {
    e = cudaEventRecord(b->joins[k], b->streams[k]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->cap, b->joins[k], 0);
  }
  cudaError_t ce = cudaStreamEndCapture(b->cap, &g);
  if (e == cudaSuccess) e = ce;
  if (r == TOGB_OK && e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, g, 0);
  if (g) cudaGraphDestroy(g);
  if (r != TOGB_OK || e != cudaSuccess) {
    batch_free(b);
    return r != TOGB_OK ? r : cuda_fail(e, "batch graph");
  }
  *out = b;
  return TOGB_OK;
}

togb_status togb_batch_run(togb_batch* b, void* stream) {
  if (!b) return fail(TOGB_ERR_INVALID, "null batch");
  TOGB_CUDA(cudaSetDevice(b->progs[0]->device));
  TOGB_CUDA(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
  return TOGB_OK;
}

togb_status togb_batch_results(togb_batch* b, void* stream, double* out, int32_t n) {
  if (!b || !out) return fail(TOGB_ERR_INVALID, "null argument");
  if (n != (int32_t)b->progs.size()) return fail(TOGB_ERR_INVALID, "n must equal the batch size");
  for (int32_t i = 0; i < n; ++i) {
    togb_program* p = b->progs[i];
    const int64_t E = pow2(p->nodes[p->root].rank);
    if (E != 1) return fail(TOGB_ERR_UNSUPPORTED, "batch results are scalar counts (root rank 0)");
    togb_status r = togb_program_result(p, stream, out + i, nullptr, 1);
    if (r != TOGB_OK) return r;
  }
  return TOGB_OK;
}

void togb_batch_destroy(togb_batch* b) {
  if (!b) return;
  cudaSetDevice(b->progs.empty() ? 0 : b->progs[0]->device);
  batch_free(b);
}

}  // extern "C"

namespace {

// One np.tensordot of binary-index tensors of 8-byte elements as a single
// join in `mode` (TOGB_MODE_F64 or TOGB_MODE_INT64, which share the layout).
togb_status tensordot_join(int mode, const void* a, int32_t ra, const void* b, int32_t rb, int32_t n_axes,
                           const int32_t* axes_a, const int32_t* axes_b, void* out, void* stream) {
  if (!a || !b || !out) return fail(TOGB_ERR_INVALID, "null tensor");
  if (ra < 0 || rb < 0 || ra > 30 || rb > 30 || n_axes < 0 || n_axes > std::min(ra, rb))
    return fail(TOGB_ERR_INVALID, "bad ranks or axis count");
  std::vector<char> in_a(ra, 0), in_b(rb, 0);
  for (int i = 0; i < n_axes; ++i) {
    if (axes_a[i] < 0 || axes_a[i] >= ra || axes_b[i] < 0 || axes_b[i] >= rb || in_a[axes_a[i]] || in_b[axes_b[i]])
      return fail(TOGB_ERR_INVALID, "bad contraction axes");
    in_a[axes_a[i]] = 1;
    in_b[axes_b[i]] = 1;
  }
  if (ra + rb - 2 * n_axes > 30) return fail(TOGB_ERR_UNSUPPORTED, "output rank above 30");
  JoinDesc jd;
  std::memset(&jd, 0, sizeof(jd));
  std::vector<int> afree, bfree;
  for (int i = 0; i < ra; ++i) if (!in_a[i]) afree.push_back(i);
  for (int i = 0; i < rb; ++i) if (!in_b[i]) bfree.push_back(i);
  jd.mb = (int)afree.size();
  jd.nb = (int)bfree.size();
  jd.kb = n_axes;
  // LSB-first: the last free axis of each operand is the lowest GEMM bit, so
  // C[m][n] row-major is np.tensordot's output order.
  for (int i = 0; i < jd.mb; ++i) jd.a.s_outer[i] = pow2(ra - 1 - afree[jd.mb - 1 - i]);
  for (int i = 0; i < jd.nb; ++i) jd.b.s_outer[i] = pow2(rb - 1 - bfree[jd.nb - 1 - i]);
  int64_t pa = 0, pb = 0, mina = INT64_MAX, minb = INT64_MAX, mino_a = INT64_MAX, mino_b = INT64_MAX;
  for (int i = 0; i < n_axes; ++i) {
    const int src = n_axes - 1 - i;
    jd.a.s_k[i] = pow2(ra - 1 - axes_a[src]);
    jd.b.s_k[i] = pow2(rb - 1 - axes_b[src]);
    jd.a.dk[i] = jd.a.s_k[i] - pa; pa += jd.a.s_k[i];
    jd.b.dk[i] = jd.b.s_k[i] - pb; pb += jd.b.s_k[i];
    mina = std::min(mina, jd.a.s_k[i]);
    minb = std::min(minb, jd.b.s_k[i]);
  }
  for (int i = 0; i < jd.mb; ++i) mino_a = std::min(mino_a, jd.a.s_outer[i]);
  for (int i = 0; i < jd.nb; ++i) mino_b = std::min(mino_b, jd.b.s_outer[i]);
  jd.a.k_fast = mina < mino_a;
  jd.b.k_fast = minb < mino_b;
  jd.a.outer_bits = jd.mb; jd.a.k_bits = jd.kb;
  jd.b.outer_bits = jd.nb; jd.b.k_bits = jd.kb;
  togb::make_runs(jd.a.s_outer, jd.mb, &jd.a.r_outer);
  togb::make_runs(jd.a.s_k, jd.kb, &jd.a.r_k);
  togb::make_runs(jd.b.s_outer, jd.nb, &jd.b.r_outer);
  togb::make_runs(jd.b.s_k, jd.kb, &jd.b.r_k);
  fill_ktab(jd.a);
  fill_ktab(jd.b);
  jd.a.ptr = a;
  jd.b.ptr = b;
  jd.a.batch_stride = pow2(ra);
  jd.b.batch_stride = pow2(rb);
  jd.c_ptr = out;
  jd.c_batch_stride = pow2(jd.mb + jd.nb);
  for (int i = 0; i < jd.nb; ++i) jd.c_s_n[i] = pow2(i);
  for (int i = 0; i < jd.mb; ++i) jd.c_s_m[i] = pow2(jd.nb + i);
  togb::make_runs(jd.c_s_m, jd.mb, &jd.r_cm);
  togb::make_runs(jd.c_s_n, jd.nb, &jd.r_cn);
  togb::make_inverse_runs(jd.c_s_m, jd.mb, &jd.r_inv_m);
  togb::make_inverse_runs(jd.c_s_n, jd.nb, &jd.r_inv_n);
  jd.c_natural = is_natural(jd);
  jd.wait_cycles = togb::kDefaultWaitCycles;
  const int kernel = choose_kernel(jd.mb, jd.nb, jd.kb);
  cudaError_t e = togb::launch_join(mode, kernel, jd, nullptr, 1, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "tensordot launch");
  return TOGB_OK;
}

}  // namespace

togb_status togb_tensordot_f64(const double* a, int32_t ra, const double* b, int32_t rb, int32_t n_axes,
                               const int32_t* axes_a, const int32_t* axes_b, double* out, void* stream) {
  return tensordot_join(TOGB_MODE_F64, a, ra, b, rb, n_axes, axes_a, axes_b, out, stream);
}

togb_status togb_tensordot_i64(const int64_t* a, int32_t ra, const int64_t* b, int32_t rb, int32_t n_axes,
                               const int32_t* axes_a, const int32_t* axes_b, int64_t* out, void* stream) {
  return tensordot_join(TOGB_MODE_INT64, a, ra, b, rb, n_axes, axes_a, axes_b, out, stream);
}

togb_status togb_probe_peak(int kind, void* stream, double* flops) {
  if (!flops || kind < 0 || kind > 3) return fail(TOGB_ERR_INVALID, "bad probe arguments");
  cudaError_t e = kind == 3 ? togb::probe_umma((cudaStream_t)stream, flops)
                            : togb::probe_peak(kind, (cudaStream_t)stream, flops);
  if (e != cudaSuccess) return cuda_fail(e, "peak probe");
  return TOGB_OK;
}

}  // extern "C"

// Contraction of a whole program in FP64 with every intermediate inside a
// caller-supplied scratch region (the library's static device array).  Layout:
// [slice base, 256 B][accumulator: 2 * 2^root_rank doubles, rounded up to
// 256 B][workspace: slice-invariant part, then per-slice part * chunk].  No
// device memory is allocated.
togb_status togb::static_contract_f64(const togb_program_desc* d, const double* d_leaf, char* scratch,
                                      size_t scratch_bytes, double* d_out, cudaStream_t st) {
  togb_program* p = nullptr;
  int64_t nvals = 0;
  togb_status r = lower_host(d, 0, &p, &nvals);
  if (r != TOGB_OK) return r;
  p->allow_fused_once = false;  // the slice-invariant arena reuses memory: smallest scratch
  plan_arena(p);
  const int64_t E = pow2(p->nodes[p->root].rank);
  const int64_t head = 256 + (2 * E * 8 + 255) / 256 * 256;
  const int64_t per = ws_per_slice(p, TOGB_MODE_F64);
  const int64_t once = ws_once(p, TOGB_MODE_F64);
  if (head + once + per > (int64_t)scratch_bytes) {
    const std::string msg = "program needs " + std::to_string(head + once + per) +
                            " bytes of device scratch for one slice; the static scratch holds " +
                            std::to_string(scratch_bytes) + " bytes";
    delete p;
    return fail(TOGB_ERR_OOM, msg);
  }
  const int64_t B = std::min<int64_t>({((int64_t)scratch_bytes - head - once) / per, p->num_slices, 65535});
  p->d_leaf64 = const_cast<double*>(d_leaf);
  p->d_s0 = (int64_t*)scratch;
  p->d_acc = (double*)(scratch + 256);
  build_descs(p, TOGB_MODE_F64, scratch + head, (int)B);
  p->cur_B = (int)B;
  togb_status out = TOGB_OK;
  cudaError_t e = cudaMemsetAsync(p->d_acc, 0, 2 * E * 8, st);
  if (e != cudaSuccess) out = cuda_fail(e, "accumulator clear");
  if (out == TOGB_OK) out = enqueue_phase(p, TOGB_MODE_F64, true, 1, st, nullptr);
  for (int64_t s = 0; out == TOGB_OK && s < p->num_slices; s += B) {
    const int nb = (int)std::min<int64_t>(B, p->num_slices - s);
    e = togb::launch_set_s0(p->d_s0, s, st);
    if (e != cudaSuccess) { out = cuda_fail(e, "slice base update"); break; }
    out = enqueue_phase(p, TOGB_MODE_F64, false, nb, st, nullptr);
  }
  if (out == TOGB_OK && (e = togb::launch_finalize(p->d_acc, E, d_out, st)) != cudaSuccess)
    out = cuda_fail(e, "result write");
  // Every device pointer above is borrowed; the host object owns none.
  delete p;
  return out;
}

togb_status togb::report(togb_status st, const char* msg) { return fail(st, msg); }
