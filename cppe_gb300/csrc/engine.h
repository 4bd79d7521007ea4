// The field engine: evaluates F_i = sum_j field(r_i - r_j; S_j) over the
// sites of one system, by direct summation or by the reference's FMM, on one
// CUDA stream.  Sites live on the device in a fixed permuted order (leaf-
// contiguous for FMM, caller order for direct summation).
#pragma once

#include <functional>
#include <memory>
#include <vector>

#include "common.cuh"
#include "fmm_ops.h"
#include "tree.h"

namespace cg {

struct TreeView {
  int n, ncells, nleaves;
  const double4_32a* center;  // x, y, z, r
  const int* parent;
  const int* child_ptr;
  const int* child_idx;
  const int* is_leaf;
  const int* leaf_cell;
  const int* leaf_start;
  const int* site_leaf;  // leaf of each (permuted) site
  const int* m2l_ptr;
  const int* m2l_src;
  const int* p2p_ptr;
  const int* p2p_src;
  // expansion centres relative to a reference site of each cell (FP32 path):
  // c - x_q = cell_off[c] + (x_ref(c) - x_q), the last term from hi/lo
  const float4* cell_off;
  const int* cell_ref;
  // per leaf: the cells on its path to the root that receive M2L terms
  const int* lanc_ptr;
  const int* lanc_cell;
};

struct OpsView {
  int m, p, msize, lsize, nt, nm2l_terms, nl2p;
  const int* exps;
  const int *p2m_ptr, *p2m_k, *p2m_j;
  const int *m2m_ptr, *m2m_k, *m2m_j;
  const int *l2l_ptr, *l2l_k, *l2l_j;
  const int *l2p_c, *l2p_n, *l2p_j;
  const int* m2l_kw;  // k | w << 16
  const int* slots;
  const int* row_slot_ptr;
  const int* row_slot_id;
  const int* drec;
};

// Site coordinates as the kernels read them (permuted order).
struct SiteView64 {
  const double4_32a* pos;  // x, y, z, s = alpha_iso^(-1/6) (0: no damping partner)
};
struct SiteView32 {
  const float4* hi;  // float(x), float(y), float(z), s
  const float4* lo;  // x - hi, ...  (hi + lo carries ~48 bits of each coordinate)
};

struct DeviceOps {
  OpTables host;
  DBuf<int> exps, p2m_ptr, p2m_k, p2m_j, m2m_ptr, m2m_k, m2m_j, l2l_ptr, l2l_k, l2l_j, l2p_c,
        l2p_n, l2p_j, m2l_kw, slots, row_slot_ptr, row_slot_id, drec;
  void build(int m, int p, cudaStream_t s);
  OpsView view() const;
};

// Distinct centre differences of a tree's M2L list entries (target minus
// source, on the grid of half the deepest half-width): vid[q] indexes vec for
// list entry q.  False (and empty outputs) where a difference is off the grid.
bool m2l_vectors(const TreeLayout& L, std::vector<int>& vid, std::vector<double4_32a>& vec);

// Row stride (coefficients) of the multipole storage of the fixed-order
// expansion kernels: the coefficient count rounded up to a multiple of four,
// so that rows start on 16-byte boundaries.
__host__ __device__ constexpr int m_stride(int ms) { return (ms + 3) & ~3; }

constexpr int M2L_CHUNK = 64;  // built-in sources of one target cell per M2L warp

// Geometry: the sites, their permutation and the interaction structure.
struct Geometry {
  int n       = 0;
  bool fmm    = false;
  int ncrit   = 64;
  double theta = 0.5;
  TreeLayout layout;
  std::vector<int> level_start;
  DBuf<double> center;
  DBuf<int> parent, child_ptr, child_idx, is_leaf, leaf_cell, leaf_start, site_leaf, m2l_ptr,
        m2l_src, p2p_ptr, p2p_src;
  DBuf<int> perm, inv_perm;  // perm[k] = caller index of site k
  DBuf<double4_32a> pos64;
  DBuf<float4> hi32, lo32;
  DBuf<float2> dd_exp;  // e^-(k/16), k = 0..320, as double-float pairs
  // pairs the reference skips (exclusions) that the near-field pass computed
  DBuf<int> corr_ptr, corr_idx;
  long near_pairs = 0;  // ordered pairs evaluated by the near-field pass
  long alg_pairs  = 0;  // of these, the pairs the reference evaluates

  // Near-field work items (target leaf, first and last+1 position in its
  // P2P list, output slot), largest first; a leaf's items write slots
  // 0..leaf_nslot-1 of the near-field buffer.  A leaf's P2P list holds the
  // source leaves that may need Thole damping first and those that do not
  // (every pair with v >= 27) from h_leaf_split[leaf] on; item_split is
  // that position clamped to each item's range.
  int nslot = 1;
  std::vector<int4> h_items;
  std::vector<int> h_leaf_nslot, h_leaf_split, h_item_split;
  DBuf<int4> items;
  DBuf<int> leaf_nslot, item_split;
  // Symmetric near field (single systems, FP32 dipole sources): P2P lists
  // are symmetric, so every unordered leaf pair is evaluated once, by an item
  // of the lower-numbered leaf A over its "upper" list (partners B >= A,
  // damping class first; B = A is the self leaf, evaluated one way).  An item
  // writes its targets' fields to its row of A and each partner's fields to
  // that partner's row for this item; leaf L owns sym_leaf_rows[L] rows of
  // 3 n_L floats from float offset sym_leaf_off[L], and the finishing pass adds
  // them in row order (fixed at set-up: deterministic, no atomics).
  std::vector<int> h_usrc, h_sym_split;
  std::vector<long long> h_usrc_off, h_sym_aoff, h_sym_leaf_off;
  std::vector<int4> h_sym_items;  // {A, first, last, 0} in the upper list
  std::vector<int> h_sym_leaf_rows;
  long long sym_floats = 0;       // size of the row buffer
  DBuf<int> usrc, sym_split, sym_leaf_rows;
  DBuf<long long> usrc_off, sym_aoff, sym_leaf_off;
  DBuf<int4> sym_items;
  bool sym_enabled = true;  // the schedule autotuner may switch it off
  int sym_pack     = 1;     // packed source pairs per lane of the symmetric kernel (1 or 2)
  bool has_sym() const { return !h_sym_items.empty(); }
  void make_sym_schedule(long W);

  // Distinct M2L translation vectors.  Cell centres lie on the tree's grid,
  // so the centre differences of the M2L list entries take few distinct
  // values (about 5,000 for 300,000 sites against 14.7 M entries): m2l_vid
  // gives each list entry's vector, vec the vectors, and the derivative
  // tensors of 1/R are tabulated once per vector (FieldWork::dtab*).  Empty
  // where the lists come from several trees (a batch) or a difference is off
  // the grid: the M2L then builds each tensor itself.
  std::vector<int> h_m2l_vid;
  std::vector<double4_32a> h_vec;
  DBuf<int> m2l_vid;
  DBuf<double4_32a> vec;
  void make_vectors();

  // Batches whose snapshots repeat once per right-hand side (ncopies):
  // the copy of each leaf's segment, the sites and leaves between copies,
  // and the items of the copy-0 leaves, which one near-field pass runs for
  // every copy (k_p2p32_m1_multi).
  int ncopies = 1;
  std::vector<int> h_leaf_copy;
  std::vector<int2> h_leaf_cstride;
  std::vector<int4> h_mitems;
  std::vector<int> h_mitem_split;
  std::vector<int2> h_mitem_stride;
  DBuf<int4> mitems;
  DBuf<int> mitem_split;
  DBuf<int2> mitem_stride;

  // Segment of each leaf and cell where several systems share one geometry
  // (a batch; empty otherwise): an evaluation given the segments' done flags
  // skips the near-field items, leaf multipoles and M2L chunks of finished
  // segments.
  std::vector<int> h_leaf_seg, h_cell_seg;
  DBuf<int> leaf_seg, cell_seg;

  // Upward pass without level-by-level M2M: leaf multipoles (P2M), then the
  // multipole of every non-leaf cell that is an M2L source from M2M shifts of
  // its subtree's leaf multipoles straight to its centre, in tasks
  // {cell, first, last} over task_leaf[] (<= 8 leaves per task);
  // cell_task_ptr (CSR over cells) lists a cell's tasks, whose partial
  // expansions are summed in order.  The downward pass shifts the M2L-only
  // local expansions of the cells on each leaf's path to the root (lanc_*)
  // straight to the leaf centre, in place of level-by-level L2L: both are
  // exact re-expansions of the same polynomials, so the operator is unchanged.
  std::vector<int4> h_p2m_tasks;
  std::vector<int> h_task_leaf, h_cell_task_ptr, h_lanc_ptr, h_lanc_cell, h_cell_ref;
  // M2L work: chunks {cell, first, last} of the cells' source lists (warp each)
  std::vector<int4> h_m2l_chunks;
  std::vector<int> h_cell_chunk_ptr;
  DBuf<int4> m2l_chunks;
  DBuf<int> cell_chunk_ptr;
  std::vector<float4> h_cell_off;
  DBuf<int4> p2m_tasks;
  DBuf<int> task_leaf, cell_task_ptr, lanc_ptr, lanc_cell, cell_ref;
  DBuf<float4> cell_off;
  // Thole damping factor of the operator (0: undamped), for the damping
  // split of the P2P lists
  double damping = 0.0;
  // tunable schedule parameters (0: the built-in choice)
  long item_pairs = 0;  // target pairs per near-field work item
  int m2l_chunk   = 0;  // sources per M2L warp
  int multi_tile  = 0;  // source pairs per tile of a batch's multi-RHS near field (96/120/144)
  int multi_copies = 0;  // right-hand sides per pass of it (4 or 8; 0: 8)
  // builds both schedules from `layout` and h_pos64
  void make_schedules();
  // re-uploads what make_schedules changes (near-field items, M2L chunks)
  void upload_schedules(cudaStream_t s);

  // host copies of the device arrays that are not part of `layout`
  std::vector<int> h_site_leaf, h_cptr, h_cidx;
  std::vector<double4_32a> h_pos64;
  std::vector<float4> h_hi, h_lo;

  // xyz in caller order; s_damp: alpha_iso^(-1/6) per site (0 = undamped partner);
  // exclusions in caller indices (CSR, may be null).
  void build(int n, const double* xyz, const double* s_damp, const int* excl_ptr,
             const int* excl_idx, bool fmm, int ncrit, double theta, cudaStream_t s);
  // host half of build(): layout, permuted coordinates, exclusion corrections
  void prepare(int n, const double* xyz, const double* s_damp, const int* excl_ptr,
               const int* excl_idx, bool fmm, int ncrit, double theta);
  void upload(cudaStream_t s);
  // Concatenates prepared geometries, each repeated `copies` times, into one
  // geometry whose passes cover all of them: cells are renumbered by (level,
  // part, cell), particles and leaves stay part-contiguous.  Direct-summation
  // parts contribute their chunks as level-0 cells without interaction lists.
  // The caller index of site i of copy r of part g is
  //   copies * site_offset[g] + r * n_g + i.
  static void combine(const std::vector<const Geometry*>& parts, int copies, Geometry& out);
  TreeView view() const;
  SiteView64 v64() const { return {pos64.p}; }
  SiteView32 v32() const { return {hi32.p, lo32.p}; }
};

// Work buffers of one (geometry, m, p, precision) evaluation.
template <typename T>
struct FieldWork {
  DBuf<T> M, L, Fnear, Mpart, Lleaf, Lpart;
  DBuf<T> Fsym;  // rows of the symmetric near field (Geometry::sym_*)
  DBuf<float2> dd_src;  // double-float copy of the sources (double-float pass)
  DBuf<float2> Mdd;     // double-float copy of the multipoles (double-float M2L)
  // derivative tensors of the geometry's M2L vectors, in T and in
  // double-float (built on first use)
  DBuf<T> dtab;
  DBuf<float2> dtab_dd;
};

// Output modes of the finishing pass.
enum FinishMode { FINISH_APPLY = 0, FINISH_FIELD = 1 };

// Per-launch scalar reduction slots (device).
struct ReduceSlots {
  double* partials;   // >= nblocks * 4 doubles
  unsigned* ticket;   // one counter, zero between uses
  double* out;        // receives the totals
  // when set, the per-site values are stored here instead of being summed
  // (segmented reductions of batched solves add them per segment)
  double* site_values = nullptr;
};

// Evaluates the field of sources `src` (ns = ncomp(m) values per permuted
// site, precision T).  FINISH_APPLY: out (T, 3n) = F + ainv6 . src and, when
// dot != nullptr, dot->out[0] = sum_i src_i . out_i (FP64).  FINISH_FIELD:
// out64 (double, 3n) += sign * F.
// Optional phase markers: recorded on the stream at the start, after P2M+M2M,
// after M2L, after L2L, after the near-field pass and after the finishing pass.
struct PhaseEvents {
  cudaEvent_t ev[6];
};

// A second stream for the far-field passes (P2M, M2M, M2L, L2L), which run
// concurrently with the near-field pass and join before the finishing pass.
struct SideStream {
  cudaStream_t s     = nullptr;  // the stream in use: hi (default) or lo
  cudaStream_t hi    = nullptr;  // highest priority
  cudaStream_t lo    = nullptr;  // lowest priority (that of the default stream)
  cudaEvent_t fork   = nullptr;
  cudaEvent_t join   = nullptr;
  void create();
  void destroy();
  void use_high_priority(bool h) { s = h ? hi : lo; }
};

// Arithmetic of the near-field pass of an FP64 evaluation.
enum NearMode {
  NEAR_FP64     = 0,  // native FP64 throughout
  NEAR_FAST_EXP = 1,  // FP64, FP32 exponential where the damping argument is >= 20
  NEAR_DD       = 2   // double-float on the FP32 pipe (dipole sources; others use FAST_EXP);
                      // the fixed-order M2L runs in double-float too
};

template <typename T>
void eval_field(const Geometry& g, const DeviceOps* ops, FieldWork<T>& w, int m, const T* src,
                bool damp, double damping, FinishMode mode, const T* ainv6, T* out,
                double* out64, double sign, const ReduceSlots* dot, cudaStream_t s,
                const PhaseEvents* pe = nullptr, int near_mode = NEAR_FP64,
                const SideStream* side = nullptr, const int* seg_done = nullptr);

// Times `apply` (one FP32 operator application ordered on `stream`) under
// three near-field work-item sizes and, with FMM, three M2L chunk sizes;
// keeps the fastest schedule in g (uploaded), then picks the priority of the
// far-field stream under it.  Returns the best apply time (ms).  The operator
// does not change, only how its work is cut into launches.
double autotune_schedule(Geometry& g, SideStream& side, cudaStream_t stream, int reps,
                         const std::function<void()>& apply);

// Permutation helpers (caller order <-> device order), all 3-vectors.
void permute_in(const Geometry& g, const double* in_caller, double* out_perm, int ncomp,
                cudaStream_t s);
void permute_out(const Geometry& g, const double* in_perm, double* out_caller, int ncomp,
                 cudaStream_t s);

}  // namespace cg
