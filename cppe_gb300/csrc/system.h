// One polarizable system on the GPU: geometry, operator data, the work
// buffers of the FP64 and mixed-precision solvers, and its stream.
#pragma once

#include <memory>

#include "engine.h"
#include "learned.h"

namespace cg {

// Scalar slots of the solver (device, FP64).
enum Scalar {
  S_RZ = 0,   // r . z of the current iterate
  S_PAP,      // p . Ap
  S_RR,       // r . r
  S_RZNEW,    // r' . z'
  S_BETA,     // beta
  S_RNORM,    // ||r||_2 after the last update
  S_TOL,      // stopping threshold of the running loop
  S_RZOLD,    // r . z before the last update (flexible CG)
  S_RED = 8,       // 4 slots receiving grid reductions
  S_RSTAGE = 12,   // ||r|| at the set-up of the running inner solve
  S_TOLF   = 13,   // final threshold of the running inner solve
  S_SW1    = 14,   // threshold handing over to inexact operator 1 (index 0)
  S_SW2    = 15,   //                        ... to inexact operator 2
  S_RSW1   = 16,   // ||r|| where the inner solve went over to inexact operator 1
  S_RSW2   = 17,   //                                      ... inexact operator 2
  S_NSCAL = 24
};

struct SolveStats {
  double final_rnorm = 0.0;
  int fp64_applies = 0, fp32_applies = 0, iterations = 0;
};

struct System {
  int n = 0;
  cppe_gpu_options opt{};
  int device = 0;
  cudaStream_t stream = nullptr;
  SideStream side;  // far-field passes, concurrent with the near field
  Geometry geo;
  std::unique_ptr<DeviceOps> ops;  // m = 1, p = order (FMM only)
  FieldWork<double> w64;
  FieldWork<float> w32;
  // Inexact inner operators of the mixed solver: the same tree walked with
  // larger opening angles (fewer near pairs), in FP32; inexact_delta[k]
  // bounds operator k's relative difference from the operator (measured at
  // set-up, times 3).  The inner solves go over to them, in order, once their
  // residual is small enough that the difference stays below what they must
  // resolve.  n_inexact counts the operators in use (a prefix).
  static constexpr int NINEXACT = 2;
  Geometry geo_x[NINEXACT];
  FieldWork<float> w32x[NINEXACT];
  int n_inexact = 0;
  double inexact_delta[NINEXACT] = {0.0, 0.0};
  int apply_level = -1;  // apply32 uses geo_x[apply_level] (set while capturing)
  void setup_inexact(const double* xyz, const double* sd);
  // operator data in device order
  DBuf<double> ainv64, alpha64;  // 6 per site
  DBuf<float> ainv32, alpha32;
  // solver vectors (device order, 3n)
  DBuf<double> F, x, r, z, p, Ap, tmp_in, tmp_out;
  DBuf<float> r32, z32, p32, Ap32, d32;
  DBuf<double> scal, partials, hist;
  DBuf<unsigned> ticket;
  DBuf<int> flags;  // [0] done, [1] iteration counter
  int* h_flags = nullptr;     // pinned mirror
  double* h_scal = nullptr;   // pinned mirror
  SolveStats last;
  std::vector<int> excl_ptr_h, excl_idx_h;  // caller-order exclusions (dense matrix)

  // learned initial guess + preconditioner correction (optional, not owned)
  Mlp* model = nullptr;
  bool use_model = false;  // set while a learned solve runs
  std::unique_ptr<NearList> near;
  DBuf<float> lf_feats, lf_v1, lf_v2, lf_v3, lf_Y, lf_c, lf_w32, lf_rold32;
  DBuf<double> lf_w64, lf_rold64;
  DBuf<float4> lf_z4;  // z of the FP32 inner solve as float4 per site (gathers)
  // device copies for the host-buffer solve entry point (kept between calls:
  // a cudaMalloc/cudaFree pair per solve costs about as much as the copies)
  DBuf<double> io_rhs, io_guess, io_mu;
  void learned_setup();
  // descriptors and basis vectors for the current F (device order)
  void learned_features_for_F();
  // x = learned guess, lf_c = preconditioner weights
  void learned_start();
  // z correction after a CG start/update (flexible CG)
  // returns the corrected preconditioned residual (the z the CG continues with)
  template <typename T>
  T* learned_precond(T* z, const T* r, T* p, bool start);
  // training rows for rhs F (device order) and converged mu (device order)
  void learned_rows(const double* mu_star_dev, std::vector<float>& feats,
                    std::vector<float>& rows);

  ~System();
  void init(int n, const double* xyz, const double* alpha6, const int* excl_ptr,
            const int* excl_idx, const cppe_gpu_options& o);
  // FP64 / FP32 operator on device-order vectors.
  // near_mode (NearMode): the plain FP64 solver keeps NEAR_FP64; the mixed
  // solver's residuals use the double-float near field (NEAR_DD)
  void apply64(const double* in, double* out, bool with_dot, int near_mode = NEAR_FP64);
  void apply32(const float* in, float* out, bool with_dot);
  // FP32 operator on FP64 device-order vectors (rounded in, widened out).
  void apply32_widen(const double* in, double* out);
  ReduceSlots slots(int k) const;
  // Average device time (ms) per phase of `reps` applies: near field, P2M+M2M,
  // M2L, L2L, finishing pass, whole apply.
  void phase_timings(int precision, int reps, double* ms);
  // solves in device order: F holds the rhs, x the start vector
  int solve_fp64(bool zero_guess, double* hist_out, int hist_cap, int* iters);
  int solve_mixed(bool zero_guess, double* hist_out, int hist_cap, int* iters);
  // Times the FP32 apply for a few near-field work-item sizes and M2L chunk
  // sizes and keeps the fastest schedule; returns its apply time (ms).
  double autotune(int reps);
  // Sets the schedule directly: FP32 near-field form (0 per target leaf, 1 or
  // 2 packed source pairs a lane of the symmetric kernel; -1 keeps it), the
  // near-field work-item size in pairs and the M2L chunk (<= 0 keep them).
  void set_schedule(int near_form, long item_pairs, int m2l_chunk);
  void size_work_buffers();
  // inner FP32 PCG loop of the mixed solver (graph-launched when possible)
  void inner_iteration_fp32(int nb, int nb3);
  void run_inner_fp32(int nb, int nb3);
  // builds the inner loop's graph on first use; false where graphs are off
  bool inner_graph_ready(int nb, int nb3, int level = -1);
  // [plain / learned body][operator, inexact operator 1, 2]
  cudaGraphExec_t inner_exec[2][1 + NINEXACT] = {};
  long long inner_body_launches[2][1 + NINEXACT] = {};
  bool inner_graph_failed = false;
  int solve_device(const double* d_rhs, const double* d_guess, int make_guess, double* d_mu,
                   int* iters, double* hist_out, int hist_cap);
};

}  // namespace cg
