// Batched solves over many (snapshot, right-hand side) segments at once.
#pragma once

#include <memory>
#include <type_traits>

#include "system.h"

namespace cg {

struct BatchSystem {
  int nrhs = 1, nseg = 0, n = 0;
  cppe_gpu_options opt{};
  int device          = 0;
  cudaStream_t stream = nullptr;
  SideStream side;  // far-field passes, concurrent with the near field
  std::vector<int> sys_sites;  // site offsets of the snapshots (caller layout)
  Geometry geo;                // all segments concatenated
  std::unique_ptr<DeviceOps> ops;
  FieldWork<double> w64;
  FieldWork<float> w32;
  DBuf<double> ainv64, alpha64;
  DBuf<float> ainv32, alpha32;
  DBuf<int> seg_start, site_seg;
  DBuf<double> F, x, r, z, p, Ap;
  DBuf<float> r32, z32, p32, Ap32, d32;
  DBuf<double> site_a, site_b;  // per-site values of the segmented dots
  DBuf<double> seg_rz, seg_pap, seg_rr, seg_rznew, seg_beta, seg_rnorm, seg_tol;
  DBuf<int> done, iters, active;
  int* h_active = nullptr;
  // Inexact inner operators of the mixed solver (FMM snapshots): the same
  // segments at the single-system solver's opening angles 0.6 and 0.8, a
  // per-segment level set on the device from the segment's residual, and
  // each operator applied to the segments at its level only.
  static constexpr int NINEXACT = 2;
  int n_inexact = 0;
  Geometry geo_x[NINEXACT];
  FieldWork<float> w32x[NINEXACT];
  std::vector<double> h_delta[NINEXACT];  // per segment: operator difference bound (0: off)
  DBuf<double> seg_sw[NINEXACT];          // hand-over residuals of the running inner solve
  DBuf<double> seg_rsw[NINEXACT];         // residual where the segment handed over (0: not)
  DBuf<int> seg_level;                    // 0: the operator, 1 + k: inexact operator k
  DBuf<int> lvl_mask[1 + NINEXACT];       // per operator: segment finished or at another level
  SolveStats stats;
  std::vector<double> last_rnorm;

  ~BatchSystem();
  void init(int nsys, const int* site_offset, const double* xyz, const double* alpha6,
            const int* excl_ptr, const int* excl_idx, int nrhs, int direct_below,
            const cppe_gpu_options& o);
  // rhs / mu in the caller layout [system][rhs][3 n_s]; iters per segment.
  int solve_device(const double* d_rhs, double* d_mu, int* iters);

  template <typename T>
  FieldWork<T>& work() {
    if constexpr (std::is_same<T, double>::value)
      return w64;
    else
      return w32;
  }
  // the operator over every segment; skip_done leaves the near field of the
  // segments flagged in `done` out (their output is then not meaningful)
  template <typename T>
  void apply_seg(const T* in, T* out, int near_mode = NEAR_FP64, bool skip_done = false);
  // FP32 operator of inexact level k (0, 1) over the segments not in `mask`
  // (every segment when null); with a segmented dot of in and out in site_a
  void apply_level32(int k, const float* in, float* out, const int* mask);
  // the iteration's FP32 apply: each segment with the operator of its level
  void apply_levels32(const float* in, float* out);
  // the same inside a graph capture on `stream`: each operator's pass in a
  // conditional node that runs only when some segment is at its level (the
  // passes captured on if_stream, far field in line)
  void apply_levels32_graph(const float* in, float* out);
  // streams that capture nested bodies: a loop's body on cap_stream, the
  // per-level passes on if_stream (cap_stream, or cap_stream2 inside a loop
  // body that cap_stream captures)
  cudaStream_t cap_stream  = nullptr;
  cudaStream_t cap_stream2 = nullptr;
  cudaStream_t if_stream   = nullptr;
  // set while a loop body nested in a larger capture is captured: the
  // operator passes then keep their far field in line (no side stream)
  bool nested_body = false;
  DBuf<double> seg_delta_d[NINEXACT];  // h_delta on the device
  // The usual course of a mixed solve -- start residual, first inner solve,
  // double-float residual, second inner solve, residual from the recursion
  // -- as one CUDA graph with the inner solves as conditional while nodes:
  // one launch and one host synchronisation per solve; the host loop takes
  // over where the course does not end the solve.
  cudaGraphExec_t course_exec = nullptr;
  bool course_failed          = false;
  long long course_launches   = 0;  // launches captured outside the inner loops
  long long course_body_launches = 0;  // launches captured into one inner iteration
  // host synchronisations with the stream in the last solve
  int host_waits = 0;
  void host_wait();
  DBuf<int> iters_first;     // the first inner solve's iterations per segment
  DBuf<double> rn_second;    // residual norms at the second inner solve's start
  bool course_graph_ready(int maxiter);
  void course_body(int maxiter);
  // a conditional while node after the capture's tip on `stream`, with one
  // FP32 PCG iteration captured into its body
  void capture_pcg_loop(int maxiter);
  // measures each segment's difference between the operator and the
  // inexact ones (part of init, after the inexact geometries are built)
  void measure_inexact(const std::vector<int>& seg_start_h, const std::vector<char>& seg_fmm);
  // PCG iterations over all segments until each has converged or reached
  // maxiter; returns the number of iterations run (operator applications)
  template <typename T>
  int run_pcg(T* x, T* r, T* z, T* p, T* Ap, const T* a6, int maxiter);
  template <typename T>
  void pcg_iteration(T* x, T* r, T* z, T* p, T* Ap, const T* a6, int maxiter, bool graph);
  void seg_norms_from_site_b();
  // The iterations as one CUDA graph with a conditional while node, per
  // precision ([FP64, FP32]); built on first use, dropped when the schedule
  // changes.  CPPE_GPU_GRAPHS=0 or a refused construction launches the
  // iterations from the host.
  template <typename T>
  bool pcg_graph_ready(T* x, T* r, T* z, T* p, T* Ap, const T* a6, int maxiter);
  cudaGraphExec_t pcg_exec[2] = {};
  long long pcg_body_launches[2] = {};
  bool pcg_graph_failed = false;
  std::vector<int> h_iters;
  // Times the FP32 operator under several near-field work-item sizes, M2L
  // chunk sizes and far-field stream priorities and keeps the fastest;
  // returns its apply time (ms).
  double autotune(int reps);
};

}  // namespace cg
