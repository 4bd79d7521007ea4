/*
 * cppe_gpu.h -- C ABI of the GB300 (sm_103a) induced-dipole library.
 *
 * Plain pointers and sizes only.  Every function returns a cppe_gpu_status;
 * cppe_gpu_last_error() gives the message of the last failure on the calling
 * thread.  Host buffers are read/written synchronously unless the name ends in
 * _device, in which case the pointers are device pointers on the handle's
 * device and the call is ordered on the handle's stream.
 *
 * Vectors follow the reference layout: site-major xyz, 3*n doubles, sites in
 * the caller's (polarizable-site) order.  alpha6 holds the polarizability
 * upper triangle xx,xy,xz,yy,yz,zz per site (Polarizability,
 * src/core/potential.hh:45-72).  Exclusions are a CSR list of 0-based site
 * indices (Potential::m_exclusions, potential.hh:79); as in the reference they
 * are compared against polarizable-site indices (tree.cc:145).
 *
 * Reference interfaces each entry point replaces (maxscheurer/cppe):
 *   cppe_gpu_create / destroy        BMatrix::BMatrix        src/core/bmatrix.hh:19-36
 *                                    InducedMoments ctor     src/core/electric_fields.hh:62-66
 *   cppe_gpu_bmatrix_apply[_device]  BMatrix::apply          src/core/bmatrix.cc:9-40
 *   cppe_gpu_apply_diagonal          BMatrix::apply_diagonal src/core/bmatrix.cc:53-62
 *   cppe_gpu_apply_diagonal_inverse  BMatrix::apply_diagonal_inverse src/core/bmatrix.cc:42-51
 *   cppe_gpu_to_dense                BMatrix::to_dense_matrix src/core/bmatrix.cc:64-92
 *   cppe_gpu_direct_inverse          BMatrix::direct_inverse src/core/bmatrix.cc:94-97
 *   cppe_gpu_solve[_device]          InducedMoments::compute src/core/electric_fields.cc:191-239
 *   cppe_gpu_multipole_fields        MultipoleFields::compute src/core/electric_fields.cc:106-189
 *   cppe_gpu_charge_fields           NuclearFields::compute  src/core/electric_fields.cc:58-75
 *   cppe_gpu_multipole_potential_energy
 *                                    MultipoleExpansion::interaction_energy
 *                                                            src/core/multipole_expansion.cc:10-33
 *   cppe_gpu_potfile_*               PotfileReader::read     src/core/potfile_reader.cc:31-179
 *   cppe_gpu_charge_field_gradient   NuclearFields::nuclear_gradient
 *                                                            src/core/electric_fields.cc:77-104
 *   cppe_gpu_multipole_energy_gradient
 *                                    MultipoleExpansion::nuclear_gradient
 *                                                            src/core/multipole_expansion.cc:35-62
 *   cppe_gpu_tree_info               build_shared_tree + interact_dehnen_lazy
 *                                    src/core/fmm/tree.cc:134-237, calculate.cc:74-127
 *                                    (host-only; no GPU needed)
 *   cppe_gpu_batch_*                 no single counterpart: many InducedMoments::compute
 *                                    calls (snapshots x right-hand sides) in one launch
 */
#ifndef CPPE_GPU_H
#define CPPE_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  CPPE_GPU_OK            = 0,
  CPPE_GPU_NOT_CONVERGED = 1, /* "Failed to converge induced dipole moments." */
  CPPE_GPU_INVALID_ARG   = 2,
  CPPE_GPU_CUDA_ERROR    = 3,
  CPPE_GPU_TIMEOUT       = 4,
  CPPE_GPU_NO_DEVICE     = 5
} cppe_gpu_status;

/* Summation schemes (PeOptions::summation_induced_fields, pe_options.hh:28-29):
 * any string other than "fmm" means direct summation (bmatrix.cc:31-36). */
enum { CPPE_GPU_DIRECT = 0, CPPE_GPU_FMM = 1 };

/* Arithmetic of the solve (no counterpart in PeOptions; GPU-only knob).
 *   FP64  : every apply, dot and update in FP64 (the reference's arithmetic).
 *   MIXED : inner PCG in FP32 (pair kernels, FMM, apply) with FP64 dots;
 *           FP64 residual recomputation and iterative refinement outside;
 *           convergence is still ||F - B x||_2 < induced_thresh in FP64. */
enum { CPPE_GPU_FP64 = 0, CPPE_GPU_MIXED = 1 };

typedef struct {
  int summation;             /* CPPE_GPU_DIRECT or CPPE_GPU_FMM               */
  int tree_ncrit;            /* PeOptions::tree_ncrit            (default 64)  */
  int tree_expansion_order;  /* PeOptions::tree_expansion_order  (default 5)   */
  double theta;              /* PeOptions::theta                 (default 0.5) */
  int damp;                  /* PeOptions::damp_induced          (default 0)   */
  double damping_factor;     /* PeOptions::damping_factor_induced (2.1304)     */
  double induced_thresh;     /* PeOptions::induced_thresh        (1e-8)        */
  int maxiter;               /* PeOptions::maxiter               (50)          */
  int precision;             /* CPPE_GPU_FP64 or CPPE_GPU_MIXED                */
  int device;                /* CUDA device ordinal                            */
} cppe_gpu_options;

typedef struct cppe_gpu_system cppe_gpu_system;

/* Fills opts with the reference defaults (pe_options.hh:17-33). */
void cppe_gpu_default_options(cppe_gpu_options* opts);

/* Message of the last failure on this thread (always NUL-terminated). */
int cppe_gpu_last_error(char* buf, size_t len);

/* Number of visible CUDA devices (0 when there is none). */
int cppe_gpu_device_count(int* count);

/* One polarizable system: n sites, positions (bohr), polarizabilities and
 * exclusions.  Builds the octree and interaction lists once (for FMM) and
 * uploads everything; later applies/solves reuse it. */
int cppe_gpu_create(int n, const double* xyz, const double* alpha6, const int* excl_ptr,
                    const int* excl_idx, const cppe_gpu_options* opts,
                    cppe_gpu_system** out);
int cppe_gpu_destroy(cppe_gpu_system* sys);

/* out = B in, B = alpha^-1 - T (T: (Thole-damped) dipole field tensor). */
int cppe_gpu_bmatrix_apply(cppe_gpu_system* sys, const double* in, double* out);
int cppe_gpu_bmatrix_apply_device(cppe_gpu_system* sys, const double* d_in, double* d_out);
/* Same operator in FP32 arithmetic (inputs/outputs still FP64). */
int cppe_gpu_bmatrix_apply_fp32(cppe_gpu_system* sys, const double* in, double* out);
/* Same operator as the mixed solver evaluates its FP64 residuals: near-field
 * pairs in double-float arithmetic on the FP32 pipe (about 1e-13 relative per
 * pair), FMM passes and the finishing pass in FP64. */
int cppe_gpu_bmatrix_apply_dd(cppe_gpu_system* sys, const double* in, double* out);
int cppe_gpu_apply_diagonal(cppe_gpu_system* sys, const double* in, double* out);
int cppe_gpu_apply_diagonal_inverse(cppe_gpu_system* sys, const double* in, double* out);
/* Dense 3n x 3n B (row-major), and its inverse. */
int cppe_gpu_to_dense(cppe_gpu_system* sys, double* out);
int cppe_gpu_direct_inverse(cppe_gpu_system* sys, double* out);

/* Induced dipoles: solves B mu = rhs to ||rhs - B mu||_2 < induced_thresh.
 * guess may be NULL; make_guess != 0 uses alpha * rhs (electric_fields.cc:198-202).
 * iters receives the number of recorded residual norms and rnorm_hist
 * (capacity hist_cap, may be NULL) the norms themselves: in FP64 one per CG
 * iteration, exactly the values the reference prints; in MIXED one per FP64
 * refinement residual (the FP32 inner iterations are counted by
 * cppe_gpu_last_solve_stats).  Returns CPPE_GPU_NOT_CONVERGED after maxiter. */
int cppe_gpu_solve(cppe_gpu_system* sys, const double* rhs, const double* guess,
                   int make_guess, double* mu, int* iters, double* rnorm_hist,
                   int hist_cap);
int cppe_gpu_solve_device(cppe_gpu_system* sys, const double* d_rhs, const double* d_guess,
                          int make_guess, double* d_mu, int* iters, double* rnorm_hist,
                          int hist_cap);
/* Final FP64 residual norm and number of FP64 / FP32 operator applications of
 * the last solve on this handle. */
int cppe_gpu_last_solve_stats(cppe_gpu_system* sys, double* final_rnorm, int* fp64_applies,
                              int* fp32_applies);

/* Static multipole field at all n sites (MultipoleFields::compute): +F(q)
 * -F(mu) +F(theta') with theta' = quadrupoles with halved diagonal; q (n),
 * mu (3n), quad (6n, xx,xy,xz,yy,yz,zz, traceless) may be NULL when max_order
 * is lower.  polarizable/alpha_iso give the Thole damping partners (damp != 0).
 * summation/ncrit/order/theta as in cppe_gpu_options. */
int cppe_gpu_multipole_fields(int n, const double* xyz, const double* q, const double* mu,
                              const double* quad, int max_order, const int* polarizable,
                              const double* alpha_iso, const int* excl_ptr,
                              const int* excl_idx, int summation, int ncrit, int order,
                              double theta, int damp, double damping_factor, int device,
                              double* F);

/* Field of point charges (charges q at xyz_src, nsrc of them) at ntgt points:
 * F_i = sum_k q_k (r_i - R_k)/|r_i - R_k|^3 (NuclearFields::compute). */
int cppe_gpu_charge_fields(int ntgt, const double* xyz_tgt, int nsrc, const double* xyz_src,
                           const double* q, int device, double* F);

/* sum_atoms Z_a * phi_multipoles(R_a) (MultipoleExpansion::interaction_energy). */
int cppe_gpu_multipole_potential_energy(int n, const double* xyz, const double* q,
                                        const double* mu, const double* quad, int max_order,
                                        int natoms, const double* atom_xyz,
                                        const double* atom_charge, int device,
                                        double* energy);

/* Derivative of the point-charge fields at the ntgt targets with respect to
 * the nsrc charge positions (NuclearFields::nuclear_gradient,
 * src/core/electric_fields.cc:77-104): G is (3 nsrc) x (3 ntgt), row-major,
 * G[3a + c][3i + d] = q_a T2(r_i - R_a)_cd with T2 = grad grad 1/R. */
int cppe_gpu_charge_field_gradient(int ntgt, const double* xyz_tgt, int nsrc,
                                   const double* xyz_src, const double* q, int device,
                                   double* G);

/* Gradient of sum_atoms Z_a * phi_multipoles(R_a) with respect to the atom
 * positions (MultipoleExpansion::nuclear_gradient,
 * src/core/multipole_expansion.cc:35-62): grad is natoms x 3, row-major.
 * Multipoles up to order 2 (q, mu, quad as in
 * cppe_gpu_multipole_potential_energy). */
int cppe_gpu_multipole_energy_gradient(int n, const double* xyz, const double* q,
                                       const double* mu, const double* quad, int max_order,
                                       int natoms, const double* atom_xyz,
                                       const double* atom_charge, int device, double* grad);

/* Host-only potfile ingest (PotfileReader::read, src/core/potfile_reader.cc:
 * 31-179) straight into the arrays cppe_gpu_create and
 * cppe_gpu_multipole_fields take: same format, unit conversion (AA -> bohr),
 * quadrupole trace removal, zero defaults and error messages, with the
 * exclusion lists as CSR (0-based site indices, file order per site) instead
 * of per-site lists.  Multipoles up to order 2.  cppe_gpu_potfile_arrays
 * copies into caller buffers (any may be NULL): xyz 3n, q n, mu 3n, quad 6n
 * (xx,xy,xz,yy,yz,zz), alpha6 6n, polarizable n, excl_ptr n+1,
 * excl_idx nexcl, elements 4n (NUL-padded symbols). */
typedef struct cppe_gpu_potfile cppe_gpu_potfile;
int cppe_gpu_potfile_read(const char* path, cppe_gpu_potfile** out);
int cppe_gpu_potfile_info(const cppe_gpu_potfile* p, int* n, int* max_order, int* npolarizable,
                          long* nexcl);
int cppe_gpu_potfile_arrays(const cppe_gpu_potfile* p, double* xyz, double* q, double* mu,
                            double* quad, double* alpha6, int* polarizable, int* excl_ptr,
                            int* excl_idx, char* elements);
int cppe_gpu_potfile_free(cppe_gpu_potfile* p);

/* Host-only: octree and interaction-list sizes for a geometry (no GPU). */
int cppe_gpu_tree_info(int n, const double* xyz, int ncrit, double theta, int* ncells,
                       int* nleaves, long* nm2l, long* np2p, long* p2p_pairs);
/* Host-only: the interaction lists themselves in the reference's cell
 * numbering (creation order): m2l (nm2l x 2, (source, target)) and p2p
 * (np2p x 2, (target, source)). */
int cppe_gpu_tree_lists(int n, const double* xyz, int ncrit, double theta, int* m2l,
                        int* p2p);
/* Host-only: the number of distinct centre differences among the M2L list
 * entries (nentries), whose derivative tensors the FMM tabulates; -1 where a
 * difference is off the tree's grid (no table). */
int cppe_gpu_tree_vectors(int n, const double* xyz, int ncrit, double theta, int* nvec,
                          long* nentries);

/* Allocation-free direct-summation apply (no counterpart in the reference).
 * d_out = B d_in with direct summation in FP64, the operator of
 * cppe_gpu_bmatrix_apply for summation = CPPE_GPU_DIRECT, for callers that
 * cannot allocate GPU memory at this point: a host program that owns a fixed
 * device pool and forbids further cudaMalloc, or a real-time loop that must
 * not enter the allocator.  All pointers are device pointers the caller owns:
 * d_xyz (3n), d_alpha6 (6n), d_excl_ptr (n+1) / d_excl_idx (CSR exclusions,
 * both NULL for none), d_in and d_out (3n).  d_out must not overlap any input
 * buffer (CPPE_GPU_INVALID_ARG otherwise).  Excluded pairs are skipped, as in
 * the reference.  Two distinct, non-excluded sites at the same position make
 * the operator undefined; the output of such a site is NaN.  No cudaMalloc or
 * cudaFree is made; the only scratch is a fixed 1.75 MiB device array that
 * every GPU loading the library holds until exit, which limits n to 8192
 * (larger n returns CPPE_GPU_INVALID_ARG before any GPU work).  The work is
 * enqueued on `stream` (a cudaStream_t, NULL for the default stream) and not
 * synchronized.  The first call on a device looks the scratch address up with
 * that device current and keeps it for the life of the process (it does not
 * survive a cudaDeviceReset); make that first call before any stream capture.
 * Calls share the scratch, so calls that overlap on the GPU (different
 * streams, no ordering) race; calls ordered on one stream are safe. */
int cppe_gpu_bmatrix_apply_direct_noalloc(int n, const double* d_xyz, const double* d_alpha6,
                                          const int* d_excl_ptr, const int* d_excl_idx,
                                          int damp, double damping_factor, const double* d_in,
                                          double* d_out, void* stream);

/* ---------------------------------------------------------------------------
 * Learned initial guess and preconditioner correction (no counterpart in the
 * reference).  An MLP (64 -> 128 -> 128 -> 4, GELU, FP32) maps 64
 * rotation-invariant descriptors of each site's environment within 6 A to
 * coefficients y: the first-call guess mu0 = y0 v1 + y1 v2 + y2 v3 with the
 * equivariant vectors v1 = alpha F, v2 = alpha T_near v1, v3 = alpha T_near v2,
 * and a preconditioner z = alpha r + y3 alpha T_near alpha r used by a
 * flexible PCG.  Plain PCG is the fallback: a learned solve that does not
 * converge is repeated from alpha F with the Jacobi preconditioner, and the
 * stopping rule is unchanged.  Training runs on the GPU (hand-written GEMM,
 * GELU, loss and Adam kernels) from rows produced by cppe_gpu_learned_data.
 * ------------------------------------------------------------------------- */
typedef struct cppe_gpu_mlp cppe_gpu_mlp;
int cppe_gpu_mlp_nparams(int* n);
int cppe_gpu_mlp_create(int device, unsigned seed, cppe_gpu_mlp** out);
int cppe_gpu_mlp_destroy(cppe_gpu_mlp* m);
int cppe_gpu_mlp_get_params(cppe_gpu_mlp* m, float* out);
int cppe_gpu_mlp_set_params(cppe_gpu_mlp* m, const float* in);
/* Descriptor normalisation (64 means and inverse standard deviations); any
 * pointer may be NULL; the *_out pointers read the current values back. */
int cppe_gpu_mlp_normalization(cppe_gpu_mlp* m, const float* mean, const float* inv_std,
                               float* mean_out, float* inv_std_out);
/* y (rows x 4) for raw descriptors (rows x 64), host buffers. */
int cppe_gpu_mlp_forward(cppe_gpu_mlp* m, int rows, const float* feats, float* y);
/* The same network on the tensor cores (tcgen05, TF32 operands with FP32
 * accumulation; the kernel the learned solves use): rows x 4 outputs.
 * CPPE_GPU_TIMEOUT if a wait on the MMA completion barrier ran out. */
int cppe_gpu_mlp_infer(cppe_gpu_mlp* m, int rows, const float* feats, float* y);
/* Loss and gradient (cppe_gpu_mlp_nparams floats) of one batch; targets are
 * rows of 24 floats: v1 v2 v3 mu* a w e (3 each), the two loss weights, pad. */
int cppe_gpu_mlp_loss_grad(cppe_gpu_mlp* m, int rows, const float* feats,
                           const float* targets, float lam, double* loss, float* grads);
/* `steps` Adam steps on random batches of `batch` rows; loss_hist (steps) may be NULL. */
int cppe_gpu_mlp_train(cppe_gpu_mlp* m, int rows, const float* feats, const float* targets,
                       int steps, int batch, float lr, float lam, unsigned seed,
                       double* loss_hist);
/* Training rows of one solve: descriptors (n x 64) and targets (n x 24) for
 * the right-hand side rhs and its converged solution mu_star (caller order
 * in, device-order rows out). */
int cppe_gpu_learned_data(cppe_gpu_system* sys, const double* rhs, const double* mu_star,
                          float* feats, float* rows);
/* Attach a model to a system (NULL detaches); first-call solves
 * (make_guess != 0) then use the learned guess and preconditioner. */
int cppe_gpu_set_model(cppe_gpu_system* sys, cppe_gpu_mlp* m);

/* ---------------------------------------------------------------------------
 * Instrumentation (no counterpart in the reference).
 * ------------------------------------------------------------------------- */
/* The cudaStream_t the system's work is ordered on (for caller-side events). */
int cppe_gpu_stream(cppe_gpu_system* sys, void** stream);
/* Number of kernels this library has launched in this process. */
int cppe_gpu_launch_count(long long* count);
/* Average device time in ms of each phase over `reps` operator applies,
 * bracketed by CUDA events on the system's stream, phases run one after the
 * other; precision: CPPE_GPU_FP64, CPPE_GPU_MIXED (the FP32 operator of the
 * inner solve) or 2 (the FP64 operator with the double-float near field of the
 * mixed solver's residuals):
 * out_ms[0] near-field pair pass, [1] P2M+M2M, [2] M2L, [3] L2L,
 * [4] finishing pass (L2P, exclusions, alpha^-1, dot), [5] whole apply.
 * near_pairs: ordered site pairs of the near-field pass that the reference
 * evaluates (self and excluded pairs not counted); m2l_pairs: M2L cell pairs. */
int cppe_gpu_kernel_timings(cppe_gpu_system* sys, int precision, int reps, double* out_ms,
                            long long* near_pairs, long long* m2l_pairs);
/* Schedule autotuning (no reference counterpart): times the FP32 operator for
 * three near-field work-item sizes and three M2L chunk sizes on this system
 * and keeps the fastest, then the faster of the two priorities of the
 * far-field stream (highest, default); best_ms (may be null) receives its
 * apply time.  The operator is unchanged; only the work partition and the
 * stream scheduling differ. */
int cppe_gpu_autotune(cppe_gpu_system* sys, int reps, double* best_ms);
/* The schedule in use (no counterpart in the reference): whether the FP32
 * near field evaluates each leaf pair once for both directions (1: two
 * sources a lane, 2: four sources a lane) or per target leaf (0), its number
 * of work items, and the sources per M2L warp. */
int cppe_gpu_schedule_info(cppe_gpu_system* sys, int* symmetric_near, long* near_items,
                           int* m2l_chunk);
/* Sets the schedule directly (no counterpart in the reference), e.g. one that
 * cppe_gpu_autotune chose earlier for the same system: near_form 0 (per
 * target leaf), 1 or 2 (each leaf pair once, two or four sources a lane; the
 * symmetric form applies to single systems with dipole sources), -1 keeps
 * it; item_pairs (>= 1024) and m2l_chunk (32, 64 or 128) keep theirs when
 * <= 0.  The operator is unchanged. */
int cppe_gpu_set_schedule(cppe_gpu_system* sys, int near_form, long item_pairs,
                          int m2l_chunk);
/* Measured FMA throughput of the device in TFLOP/s (2 FLOP per FMA), FP32 or FP64. */
int cppe_gpu_fma_peak(int device, int fp64, double* tflops);

/* ---------------------------------------------------------------------------
 * Batched solves: nsys independent systems (snapshots) of uneven size, each
 * with nrhs right-hand sides, solved together.  Site arrays are concatenated
 * over systems; site_offset (nsys+1) gives each system's range.  Exclusion
 * indices are local to their system.  rhs and mu are [system][rhs][3*n_s]
 * concatenated (offset 3*nrhs*site_offset[s]).  Systems with fewer than
 * direct_below sites use direct summation, the rest FMM with opts.
 * ------------------------------------------------------------------------- */
typedef struct cppe_gpu_batch cppe_gpu_batch;
int cppe_gpu_batch_create(int nsys, const int* site_offset, const double* xyz,
                          const double* alpha6, const int* excl_ptr, const int* excl_idx,
                          int nrhs, int direct_below, const cppe_gpu_options* opts,
                          cppe_gpu_batch** out);
int cppe_gpu_batch_destroy(cppe_gpu_batch* b);
int cppe_gpu_batch_solve(cppe_gpu_batch* b, const double* rhs, double* mu, int* iters);
int cppe_gpu_batch_solve_device(cppe_gpu_batch* b, const double* d_rhs, double* d_mu,
                                int* iters);
/* Operator applications of the last batched solve (each covers every
 * segment) and the largest final residual norm over the segments. */
int cppe_gpu_batch_stats(cppe_gpu_batch* b, int* fp64_applies, int* fp32_applies,
                         double* max_rnorm);
/* Host synchronisations with the batch's stream in the last batched solve
 * (cppe_gpu_batch_solve_device): 2 where a mixed solve runs its usual course
 * -- start residual, two inner solves around a double-float residual, the
 * residual from the recursion -- as one graph launch (the second is the
 * copy-out); more where the host loop takes further outer iterations, runs
 * with graphs disabled (CPPE_GPU_GRAPHS=0), or solves in FP64. */
int cppe_gpu_batch_host_waits(cppe_gpu_batch* b, int* waits);
/* Schedule autotuning of a batch, as cppe_gpu_autotune: the FP32 operator
 * over all segments under three near-field work-item sizes, three M2L chunk
 * sizes and both far-field stream priorities; keeps the fastest. */
int cppe_gpu_batch_autotune(cppe_gpu_batch* b, int reps, double* best_ms);
/* The cudaStream_t the batch's work is ordered on. */
int cppe_gpu_batch_stream(cppe_gpu_batch* b, void** stream);

#ifdef __cplusplus
}
#endif

#endif /* CPPE_GPU_H */
