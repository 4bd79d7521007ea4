// Learned initial guess and preconditioner correction for the induced-dipole
// PCG (no counterpart in the reference; plain PCG stays the fallback).
//
// Per site i, with neighbours j within rc = 6 A:
//   v1 = alpha_i F_i,  v2 = alpha_i sum_j T_ij v1_j,  v3 = alpha_i sum_j T_ij v2_j
// (T the Thole-damped dipole tensor restricted to rc, excluded pairs skipped)
// are rotation-equivariant; 64 rotation-invariant descriptors of the
// environment (radial densities of neighbours and of their polarizability,
// angular moments about the field direction, ratios and angles of v1..v3)
// feed the MLP, whose four outputs y give
//   initial guess      mu0_i = y0 v1_i + y1 v2_i + y2 v3_i
//   preconditioner     z_i   = alpha_i r_i + y3 (alpha T_near alpha r)_i
// The corrected preconditioner varies per site, so the CG uses the flexible
// (Polak-Ribiere) beta.
#pragma once

#include <cuda_fp16.h>

#include "engine.h"
#include "mlp.h"

namespace cg {

constexpr double LEARN_RC = 6.0 * 1.8897261246;  // 6 A in bohr

// Neighbour lists within LEARN_RC of every site (device order, the site
// itself removed), built once per system on the GPU, with the damped dipole
// tensor of each pair stored as its six upper-triangle components:
// T_ij = G1 I + G2 r r^T (r = r_i - r_j; G1, G2 the radial factors of the
// operator), so that (T v)_i = sum_j T_ij v_j is the field at i of dipoles v;
// excluded pairs are listed (for the descriptors) with T_ij = 0.  Entry k of site i (ptr[i] <= k < ptr[i+1]) holds idx[k] = j,
// t6[6k..6k+5] (FP16: the tensors feed only the guess basis and the
// preconditioner) and d[k] = (r_j - r_i, |r_j - r_i|).
struct NearList {
  int n    = 0;
  long nnz = 0;
  DBuf<int> ptr, idx;
  DBuf<__half> t6;
  DBuf<float4> d;
  // the operator's entries packed for one 16-byte load each:
  // {j, half2(t0, t1), half2(t2, t3), half2(t4, t5)}
  DBuf<int4> ent;
  // exclusions in caller indices (CSR, may be null)
  void build(const Geometry& g, const int* caller_excl_ptr, const int* caller_excl_idx,
             int damp, double damping, cudaStream_t s);
};

struct NearListView {
  int n;
  const int* ptr;
  const int* idx;
  const __half* t6;
  const float4* d;
  const int4* ent;
};

NearListView view(const NearList& g);

// descriptors (n x 64) and v1 (3n) from the field F (device order)
void learned_features(const NearListView& nl, const float* a6f, const double* F, float* feats,
                      float* v1, cudaStream_t s);
// out_i = alpha_i sum_{j near} T_ij in_j
template <typename T>
void near_T(const NearListView& nl, const T* a6, const T* in, T* out, cudaStream_t s);
void learned_basis_features(int n, const float* v1, const float* v2, const float* v3,
                            float* feats, cudaStream_t s);
void learned_guess(int n, const float* Y, const float* v1, const float* v2, const float* v3,
                   double* x, float* c, cudaStream_t s);
// Corrected preconditioner in one pass: zc = a + c alpha T_near a for a = alpha r
// (the plain preconditioned residual); at a start p = zc; rz = zc.r and, after
// a start, beta = (zc.r - zc.r_old) / rz_old (Polak-Ribiere).
// a4 (may be null): a as one float4 per site, read by the gathers instead.
template <typename T>
void precond_near(const NearListView& nl, const T* a6, const float* c, const T* a, const T* r,
                  const T* r_old, T* zc, T* p, bool start, double* partials, unsigned* ticket,
                  double* scal, const int* flags, cudaStream_t s,
                  const float4* a4 = nullptr);

}  // namespace cg
