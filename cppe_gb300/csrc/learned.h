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

#include "engine.h"
#include "mlp.h"

namespace cg {

constexpr double LEARN_RC = 6.0 * 1.8897261246;  // 6 A in bohr

struct NearGrid {
  int n = 0;
  double rc = LEARN_RC;
  double origin[3] = {0, 0, 0};
  int dims[3]      = {1, 1, 1};
  DBuf<int> cell_start, cell_site, excl_ptr, excl_idx;
  // sites in device order; exclusions given in caller indices
  void build(const Geometry& g, const int* caller_excl_ptr, const int* caller_excl_idx,
             cudaStream_t s);
};

struct NearGridView {
  int n;
  double rc, ox, oy, oz;
  int dx, dy, dz;
  const int* cell_start;
  const int* cell_site;
  const int* excl_ptr;
  const int* excl_idx;
};

NearGridView view(const NearGrid& g);

// descriptors (n x 64) and v1 (3n) from the field F (device order)
void learned_features(const NearGridView& ng, const double4_32a* pos, const float* a6f,
                      const double* F, float* feats, float* v1, cudaStream_t s);
// out_i = alpha_i sum_{j near} T_ij in_j  (T damped with a_ij = damping s_i s_j)
template <typename T>
void near_T(const NearGridView& ng, const double4_32a* pos, const T* a6, int damp, double damping,
            const T* in, T* out, cudaStream_t s);
void learned_basis_features(int n, const float* v1, const float* v2, const float* v3,
                            float* feats, cudaStream_t s);
void learned_guess(int n, const float* Y, const float* v1, const float* v2, const float* v3,
                   double* x, float* c, cudaStream_t s);
// z += c w; with r_old: beta = (z.r - z.r_old) / rz_old (Polak-Ribiere), rz = z.r
template <typename T>
void precond_fix(int n, T* z, const T* w, const float* c, const T* r, const T* r_old, T* p,
                 bool start, double* partials, unsigned* ticket, double* scal, const int* flags,
                 cudaStream_t s);

}  // namespace cg
