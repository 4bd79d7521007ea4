// M2L with the expansion order fixed at compile time (the orders the
// benchmark configurations use; other orders take the table-driven k_m2l).
//
// Same operator as k_m2l (src/core/fmm/calculate.cc:186-203 with the
// field_m*.cc M2L kernels), organised for registers: each lane of a warp
// takes its own source cell of the target's interaction list, evaluates the
// straight-line translation generated by gen_m2l.py (derivative tensor and
// partial local expansion in registers, the source multipole streamed one
// coefficient at a time), and the lanes' partial expansions are added with
// warp shuffles in a fixed order at the end.
#pragma once

#include "engine.h"

namespace cg {

// generated straight-line translations (function templates + an X-macro list)
#include "m2l_gen.cuh"

#define CPPE_DEF_M2L_KERNEL(M, P, NAME, LS, MS)                                            \
  template <typename T>                                                                    \
  __global__ void __launch_bounds__(128)                                                   \
        k_##NAME(TreeView tv, const T* __restrict__ Mexp, T* __restrict__ L) {             \
    const int lane = threadIdx.x & 31;                                                     \
    const int A    = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;                         \
    if (A >= tv.ncells) return;                                                            \
    T acc[LS];                                                                             \
    _Pragma("unroll") for (int q = 0; q < LS; ++q) acc[q] = T(0);                          \
    const double4_32a cA = tv.center[A];                                                   \
    const int s1         = tv.m2l_ptr[A + 1];                                              \
    for (int idx = tv.m2l_ptr[A] + lane; idx < s1; idx += 32) {                            \
      const int B          = tv.m2l_src[idx];                                              \
      const double4_32a cB = tv.center[B];                                                 \
      NAME<T>((T)(cA.x - cB.x), (T)(cA.y - cB.y), (T)(cA.z - cB.z),                        \
              Mexp + (size_t)B * (MS), acc);                                               \
    }                                                                                      \
    _Pragma("unroll") for (int q = 0; q < LS; ++q) {                                       \
      T v = acc[q];                                                                        \
      _Pragma("unroll") for (int off = 16; off > 0; off >>= 1) v +=                        \
            __shfl_xor_sync(0xffffffffu, v, off);                                          \
      acc[q] = v;                                                                          \
    }                                                                                      \
    T* LA = L + (size_t)A * (LS);                                                          \
    _Pragma("unroll") for (int q = 0; q < LS; ++q) if ((q & 31) == lane) LA[q] = acc[q];   \
  }

CPPE_M2L_GENERATED(CPPE_DEF_M2L_KERNEL)
#undef CPPE_DEF_M2L_KERNEL

// Launches the fixed-order kernel when one is compiled for (m, p); returns
// false otherwise.
template <typename T>
bool launch_m2l_fixed(const TreeView& tv, int m, int p, const T* Mexp, T* L, cudaStream_t s) {
  const int blocks = (int)(((long)tv.ncells * 32 + 127) / 128);
#define CPPE_LAUNCH_M2L(MM, PP, NAME, LS, MS)                 \
  if (m == MM && p == PP) {                                   \
    k_##NAME<T><<<blocks, 128, 0, s>>>(tv, Mexp, L);          \
    return true;                                              \
  }
  CPPE_M2L_GENERATED(CPPE_LAUNCH_M2L)
#undef CPPE_LAUNCH_M2L
  return false;
}

}  // namespace cg
