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

#include "dd.cuh"
#include "engine.h"

namespace cg {

// generated straight-line translations (function templates + an X-macro list)
#include "m2l_gen.cuh"

constexpr int nterms_c(int p) { return p < 0 ? 0 : (p + 1) * (p + 2) * (p + 3) / 6; }

// Derivative tensors of the distinct M2L vectors (Geometry::make_vectors),
// thread per vector, in T or in double-float.
#define CPPE_DEF_DTAB(MM, PP, NAME, NT, LS, MS)                                             \
  template <typename T>                                                                     \
  __global__ void k_dtab_##NAME(int nvec, const double4_32a* __restrict__ vec,              \
                                T* __restrict__ D) {                                        \
    const int v = blockIdx.x * blockDim.x + threadIdx.x;                                    \
    if (v >= nvec) return;                                                                  \
    const double4_32a r = vec[v];                                                           \
    dtensor_##NAME<T>((T)r.x, (T)r.y, (T)r.z, D + (size_t)v * (NT));                        \
  }                                                                                         \
  __global__ void k_dtab_##NAME##_dd(int nvec, const double4_32a* __restrict__ vec,         \
                                     float2* __restrict__ D) {                              \
    const int v = blockIdx.x * blockDim.x + threadIdx.x;                                    \
    if (v >= nvec) return;                                                                  \
    const double4_32a r = vec[v];                                                           \
    ddv t[NT];                                                                              \
    dtensor_##NAME<ddv>(ddv(dd_from(r.x)), ddv(dd_from(r.y)), ddv(dd_from(r.z)), t);       \
    _Pragma("unroll") for (int j = 0; j < (NT); ++j)                                        \
          D[(size_t)v * (NT) + j] = make_float2(t[j].h, t[j].l);                            \
  }
CPPE_M2L_TABLES(CPPE_DEF_DTAB)
#undef CPPE_DEF_DTAB

// Builds the tensor table of g's M2L vectors for order p into w (T, or
// double-float when dd) on first use; returns it, or null when g has no
// vector table or no fixed-order kernel serves (m, p).
template <typename T>
const void* m2l_dtab(const Geometry& g, int m, int p, FieldWork<T>& w, bool dd, cudaStream_t s) {
  const int nv = (int)g.h_vec.size();
  if (nv == 0) return nullptr;
  const void* out = nullptr;
#define CPPE_BUILD_DTAB(MM, PP, NAME, NT, LS, MS)                                            \
  if (!out && m == MM && p == PP) {                                                          \
    const size_t cnt = (size_t)nv * (NT);                                                    \
    if (dd) {                                                                                \
      if (w.dtab_dd.n != cnt) {                                                              \
        w.dtab_dd.alloc(cnt);                                                                \
        k_dtab_##NAME##_dd<<<(nv + 63) / 64, 64, 0, s>>>(nv, g.vec.p, w.dtab_dd.p);          \
        CG_LAUNCH();                                                                         \
      }                                                                                      \
      out = w.dtab_dd.p;                                                                     \
    } else {                                                                                 \
      if (w.dtab.n != cnt) {                                                                 \
        w.dtab.alloc(cnt);                                                                   \
        k_dtab_##NAME<T><<<(nv + 63) / 64, 64, 0, s>>>(nv, g.vec.p, w.dtab.p);               \
        CG_LAUNCH();                                                                         \
      }                                                                                      \
      out = w.dtab.p;                                                                        \
    }                                                                                        \
  }
  CPPE_M2L_TABLES(CPPE_BUILD_DTAB)
#undef CPPE_BUILD_DTAB
  return out;
}

#define CPPE_DEF_M2L_KERNEL(M, P, NAME, LS, MS)                                            \
  template <typename T, bool PRE>                                                          \
  __global__ void __launch_bounds__(128, sizeof(T) == 4 ? ((P) == 5 ? 4 : 3) : 1)          \
        k_##NAME(TreeView tv, const int4* __restrict__ chunks, int nchunks,                \
                 const T* __restrict__ Mexp, T* __restrict__ Lpart,                        \
                 const int* __restrict__ cell_seg, const int* __restrict__ seg_done,       \
                 const T* __restrict__ Dtab, const int* __restrict__ vid) {                \
    const int lane = threadIdx.x & 31;                                                     \
    const int w    = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;                         \
    if (w >= nchunks) return;                                                              \
    const int4 ch = chunks[w];                                                             \
    const int A   = ch.x;                                                                  \
    if (seg_done && seg_done[cell_seg[A]]) return; /* finished segment of a batch */       \
    T acc[LS];                                                                             \
    _Pragma("unroll") for (int q = 0; q < LS; ++q) acc[q] = T(0);                          \
    const double4_32a cA = tv.center[A];                                                   \
    for (int idx = ch.y + lane; idx < ch.z; idx += 32) {                                   \
      const int B = tv.m2l_src[idx];                                                       \
      const T* Mb = static_cast<const T*>(                                                 \
            __builtin_assume_aligned(Mexp + (size_t)B * m_stride(MS), 16));                \
      if constexpr (PRE) {                                                                 \
        const T* Dv = static_cast<const T*>(                                               \
              __builtin_assume_aligned(Dtab + (size_t)vid[idx] * nterms_c(P), 16));        \
        NAME##_pre<T>(Dv, Mb, acc);                                                        \
      } else {                                                                             \
        const double4_32a cB = tv.center[B];                                               \
        NAME<T>((T)(cA.x - cB.x), (T)(cA.y - cB.y), (T)(cA.z - cB.z), Mb, acc);            \
      }                                                                                    \
    }                                                                                      \
    _Pragma("unroll") for (int q = 0; q < LS; ++q) {                                       \
      T v = acc[q];                                                                        \
      _Pragma("unroll") for (int off = 16; off > 0; off >>= 1) v +=                        \
            __shfl_xor_sync(0xffffffffu, v, off);                                          \
      acc[q] = v;                                                                          \
    }                                                                                      \
    T* LA = Lpart + (size_t)w * (LS);                                                      \
    _Pragma("unroll") for (int q = 0; q < LS; ++q) if ((q & 31) == lane) LA[q] = acc[q];   \
  }

CPPE_M2L_GENERATED(CPPE_DEF_M2L_KERNEL)
#undef CPPE_DEF_M2L_KERNEL

// Double-float variant for the mixed solver's FP64-accurate residual: the
// same chunks, the source multipoles as double-float pairs (split once per
// apply), the partial expansions written in FP64.  In double-float the
// straight-line translation is longer than the instruction cache holds, so
// this kernel runs the loop form of the same arithmetic from the generated
// tables: each lane builds the derivative tensor of its source in its own
// slice of shared memory (a row of nterms(p) | 1 pairs: conflict-free), then
// adds D_{n+k} M_k over the multipole coefficients k, order by order, with
// the local coefficients n unrolled into registers.
// first w-table entry of the multipole coefficients of order ko
constexpr int m2l_wbase(int m, int p, int ko) {
  int b = 0;
  for (int o = m; o < ko; ++o) b += (nterms_c(o) - nterms_c(o - 1)) * nterms_c(p - o);
  return b;
}
template <int M, int P, int KO, typename WT>
__device__ __forceinline__ void m2l_contract_dd(const float2* __restrict__ D,
                                                const float2* __restrict__ Mb, WT wtab,
                                                dd* acc) {
  constexpr int R = nterms_c(P - KO), k0 = nterms_c(KO - 1), k1 = nterms_c(KO);
  constexpr int base = m2l_wbase(M, P, KO), moff = nterms_c(M - 1);
#pragma unroll 1
  for (int k = k0; k < k1; ++k) {
    const float2 mv = Mb[k - moff];
    const int wr    = base + (k - k0) * R;
#pragma unroll
    for (int n = 0; n < R; ++n) {
      const float2 d = D[wtab(wr + n)];
      acc[n]         = dd_fma_lazy(dd{d.x, d.y}, dd{mv.x, mv.y}, acc[n]);
    }
  }
  if constexpr (KO < P) m2l_contract_dd<M, P, KO + 1>(D, Mb, wtab, acc);
}

#define CPPE_DEF_M2L_DD_KERNEL(MM, PP, NAME, NT, LS, MS)                                    \
  __global__ void __launch_bounds__(64)                                                     \
        k_m2l_##NAME##_dd(TreeView tv, const int4* __restrict__ chunks, int nchunks,        \
                          const float2* __restrict__ Mdd, double* __restrict__ Lpart,       \
                          const float2* __restrict__ Dtab, const int* __restrict__ vid) {   \
    constexpr int DS = (NT) | 1;                                                            \
    __shared__ float2 s_D[2 * 32 * DS];                                                     \
    const int lane = threadIdx.x & 31;                                                      \
    const int w    = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;                          \
    if (w >= nchunks) return;                                                               \
    float2* D     = s_D + (threadIdx.x >> 5) * 32 * DS + lane * DS;                         \
    const int4 ch = chunks[w];                                                              \
    dd acc[LS];                                                                             \
    _Pragma("unroll") for (int q = 0; q < LS; ++q) acc[q] = dd{0.f, 0.f};                   \
    const double4_32a cA = tv.center[ch.x];                                                 \
    auto wtab = [](int i) { return (int)m2l_w_##NAME[i]; };                                 \
    for (int idx = ch.y + lane; idx < ch.z; idx += 32) {                                    \
      const int B = tv.m2l_src[idx];                                                        \
      const float2* Mb = static_cast<const float2*>(                                        \
            __builtin_assume_aligned(Mdd + (size_t)B * m_stride(MS), 16));                  \
      if (Dtab) {                                                                           \
        /* the tabulated tensor of this entry's vector into the lane's row */               \
        const float4* Dv = reinterpret_cast<const float4*>(Dtab + (size_t)vid[idx] * (NT)); \
        _Pragma("unroll 6") for (int i = 0; i < (NT) / 2; ++i) {                            \
          const float4 t = Dv[i];                                                           \
          D[2 * i]       = make_float2(t.x, t.y);                                           \
          D[2 * i + 1]   = make_float2(t.z, t.w);                                           \
        }                                                                                   \
        m2l_contract_dd<MM, PP, MM>(D, Mb, wtab, acc);                                      \
        continue;                                                                           \
      }                                                                                     \
      const double4_32a cB = tv.center[B];                                                  \
      const dd x = dd_from(cA.x - cB.x), y = dd_from(cA.y - cB.y), z = dd_from(cA.z - cB.z); \
      const dd r2  = dd_add(dd_add(dd_sqr(x), dd_sqr(y)), dd_sqr(z));                       \
      const ddv ir2 = ddv(1) / ddv(r2);                                                     \
      const dd d0  = dd_rsqrt(r2);                                                          \
      D[0]         = make_float2(d0.h, d0.l);                                               \
      _Pragma("unroll 1") for (int j = 1; j < (NT); ++j) {                                  \
        const short* q = m2l_rec_##NAME + 8 * j;                                            \
        const float* c = m2l_coef_##NAME + 8 * j;                                           \
        dd s           = {0.f, 0.f};                                                        \
        const dd rv[3] = {x, y, z};                                                         \
        _Pragma("unroll") for (int i = 0; i < 3; ++i) if (q[i] >= 0) {                      \
          const float2 t = D[q[i]];                                                         \
          s = dd_add(s, dd_mul_f(dd_mul(rv[i], dd{t.x, t.y}), c[i]));                       \
        }                                                                                   \
        _Pragma("unroll") for (int i = 3; i < 6; ++i) if (q[i] >= 0) {                      \
          const float2 t = D[q[i]];                                                         \
          s = dd_add(s, dd_mul_f(dd{t.x, t.y}, c[i]));                                      \
        }                                                                                   \
        const dd v = dd_mul(s, dd_mul(ir2, dd{c[6], c[7]}));                                \
        D[j]       = make_float2(-v.h, -v.l);                                               \
      }                                                                                     \
      m2l_contract_dd<MM, PP, MM>(D, Mb, wtab, acc);                                        \
    }                                                                                       \
    double* LA = Lpart + (size_t)w * (LS);                                                  \
    _Pragma("unroll") for (int q = 0; q < LS; ++q) {                                        \
      dd v = acc[q];                                                                        \
      _Pragma("unroll") for (int off = 16; off > 0; off >>= 1) {                            \
        const dd o{__shfl_xor_sync(0xffffffffu, v.h, off),                                  \
                   __shfl_xor_sync(0xffffffffu, v.l, off)};                                 \
        v = dd_add(v, o);                                                                   \
      }                                                                                     \
      if ((q & 31) == lane) LA[q] = dd_to(v);                                               \
    }                                                                                       \
  }

CPPE_M2L_TABLES(CPPE_DEF_M2L_DD_KERNEL)
#undef CPPE_DEF_M2L_DD_KERNEL

// L of every cell: the sum of its chunk partials in order (0 without chunks).
template <typename T>
__global__ void k_lsum(int ncells, int lsize, const int* __restrict__ cell_chunk_ptr,
                       const T* __restrict__ Lpart, T* __restrict__ L,
                       const int* __restrict__ cell_seg = nullptr,
                       const int* __restrict__ seg_done = nullptr) {
  const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int cell = (int)(gid / lsize), row = (int)(gid % lsize);
  if (cell >= ncells) return;
  if (seg_done && seg_done[cell_seg[cell]]) return;  // a batch's masked segment
  T acc = 0;
  for (int t = cell_chunk_ptr[cell]; t < cell_chunk_ptr[cell + 1]; ++t)
    acc += Lpart[(size_t)t * lsize + row];
  L[(size_t)cell * lsize + row] = acc;
}

// Launches the fixed-order kernel when one is compiled for (m, p): a warp per
// chunk of at most M2L_CHUNK sources of one target cell (so that the GPU holds
// several warps per cell), then the per-cell sums.  Returns false otherwise.
template <typename T>
bool launch_m2l_fixed(const TreeView& tv, int m, int p, const int4* chunks, int nchunks,
                      const int* cell_chunk_ptr, const T* Mexp, T* Lpart, T* L, int lsize,
                      cudaStream_t s, const int* cell_seg = nullptr,
                      const int* seg_done = nullptr, const T* dtab = nullptr,
                      const int* vid = nullptr) {
  const int blocks = (int)(((long)std::max(1, nchunks) * 32 + 127) / 128);
  bool ok = false;
#define CPPE_LAUNCH_M2L(MM, PP, NAME, LS, MS)                              \
  if (!ok && m == MM && p == PP) {                                         \
    if (nchunks > 0) {                                                     \
      bool pre = false;                                                    \
      if constexpr (sizeof(T) == 8) {                                      \
        if (dtab) {                                                        \
          k_##NAME<T, true><<<blocks, 128, 0, s>>>(tv, chunks, nchunks,      \
                Mexp, Lpart, cell_seg, seg_done, dtab, vid);                 \
          pre = true;                                                      \
        }                                                                  \
      }                                                                    \
      if (!pre)                                                            \
        k_##NAME<T, false><<<blocks, 128, 0, s>>>(tv, chunks, nchunks, Mexp, \
              Lpart, cell_seg, seg_done, nullptr, nullptr);                  \
      CG_LAUNCH();                                                         \
    }                                                                      \
    ok = true;                                                             \
  }
  CPPE_M2L_GENERATED(CPPE_LAUNCH_M2L)
#undef CPPE_LAUNCH_M2L
  if (!ok) return false;
  const long work = (long)tv.ncells * lsize;
  if (work > 0) {
    k_lsum<T><<<(unsigned)((work + 255) / 256), 256, 0, s>>>(tv.ncells, lsize, cell_chunk_ptr,
                                                             Lpart, L, cell_seg, seg_done);
    CG_LAUNCH();
  }
  return true;
}

// The double-float M2L for (m, p) when compiled: splits M into pairs, runs
// the chunks, sums per cell in FP64.  Returns false otherwise.
__global__ void k_split_dd_vec(long n, const double* __restrict__ in, float2* __restrict__ out);
inline bool launch_m2l_dd(const TreeView& tv, int m, int p, const int4* chunks, int nchunks,
                          const int* cell_chunk_ptr, const double* Mexp, int msize,
                          float2* Mdd, double* Lpart, double* L, int lsize, cudaStream_t s,
                          const float2* dtab = nullptr, const int* vid = nullptr) {
  bool ok = false;
  const long nm = (long)tv.ncells * msize;
#define CPPE_LAUNCH_M2L_DD(MM, PP, NAME, NT, LS, MS)                                       \
  if (!ok && m == MM && p == PP) {                                                         \
    if (nchunks > 0) {                                                                     \
      k_split_dd_vec<<<(unsigned)((nm + 255) / 256), 256, 0, s>>>(nm, Mexp, Mdd);          \
      CG_LAUNCH();                                                                         \
      k_m2l_##NAME##_dd<<<(unsigned)(((long)nchunks * 32 + 63) / 64), 64, 0, s>>>(         \
            tv, chunks, nchunks, Mdd, Lpart, dtab, vid);                                   \
      CG_LAUNCH();                                                                         \
    }                                                                                      \
    ok = true;                                                                             \
  }
  CPPE_M2L_TABLES(CPPE_LAUNCH_M2L_DD)
#undef CPPE_LAUNCH_M2L_DD
  if (!ok) return false;
  const long work = (long)tv.ncells * lsize;
  if (work > 0) {
    k_lsum<double><<<(unsigned)((work + 255) / 256), 256, 0, s>>>(tv.ncells, lsize,
                                                                  cell_chunk_ptr, Lpart, L);
    CG_LAUNCH();
  }
  return true;
}

}  // namespace cg
