// MLP inference on the 5th-generation tensor cores (tcgen05): the learned
// guess/preconditioner model (64 -> 128 -> 128 -> 4, GELU) evaluated for every
// site of a system, 128 sites (rows) per tile.
//
// Per tile, three chained GEMMs D = A W^T with M = 128 rows:
//   layer 1: A = normalised descriptors (128 x 64),  W1 (128 x 64),  N = 128
//   layer 2: A = GELU(layer 1 + b1)     (128 x 128), W2 (128 x 128), N = 128
//   layer 3: A = GELU(layer 2 + b2)     (128 x 128), W3 (4 x 128, padded to 16 rows)
// Operands are TF32 (FP32 storage rounded to nearest TF32 when staged) in
// shared memory in the canonical K-major layout without swizzle: 8-row x
// 16-byte core matrices, element (r, k) at byte
//   (r / 8) * SBO + (k / 4) * 128 + (r % 8) * 16 + (k % 4) * 4,  SBO = 32 K,
// so the leading-dimension offset (next core matrix along K) is 128 bytes and
// the stride-dimension offset (next 8 rows) is SBO.  One thread issues the
// tcgen05.mma instructions (K = 8 each) into an FP32 accumulator of 128 lanes
// x N columns in tensor memory and commits them to an mbarrier; sixteen warps
// read the accumulator back with tcgen05.ld (warp w: lanes 32 (w mod 4) on,
// columns 32 (w / 4) on -- a warp may only reach its own quarter of the
// lanes), add the bias, apply GELU and store the next layer's operand.  The
// weights stay in shared memory for the CTA's lifetime (persistent CTAs, one
// per SM, looping over row tiles).
//
// Every mbarrier wait is bounded by the global timer (1 s): on expiry the
// kernel records an error code, stops issuing work, waits (bounded again) for
// the MMAs it committed, frees its tensor memory and returns.
#include <cstdint>

#include "mlp.h"

namespace cg {

namespace {

constexpr int TC_ROWS    = 128;  // rows (sites) per tile = MMA M
constexpr int TC_THREADS = 512;  // 16 warps: 4 lane quarters x 4 column groups
constexpr int TC_W3N  = 16;   // layer-3 N (4 outputs padded to the smallest N for M = 128)
constexpr int TC_COLS = 128;  // tensor-memory columns of the accumulator

// shared-memory map (bytes, every operand 1024-byte aligned)
constexpr int OFF_W1   = 0;                                   // 128 x 64  tf32
constexpr int OFF_W2   = OFF_W1 + Mlp::H * Mlp::IN * 4;       // 128 x 128
constexpr int OFF_W3   = OFF_W2 + Mlp::H * Mlp::H * 4;        // 16 x 128
constexpr int OFF_X    = OFF_W3 + TC_W3N * Mlp::H * 4;        // 128 x 64
constexpr int OFF_H    = OFF_X + TC_ROWS * Mlp::IN * 4;       // 128 x 128
constexpr int OFF_VEC  = OFF_H + TC_ROWS * Mlp::H * 4;        // b1, b2, b3, mean, inv_std
constexpr int VEC_LEN  = Mlp::H + Mlp::H + 4 + 2 * Mlp::IN;
constexpr int OFF_BAR  = OFF_VEC + VEC_LEN * 4;               // mbarrier (8 bytes)
constexpr int OFF_TMEM = OFF_BAR + 8;                         // tensor-memory address slot
constexpr int SMEM_BYTES = OFF_TMEM + 8 + 1024;               // + alignment slack

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// byte offset of element (r, k) of a K-major operand with K columns
__device__ __forceinline__ int kmajor_off(int r, int k, int K) {
  return (r >> 3) * (K * 32) + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4;
}

// shared-memory matrix descriptor: start address, leading-dimension offset
// 128 B, stride-dimension offset `sbo`, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)(128 >> 4) << 16) |
         ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
}

// instruction descriptor: kind::tf32, D FP32, A and B TF32, both K-major
__device__ __forceinline__ uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// waits for the given phase of the barrier for at most one second
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  const uint64_t t0 = global_ns();
  while (!mbar_try(bar, parity))
    if (global_ns() - t0 > 1000000000ull) return false;
  return true;
}

__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 32 consecutive accumulator columns of this thread's lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
        "%28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ float gelu_tc(float z) {
  return 0.5f * z * (1.f + erff(z * 0.70710678f));
}

}  // namespace

// Error codes written to *err: 1 = an mbarrier wait ran out of time.
__global__ void __launch_bounds__(TC_THREADS, 1)
      k_mlp_infer_tc(int rows, const float* __restrict__ raw, const float* __restrict__ params,
                     const float* __restrict__ mean, const float* __restrict__ inv_std,
                     float* __restrict__ Y, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  float* vec       = reinterpret_cast<float*>(sm + OFF_VEC);
  float* b1        = vec;
  float* b2        = b1 + Mlp::H;
  float* b3        = b2 + Mlp::H;
  float* nmean     = b3 + 4;
  float* ninv      = nmean + Mlp::IN;
  uint64_t* bar    = reinterpret_cast<uint64_t*>(sm + OFF_BAR);
  uint32_t* tslot  = reinterpret_cast<uint32_t*>(sm + OFF_TMEM);
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5;

  // tensor memory (warp 0) and the completion barrier (thread 0)
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                       smem_addr(tslot)),
                 "r"(TC_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_fail = 0;
  }
  // weights (TF32, K-major), biases and the input normalisation
  const float* gW1 = params;
  const float* gb1 = gW1 + Mlp::NW1;
  const float* gW2 = gb1 + Mlp::NB1;
  const float* gb2 = gW2 + Mlp::NW2;
  const float* gW3 = gb2 + Mlp::NB2;
  const float* gb3 = gW3 + Mlp::NW3;
  for (int q = tid; q < Mlp::H * Mlp::IN / 4; q += blockDim.x) {
    const int o = q / (Mlp::IN / 4), k = 4 * (q % (Mlp::IN / 4));
    const float4 w = *reinterpret_cast<const float4*>(gW1 + o * Mlp::IN + k);
    *reinterpret_cast<float4*>(sm + OFF_W1 + kmajor_off(o, k, Mlp::IN)) =
          make_float4(to_tf32(w.x), to_tf32(w.y), to_tf32(w.z), to_tf32(w.w));
  }
  for (int q = tid; q < Mlp::H * Mlp::H / 4; q += blockDim.x) {
    const int o = q / (Mlp::H / 4), k = 4 * (q % (Mlp::H / 4));
    const float4 w = *reinterpret_cast<const float4*>(gW2 + o * Mlp::H + k);
    *reinterpret_cast<float4*>(sm + OFF_W2 + kmajor_off(o, k, Mlp::H)) =
          make_float4(to_tf32(w.x), to_tf32(w.y), to_tf32(w.z), to_tf32(w.w));
  }
  for (int q = tid; q < TC_W3N * Mlp::H / 4; q += blockDim.x) {
    const int o = q / (Mlp::H / 4), k = 4 * (q % (Mlp::H / 4));
    float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
    if (o < Mlp::OUT) w = *reinterpret_cast<const float4*>(gW3 + o * Mlp::H + k);
    *reinterpret_cast<float4*>(sm + OFF_W3 + kmajor_off(o, k, Mlp::H)) =
          make_float4(to_tf32(w.x), to_tf32(w.y), to_tf32(w.z), to_tf32(w.w));
  }
  for (int k = tid; k < Mlp::H; k += blockDim.x) b1[k] = gb1[k], b2[k] = gb2[k];
  if (tid < Mlp::OUT) b3[tid] = gb3[tid];
  for (int k = tid; k < Mlp::IN; k += blockDim.x) nmean[k] = mean[k], ninv[k] = inv_std[k];
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tslot;
  const int quarter = warp & 3, cgroup = warp >> 2;
  const uint32_t lane_base = tmem + ((uint32_t)(32 * quarter) << 16);
  const int row_local = 32 * quarter + (tid & 31);  // TMEM lane = row of the tile
  uint32_t parity = 0;
  const uint32_t aX = smem_addr(sm + OFF_X), aH = smem_addr(sm + OFF_H);
  const uint32_t aW1 = smem_addr(sm + OFF_W1), aW2 = smem_addr(sm + OFF_W2),
                 aW3 = smem_addr(sm + OFF_W3);
  int committed = 0;  // MMA groups committed, for the bounded drain at the end
  int completed = 0;

  // one layer: K/8 MMAs into the accumulator, committed to the barrier
  auto run_layer = [&](uint32_t aA, uint32_t aB, int K, int N) -> bool {
    if (tid == 0) {
      fence_after();
      const uint32_t id = idesc_tf32(TC_ROWS, N);
      for (int s = 0; s < K / 8; ++s)
        mma_tf32(tmem, smem_desc(aA + 256 * s, 32 * K), smem_desc(aB + 256 * s, 32 * K), id,
                 s > 0 ? 1u : 0u);
      mma_commit(bar);
    }
    ++committed;
    const bool ok = mbar_wait_bounded(bar, parity);
    if (ok) ++completed, parity ^= 1u;
    if (!ok) atomicExch(&s_fail, 1);
    fence_after();
    __syncthreads();
    return s_fail == 0;
  };
  // hidden-layer epilogue: GELU(acc + b) into the next layer's operand
  auto hidden_epilogue = [&](const float* bias) {
    {
      const int c = cgroup;  // this warp's 32 columns
      float v[32];
      tmem_ld32(lane_base + 32 * c, v);
#pragma unroll
      for (int j = 0; j < 32; j += 4) {
        const int k = 32 * c + j;
        const float4 h = make_float4(to_tf32(gelu_tc(v[j] + bias[k])),
                                     to_tf32(gelu_tc(v[j + 1] + bias[k + 1])),
                                     to_tf32(gelu_tc(v[j + 2] + bias[k + 2])),
                                     to_tf32(gelu_tc(v[j + 3] + bias[k + 3])));
        *reinterpret_cast<float4*>(sm + OFF_H + kmajor_off(row_local, k, Mlp::H)) = h;
      }
    }
    fence_before();
    fence_async_smem();
    __syncthreads();
  };

  const int ntiles = (rows + TC_ROWS - 1) / TC_ROWS;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long row0 = (long)tile * TC_ROWS;
    // normalised descriptors of the tile (coalesced float4 loads)
    for (int q = tid; q < TC_ROWS * Mlp::IN / 4; q += blockDim.x) {
      const int r = q / (Mlp::IN / 4), k = 4 * (q % (Mlp::IN / 4));
      float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
      if (row0 + r < rows) {
        x = *reinterpret_cast<const float4*>(raw + (row0 + r) * Mlp::IN + k);
        x.x = to_tf32((x.x - nmean[k]) * ninv[k]);
        x.y = to_tf32((x.y - nmean[k + 1]) * ninv[k + 1]);
        x.z = to_tf32((x.z - nmean[k + 2]) * ninv[k + 2]);
        x.w = to_tf32((x.w - nmean[k + 3]) * ninv[k + 3]);
      }
      *reinterpret_cast<float4*>(sm + OFF_X + kmajor_off(r, k, Mlp::IN)) = x;
    }
    fence_async_smem();
    __syncthreads();
    if (!run_layer(aX, aW1, Mlp::IN, Mlp::H)) break;
    hidden_epilogue(b1);
    if (!run_layer(aH, aW2, Mlp::H, Mlp::H)) break;
    hidden_epilogue(b2);
    if (!run_layer(aH, aW3, Mlp::H, TC_W3N)) break;
    if (cgroup == 0) {
      float v[32];
      tmem_ld32(lane_base, v);  // columns 0..31; 0..3 are the outputs
      const long row = row0 + row_local;
      if (row < rows) {
        float4 y = make_float4(v[0] + b3[0], v[1] + b3[1], v[2] + b3[2], v[3] + b3[3]);
        *reinterpret_cast<float4*>(Y + row * Mlp::OUT) = y;
      }
    }
    fence_before();
    __syncthreads();
  }
  if (s_fail) {
    if (tid == 0) atomicExch(err, 1);
    // drain the MMAs still in flight (bounded), so that tensor memory is idle
    while (completed < committed && mbar_wait_bounded(bar, parity)) ++completed, parity ^= 1u;
  }
  fence_before();
  __syncthreads();
  if (warp == 0) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TC_COLS)
                 : "memory");
  }
}

void mlp_infer_tc(int device, int rows, const float* raw, const float* params,
                  const float* mean, const float* inv_std, float* Y, int* err, cudaStream_t s) {
  if (rows <= 0) return;
  static int attr_device = -1;
  if (attr_device != device) {
    CG_CUDA(cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 SMEM_BYTES));
    attr_device = device;
  }
  int sms = 0;
  CG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const int ntiles = (rows + TC_ROWS - 1) / TC_ROWS;
  const int grid   = std::max(1, std::min(ntiles, sms));
  k_mlp_infer_tc<<<grid, TC_THREADS, SMEM_BYTES, s>>>(rows, raw, params, mean, inv_std, Y, err);
  CG_LAUNCH();
}

}  // namespace cg
