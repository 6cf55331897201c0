// Fused surrogate inference on the 5th-generation tensor cores (sm_103a).
//
// One persistent CTA per SM runs tiles of 128 rows through all five layers
// of the 12 -> 4 x 256 -> 10 network without leaving the SM:
//   * activations (BF16) stay in shared memory between layers, in the
//     no-swizzle K-major core-matrix layout that tcgen05.mma reads;
//   * the FP32 accumulator of every layer lives in tensor memory (TMEM,
//     256 columns x 128 lanes), written by tcgen05.mma (kind::f16, BF16 x
//     BF16 -> FP32, M = 128, K = 16 per instruction) issued by one thread and
//     read back by the epilogue warps with tcgen05.ld;
//   * weights are pre-laid-out in global memory in that same core-matrix
//     layout, so each layer's 128 KB arrives in shared memory by bulk copies
//     (cp.async.bulk, completion counted on an mbarrier), the next layer's
//     copy overlapping the current layer's epilogue;
//   * the epilogue (bias + GELU in its tanh form, then BF16) is split over 16 warps:
//     warp w reads TMEM lanes 32 (w % 4) .. + 31 (the rows it owns) and the
//     64 columns of quarter w / 4.
// Every wait on an mbarrier is bounded; on a timeout the kernel records it
// in *err, waits (bounded) for its own operations, frees its TMEM and
// returns.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>

namespace mlptc {

constexpr int TM = 128;             // rows per tile (MMA M)
constexpr int KH = 256;             // hidden width
constexpr int KIN = 16;             // padded input width
constexpr int NOUT = 16;            // padded output width
constexpr int THREADS = 512;
constexpr uint32_t TMEM_COLS = 256;
// shared memory map (bytes)
constexpr uint32_t SA = 0;                        // activations, 128 x 256 BF16 = 64 KB
constexpr uint32_t SB = SA + TM * KH * 2;         // hidden weights, 256 x 256 BF16 = 128 KB
constexpr uint32_t SW0 = SB + KH * KH * 2;        // layer 0 weights, 256 x 16 = 8 KB
constexpr uint32_t SW4 = SW0 + KH * KIN * 2;      // layer 4 weights, 16 x 256 = 8 KB
constexpr uint32_t SBIAS = SW4 + NOUT * KH * 2;   // biases of the five layers, 4 x 256 + 16 FP32
constexpr uint32_t SBAR = SBIAS + (4 * KH + NOUT) * 4;   // two mbarriers (8 B each) + TMEM address
constexpr uint32_t SMEM_BYTES = SBAR + 64;
constexpr int kWaitLimit = 1 << 24;              // non-blocking polls (about 1 s) before a wait gives up

// Instruction descriptor of tcgen05.mma kind::f16: D FP32 (bits 4-5 = 1),
// A and B BF16 (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Shared-memory matrix descriptor, no swizzle: start address >> 4 (bits
// 0-13), leading (K-direction) core-matrix offset >> 4 (bits 16-29), stride
// (M/N-direction) core-matrix offset >> 4 (bits 32-45), the fixed 0b001 in
// bits 46-48, base offset 0, swizzle mode 0.
__host__ __device__ constexpr uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// Byte offset of element (r, k) of an R x K K-major operand stored as
// 8 x 8 core matrices (128 B each, rows of 16 B), K-adjacent core matrices
// 128 B apart (LBO), row-group-adjacent ones K * 16 B apart (SBO).
__host__ __device__ constexpr uint32_t core_off(int r, int k, int K) {
  return (uint32_t)(((r >> 3) * (K >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// true once the phase with the given parity has completed; false after
// kWaitLimit polls
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int i = 0; i < kWaitLimit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// bulk copy global -> shared (16-byte aligned, size a multiple of 16),
// completion counted in bytes on the mbarrier
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, one instruction (M = 128, K = 16)
__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}

// arrive on the mbarrier once all previously issued MMAs of this thread completed
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* v) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
}

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* v) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }


struct TcArgs {
  const __nv_bfloat16* x;          // M x 16 input features (BF16, normalised)
  float* out;                      // M x 16 network output (FP32)
  int M;
  const __nv_bfloat16* blob[5];    // B_l = W_l^T (N x K) in core-matrix layout
  const float* bias[5];
  int* err;                        // set to 1 when a wait gave up
};

// Weights W_l (K x N, row-major BF16) -> the K-major core-matrix layout of
// B_l = W_l^T that a bulk copy moves into shared memory unchanged.
__global__ void k_tc_blob(const __nv_bfloat16* __restrict__ W, int K, int N, __nv_bfloat16* __restrict__ blob) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= K * N) return;
  const int k = idx / N, n = idx % N;
  blob[core_off(n, k, K) >> 1] = W[idx];
}

// bias + GELU of one layer's 128 x 256 accumulator, written back as the
// next layer's BF16 K-major operand; warp w owns rows 32 (w % 4) + lane and
// columns 64 (w / 4) .. + 63; `bias` is the layer's 256 biases in shared
// memory (the same address in every lane: broadcast loads)
__device__ __forceinline__ void epilogue_hidden(uint8_t* sm, uint32_t tmem, int warp, int lane, const float* bias) {
  const int r = (warp & 3) * 32 + lane;
  const uint32_t lane_addr = tmem + ((uint32_t)((warp & 3) * 32) << 16);
#pragma unroll 1
  for (int c = 0; c < 2; ++c) {
    const int col = (warp >> 2) * 64 + c * 32;
    uint32_t v[32];
    tmem_ld32(lane_addr + (uint32_t)col, v);
    tmem_wait_ld();
    uint32_t pk[16];
    const float4* b4 = reinterpret_cast<const float4*>(bias + col);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const float4 b = b4[j];
      const float f0 = gelu(__uint_as_float(v[4 * j]) + b.x);
      const float f1 = gelu(__uint_as_float(v[4 * j + 1]) + b.y);
      const float f2 = gelu(__uint_as_float(v[4 * j + 2]) + b.z);
      const float f3 = gelu(__uint_as_float(v[4 * j + 3]) + b.w);
      __nv_bfloat162 h0 = __floats2bfloat162_rn(f0, f1), h1 = __floats2bfloat162_rn(f2, f3);
      pk[2 * j] = *reinterpret_cast<uint32_t*>(&h0);
      pk[2 * j + 1] = *reinterpret_cast<uint32_t*>(&h1);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
      *reinterpret_cast<uint4*>(sm + SA + core_off(r, col + q * 8, KH)) =
          make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
  }
}

__global__ void __launch_bounds__(THREADS, 1) k_mlp_tc(TcArgs a) {
  extern __shared__ __align__(1024) uint8_t sm[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t base = saddr(sm);
  const uint32_t bar_mma = base + SBAR, bar_ld = base + SBAR + 8;
  if (tid == 0) {
    mbar_init(bar_mma, 1);
    mbar_init(bar_ld, 1);
    fence_async_smem();
  }
  if (warp == 0) tmem_alloc(base + SBAR + 16, TMEM_COLS);
  {   // biases of all layers, once per CTA
    float* bs = reinterpret_cast<float*>(sm + SBIAS);
    for (int q = tid; q < 4 * KH; q += THREADS) bs[q] = a.bias[q / KH][q % KH];
    if (tid < NOUT) bs[4 * KH + tid] = a.bias[4][tid];
  }
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + SBAR + 16);
  uint32_t ph_mma = 0, ph_ld = 0;
  int failed = 0;   // 1: an MMA wait gave up, 2: a copy wait gave up
  // layers 0 and 4 stay resident for all tiles
  if (tid == 0) {
    mbar_expect_tx(bar_ld, (uint32_t)(KH * KIN * 2 + NOUT * KH * 2));
    bulk_g2s(base + SW0, a.blob[0], KH * KIN * 2, bar_ld);
    bulk_g2s(base + SW4, a.blob[4], NOUT * KH * 2, bar_ld);
  }
  if (!__syncthreads_and(mbar_wait(bar_ld, ph_ld))) failed = 2;
  ph_ld ^= 1;
  const int ntiles = (a.M + TM - 1) / TM;
  const uint32_t id_h = idesc_bf16(TM, KH), id_o = idesc_bf16(TM, NOUT);
  for (int tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
    const int row0 = tile * TM;
    if (tid == 0) {   // first hidden layer's weights, overlapping the input staging and layer 0
      mbar_expect_tx(bar_ld, (uint32_t)(KH * KH * 2));
      for (int q = 0; q < 4; ++q)
        bulk_g2s(base + SB + q * 32768, reinterpret_cast<const uint8_t*>(a.blob[1]) + q * 32768, 32768, bar_ld);
    }
    if (tid < TM) {
      const int gr = row0 + tid;
      uint4 v0 = make_uint4(0, 0, 0, 0), v1 = v0;
      if (gr < a.M) {
        const uint4* src = reinterpret_cast<const uint4*>(a.x + (size_t)gr * KIN);
        v0 = src[0];
        v1 = src[1];
      }
      *reinterpret_cast<uint4*>(sm + SA + core_off(tid, 0, KIN)) = v0;
      *reinterpret_cast<uint4*>(sm + SA + core_off(tid, 8, KIN)) = v1;
    }
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    if (tid == 0) {   // layer 0: 128 x 256 = (128 x 16) (16 x 256)
      tc_after_sync();
      mma_bf16(tmem, sdesc(base + SA, 128, KIN * 16), sdesc(base + SW0, 128, KIN * 16), id_h, 0);
      mma_commit(bar_mma);
    }
    if (!__syncthreads_and(mbar_wait(bar_mma, ph_mma))) { failed = 1; break; }
    ph_mma ^= 1;
    tc_after_sync();
    epilogue_hidden(sm, tmem, warp, lane, reinterpret_cast<const float*>(sm + SBIAS));
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    for (int l = 1; l <= 3 && !failed; ++l) {
      if (!__syncthreads_and(mbar_wait(bar_ld, ph_ld))) { failed = 2; break; }
      ph_ld ^= 1;
      if (tid == 0) {   // hidden layer: 16 MMAs along K = 256
        tc_after_sync();
        for (int k = 0; k < KH / 16; ++k)
          mma_bf16(tmem, sdesc(base + SA + k * 256, 128, KH * 16), sdesc(base + SB + k * 256, 128, KH * 16), id_h,
                   k > 0);
        mma_commit(bar_mma);
      }
      if (!__syncthreads_and(mbar_wait(bar_mma, ph_mma))) { failed = 1; break; }
      ph_mma ^= 1;
      tc_after_sync();
      if (l < 3 && tid == 0) {   // next layer's weights while this epilogue runs
        mbar_expect_tx(bar_ld, (uint32_t)(KH * KH * 2));
        for (int q = 0; q < 4; ++q)
          bulk_g2s(base + SB + q * 32768, reinterpret_cast<const uint8_t*>(a.blob[l + 1]) + q * 32768, 32768, bar_ld);
      }
      epilogue_hidden(sm, tmem, warp, lane, reinterpret_cast<const float*>(sm + SBIAS) + l * KH);
      fence_async_smem();
      tc_before_sync();
      __syncthreads();
    }
    if (failed) break;
    if (tid == 0) {   // layer 4: 128 x 16 = (128 x 256) (256 x 16)
      tc_after_sync();
      for (int k = 0; k < KH / 16; ++k)
        mma_bf16(tmem, sdesc(base + SA + k * 256, 128, KH * 16), sdesc(base + SW4 + k * 256, 128, KH * 16), id_o,
                 k > 0);
      mma_commit(bar_mma);
    }
    if (!__syncthreads_and(mbar_wait(bar_mma, ph_mma))) { failed = 1; break; }
    ph_mma ^= 1;
    tc_after_sync();
    if (warp < 4) {
      uint32_t v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16), v);
      tmem_wait_ld();
      const int gr = row0 + warp * 32 + lane;
      if (gr < a.M) {
        float4* dst = reinterpret_cast<float4*>(a.out + (size_t)gr * NOUT);
#pragma unroll
        for (int q = 0; q < 4; ++q)
          dst[q] = make_float4(__uint_as_float(v[4 * q]) + a.bias[4][4 * q], __uint_as_float(v[4 * q + 1]) + a.bias[4][4 * q + 1],
                               __uint_as_float(v[4 * q + 2]) + a.bias[4][4 * q + 2],
                               __uint_as_float(v[4 * q + 3]) + a.bias[4][4 * q + 3]);
      }
    }
    tc_before_sync();
    __syncthreads();
  }
  if (failed) {
    if (tid == 0) atomicExch(a.err, 1);
    // give the operation that did not complete a second bounded wait
    if (failed == 1) mbar_wait(bar_mma, ph_mma);
    else mbar_wait(bar_ld, ph_ld);
  }
  tc_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc_after_sync();
    tmem_dealloc(tmem, TMEM_COLS);
  }
}

}  // namespace mlptc
