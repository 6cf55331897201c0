// Training GEMMs of the surrogate network on the 5th-generation tensor
// cores (sm_103a).
//
// Every GEMM of one training step -- the forward layers, the input
// gradients and the weight gradients -- is D (128 x NT) = A (128 x K) B^T
// with both operands K-major, issued as tcgen05.mma kind::f16 (BF16 x BF16
// -> FP32, M = 128, K = 16 per instruction) by one thread, with the
// accumulator in tensor memory.  The operands are kept in global memory in
// the "K-slab" layout below, so the block of 128 (or NT) rows by one K chunk
// that a pipeline stage needs is one contiguous run of bytes: it arrives in
// shared memory by one cp.async.bulk, counted on that stage's mbarrier.
// Four stages overlap the copies with the MMAs.  The epilogue (4 warps, one
// TMEM lane = one output row per thread) fuses bias and GELU (forward),
// GELU' (backward) and writes each result in the layouts the next GEMMs read:
//   * activations and output gradients as A operands (rows = batch rows,
//     K = features) and, transposed, as operands of the weight gradient
//     (rows = features, K = batch rows);
//   * weight gradients as FP32 partial sums of a K split (the batch is split
//     over CTAs), added in a fixed order afterwards.
// Every mbarrier wait is bounded; on a timeout the kernel records it in
// *err, waits (bounded) once more, frees its TMEM and returns.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>

namespace mlptt {

using mlptc::core_off;

constexpr int GT_THREADS = 128;   // 4 warps: warp w owns TMEM lanes (tile rows) 32 w .. 32 w + 31
constexpr int STAGES = 4;
constexpr int KCMAX = 64;          // K columns per pipeline stage

// K-slab layout of a BF16 matrix X with R rows and K columns (R a multiple
// of 8, K a multiple of 8, K <= 64 or a multiple of 64): K is cut into
// chunks of kc = min(K, 64) columns; chunk c holds all R rows in the
// core-matrix K-major layout of an R x kc block (core_off), chunks one after
// the other.  Rows r0 .. r0 + n - 1 of one chunk are n * kc * 2 contiguous
// bytes starting at byte kslab_off(r0, c * kc, R, K).
__host__ __device__ constexpr int kslab_kc(int K) { return K < KCMAX ? K : KCMAX; }
__host__ __device__ constexpr size_t kslab_off(int r, int k, int R, int K) {
  return (size_t)(k / kslab_kc(K)) * (size_t)R * kslab_kc(K) * 2 + core_off(r, k % kslab_kc(K), kslab_kc(K));
}

enum TgMode { TG_FWD_GELU = 0, TG_FWD_OUT = 1, TG_BWD_GELU = 2, TG_WGRAD = 3 };

struct TgArgs {
  const uint8_t* A;     // K-slab, RA rows x K
  const uint8_t* B;     // K-slab, RB rows x K
  int RA, RB, K;
  int chunks;           // K chunks per CTA (the grid's z dimension splits K)
  int N;                // columns of the FP32 outputs (their row stride)
  const float* bias;    // TG_FWD_*: per column
  float* outf;          // TG_FWD_GELU: pre-activation; TG_FWD_OUT: output; TG_BWD_GELU: gradient;
                        // TG_WGRAD: partial sums [z][RA][N]
  const float* zin;     // TG_BWD_GELU: pre-activation of the layer below (stride N)
  uint8_t* oa;          // TG_FWD_GELU / TG_BWD_GELU: BF16 result as an A operand (K-slab, oaR rows x N)
  uint8_t* ot;          // ... and transposed (K-slab, N rows x otK)
  int oaR, otK;
  int* err;
};

__host__ __device__ constexpr uint32_t tg_stage_bytes(int NT) { return (uint32_t)(128 + NT) * KCMAX * 2; }
__host__ __device__ constexpr uint32_t tg_smem_bytes(int NT) { return STAGES * tg_stage_bytes(NT) + 128; }

template <int NT, int MODE>
__global__ void __launch_bounds__(GT_THREADS, 1) k_tgemm(TgArgs a) {
  using namespace mlptc;
  constexpr uint32_t TCOLS = NT < 32 ? 32 : NT;
  extern __shared__ __align__(1024) uint8_t sm[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t base = saddr(sm);
  const uint32_t bars = base + STAGES * tg_stage_bytes(NT);   // full[s], empty[s], done, TMEM address
  auto full = [&](int s) { return bars + 8 * s; };
  auto empty = [&](int s) { return bars + 8 * (STAGES + s); };
  const uint32_t done = bars + 16 * STAGES;
  const uint32_t tslot = done + 8;
  const int kc = kslab_kc(a.K);
  const uint32_t abytes = 128u * kc * 2, bbytes = (uint32_t)NT * kc * 2;
  const int m0 = blockIdx.x * 128, n0 = blockIdx.y * NT;
  const int nkc = a.K / kc;
  const int c0 = blockIdx.z * a.chunks;
  const int nk = min(a.chunks, nkc - c0);
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full(s), 1);
      mbar_init(empty(s), 1);
    }
    mbar_init(done, 1);
    fence_async_smem();
  }
  if (warp == 0) tmem_alloc(tslot, TCOLS);
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + (tslot - base));
  int failed = 0;
  if (tid == 0 && nk > 0) {
    auto load = [&](int i) {
      const int s = i % STAGES, c = c0 + i;
      const uint32_t sa = base + s * tg_stage_bytes(NT), sb = sa + 128u * KCMAX * 2;
      mbar_expect_tx(full(s), abytes + bbytes);
      bulk_g2s(sa, a.A + kslab_off(m0, c * kc, a.RA, a.K), abytes, full(s));
      bulk_g2s(sb, a.B + kslab_off(n0, c * kc, a.RB, a.K), bbytes, full(s));
    };
    for (int i = 0; i < STAGES && i < nk; ++i) load(i);
    const uint32_t idesc = idesc_bf16(128, NT);
    for (int i = 0; i < nk && !failed; ++i) {
      const int s = i % STAGES;
      const uint32_t par = (uint32_t)(i / STAGES) & 1u;
      if (!mbar_wait(full(s), par)) { failed = 2; break; }
      tc_after_sync();
      const uint32_t sa = base + s * tg_stage_bytes(NT), sb = sa + 128u * KCMAX * 2;
      for (int k = 0; k < kc / 16; ++k)
        mma_bf16(tmem, sdesc(sa + k * 256, 128, kc * 16), sdesc(sb + k * 256, 128, kc * 16), idesc, (i > 0 || k > 0));
      mma_commit(empty(s));
      if (i + STAGES < nk) {   // this stage is refilled once its MMAs have read it
        if (!mbar_wait(empty(s), par)) { failed = 1; break; }
        load(i + STAGES);
      }
    }
    if (!failed) mma_commit(done);
  }
  // everyone waits for the accumulator
  bool ok = true;
  if (nk > 0) {
    const int f = __syncthreads_or(failed);
    ok = f == 0 && __syncthreads_and(mbar_wait(done, 0));
  }
  tc_after_sync();
  if (ok && nk > 0) {
    const int r = warp * 32 + lane;   // tile row = TMEM lane
    const int gr = m0 + r;
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
    constexpr int CW = NT < 32 ? NT : 32;
#pragma unroll 1
    for (int cb = 0; cb < NT; cb += CW) {
      uint32_t v[32];
      if constexpr (CW == 32) tmem_ld32(lane_addr + (uint32_t)cb, v);
      else tmem_ld16(lane_addr + (uint32_t)cb, v);
      tmem_wait_ld();
      const int gc0 = n0 + cb;
      if constexpr (MODE == TG_WGRAD) {
        float4* dst = reinterpret_cast<float4*>(a.outf + ((size_t)blockIdx.z * a.RA + gr) * a.N + gc0);
#pragma unroll
        for (int q = 0; q < CW / 4; ++q)
          dst[q] = make_float4(__uint_as_float(v[4 * q]), __uint_as_float(v[4 * q + 1]), __uint_as_float(v[4 * q + 2]),
                               __uint_as_float(v[4 * q + 3]));
      } else if constexpr (MODE == TG_FWD_OUT) {
        float4* dst = reinterpret_cast<float4*>(a.outf + (size_t)gr * a.N + gc0);
#pragma unroll
        for (int q = 0; q < CW / 4; ++q)
          dst[q] = make_float4(__uint_as_float(v[4 * q]) + a.bias[gc0 + 4 * q],
                               __uint_as_float(v[4 * q + 1]) + a.bias[gc0 + 4 * q + 1],
                               __uint_as_float(v[4 * q + 2]) + a.bias[gc0 + 4 * q + 2],
                               __uint_as_float(v[4 * q + 3]) + a.bias[gc0 + 4 * q + 3]);
      } else {
        float f[CW];
        if constexpr (MODE == TG_FWD_GELU) {
#pragma unroll
          for (int q = 0; q < CW; ++q) f[q] = __uint_as_float(v[q]) + a.bias[gc0 + q];
          float4* zd = reinterpret_cast<float4*>(a.outf + (size_t)gr * a.N + gc0);
#pragma unroll
          for (int q = 0; q < CW / 4; ++q) zd[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
#pragma unroll
          for (int q = 0; q < CW; ++q) f[q] = gelu(f[q]);
        } else {   // TG_BWD_GELU
          const float4* zs = reinterpret_cast<const float4*>(a.zin + (size_t)gr * a.N + gc0);
#pragma unroll
          for (int q = 0; q < CW / 4; ++q) {
            const float4 z = zs[q];
            f[4 * q] = __uint_as_float(v[4 * q]) * gelu_grad(z.x);
            f[4 * q + 1] = __uint_as_float(v[4 * q + 1]) * gelu_grad(z.y);
            f[4 * q + 2] = __uint_as_float(v[4 * q + 2]) * gelu_grad(z.z);
            f[4 * q + 3] = __uint_as_float(v[4 * q + 3]) * gelu_grad(z.w);
          }
          float4* gd = reinterpret_cast<float4*>(a.outf + (size_t)gr * a.N + gc0);
#pragma unroll
          for (int q = 0; q < CW / 4; ++q) gd[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
        }
        // BF16 copies: as an A operand (row gr, K = column), 16-byte stores
        // of 8 columns; transposed (row = column, K = gr), 2-byte stores
#pragma unroll
        for (int q = 0; q < CW / 8; ++q) {
          uint32_t pk[4];
#pragma unroll
          for (int h = 0; h < 4; ++h) {
            __nv_bfloat162 b2 = __floats2bfloat162_rn(f[8 * q + 2 * h], f[8 * q + 2 * h + 1]);
            pk[h] = *reinterpret_cast<uint32_t*>(&b2);
          }
          *reinterpret_cast<uint4*>(a.oa + kslab_off(gr, gc0 + 8 * q, a.oaR, a.N)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
#pragma unroll
        for (int q = 0; q < CW; ++q)
          *reinterpret_cast<__nv_bfloat16*>(a.ot + kslab_off(gc0 + q, gr, a.N, a.otK)) = __float2bfloat16(f[q]);
      }
    }
  }
  if (!ok && nk > 0) {
    if (tid == 0) atomicExch(a.err, 1);
    mbar_wait(done, 0);   // a second bounded wait for the MMAs this CTA issued
  }
  tc_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc_after_sync();
    tmem_dealloc(tmem, TCOLS);
  }
}

// Normalised inputs of one batch (rows r0 .. r0 + M - 1 of x, 12 FP32
// columns; the caller passes x + 12 r0) -> BF16 K-slab operands: xa
// (M x 16, columns 12..15 zero) for the first layer and xt (rows 0..15 of a
// 128 x M K-slab; rows 16..127 stay zero) for its weight gradient.  Rows at
// or beyond M_valid are zero.
__global__ void k_tg_pack_input(const float* __restrict__ x, int M, int M_valid, uint8_t* __restrict__ xa,
                                uint8_t* __restrict__ xt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M * 16) return;
  const int r = i >> 4, c = i & 15;
  const __nv_bfloat16 b = __float2bfloat16(c < 12 && r < M_valid ? x[(size_t)r * 12 + c] : 0.0f);
  *reinterpret_cast<__nv_bfloat16*>(xa + kslab_off(r, c, M, 16)) = b;
  *reinterpret_cast<__nv_bfloat16*>(xt + kslab_off(c, r, 128, M)) = b;
}

// MSE loss on the 10 real outputs of rows < M_valid (targets t, 10 FP32
// columns) and its gradient 2 (out - t) / (M_valid * 10): FP32 (M x 16),
// BF16 as an A operand (M x 16 K-slab) and transposed (16 x M K-slab); the
// padded columns and rows get zero.  The loss sum is reduced per block, then
// added to *loss.
__global__ void k_tg_mse(const float* __restrict__ out, const float* __restrict__ t, int M, int M_valid,
                         float* __restrict__ gf, uint8_t* __restrict__ ga, uint8_t* __restrict__ gt,
                         double* __restrict__ loss) {
  __shared__ double red[8];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double l2 = 0.0;
  if (i < M * 16) {
    const int r = i >> 4, c = i & 15;
    float g = 0.0f;
    if (c < 10 && r < M_valid) {
      const float d = out[(size_t)r * 16 + c] - t[(size_t)r * 10 + c];
      l2 = (double)d * (double)d;
      g = 2.0f * d / (float)(M_valid * 10);
    }
    gf[i] = g;
    const __nv_bfloat16 b = __float2bfloat16(g);
    *reinterpret_cast<__nv_bfloat16*>(ga + kslab_off(r, c, M, 16)) = b;
    *reinterpret_cast<__nv_bfloat16*>(gt + kslab_off(c, r, 16, M)) = b;
  }
  for (int o = 16; o > 0; o >>= 1) l2 += __shfl_xor_sync(0xffffffffu, l2, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = l2;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    atomicAdd(loss, s);
  }
}

// Bias gradient: column sums of the FP32 output gradient (M x N), one block
// of 256 threads per column, a fixed reduction order.
__global__ void k_tg_colsum(const float* __restrict__ g, int M, int N, float* __restrict__ gb) {
  __shared__ float red[8];
  const int c = blockIdx.x;
  float s = 0.0f;
  for (int r = threadIdx.x; r < M; r += blockDim.x) s += g[(size_t)r * N + c];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    gb[c] = t;
  }
}

// Weight gradient of one layer from its split-K partials (added in split
// order) into gw (lin x lout, row-major).
__global__ void k_tg_reduce(const float* __restrict__ part, int splits, int rows_pad, int lin, int lout,
                            float* __restrict__ gw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= lin * lout) return;
  const int r = i / lout, c = i % lout;
  float s = 0.0f;
  for (int z = 0; z < splits; ++z) s += part[((size_t)z * rows_pad + r) * lout + c];
  gw[i] = s;
}

// The BF16 operand copies of layer weights W (lin x lout, row-major FP32):
// wb (row-major), wt = W^T as a K-slab (lout rows, K = lin; forward) and
// wn = W as a K-slab (lin rows, K = lout; input gradient).
__global__ void k_tg_weights(const float* __restrict__ w, int lin, int lout, __nv_bfloat16* __restrict__ wb,
                             uint8_t* __restrict__ wt, uint8_t* __restrict__ wn) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= lin * lout) return;
  const int r = i / lout, c = i % lout;
  const __nv_bfloat16 b = __float2bfloat16(w[i]);
  wb[i] = b;
  *reinterpret_cast<__nv_bfloat16*>(wt + kslab_off(c, r, lout, lin)) = b;
  *reinterpret_cast<__nv_bfloat16*>(wn + kslab_off(r, c, lin, lout)) = b;
}

}  // namespace mlptt
