// Learned chemistry surrogate: a 12 -> 4 x 256 (GELU) -> 10 MLP in BF16 with
// FP32 accumulation on the tensor cores, trained on the GPU by hand-written
// forward, backward and Adam kernels.  It has no counterpart in the
// reference: it replaces, per cell, the chemistry increment that
// reaction_dvode (module_reaction.f90:102-321) computes with DVODE; an error
// gate sends every cell it does not trust back to that integrator.
//
// Inputs  : T [K], ln p [atm], ln(Y_k + 1e-10) (9 species), ln dt [s]
// Outputs : dY_k (9 species), dT [K] over dt, in normalised units.
//
// GEMMs use mma.sync.m16n8k16 (BF16 x BF16 -> FP32) from shared-memory
// tiles; epilogues fuse bias, GELU and its derivative.
#include <cstdio>
#include <cstring>
#include <cmath>
#include <mutex>
#include <vector>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include "../../include/izem_gpu.h"
#include "chem.h"

namespace {

constexpr int IN = 12, INP = 16, OUT = 10, OUTP = 16, H = 256, NL = 5;
constexpr int LIN[NL] = {INP, H, H, H, H};
constexpr int LOUT[NL] = {H, H, H, H, OUTP};

// ---------------------------------------------------------------- GEMM ------
// C[M,N] (+)= op(A)[M,K] * op(B)[K,N].  A is given row-major [M][K] (TA = 0)
// or as [K][M] (TA = 1); B is given as [K][N] (TB = 0) or [N][K] (TB = 1).
// Tiles are staged in shared memory K-contiguous for both operands, so the
// mma fragments are plain 32-bit shared loads.
constexpr int BM = 128, BN = 128, BK = 32;

enum Epi { EPI_STORE_F32 = 0, EPI_BIAS_GELU = 1, EPI_BIAS = 2, EPI_GELU_BWD = 3 };

// GELU in the tanh form of Hendrycks and Gimpel (2016),
//   gelu(z) = 0.5 z (1 + tanh(u)),  u = sqrt(2/pi) (z + 0.044715 z^3),
// with the tanh of the special-function unit (tanh.approx.f32, relative
// error about 2^-11, below the BF16 rounding of the activations it feeds).
// Training, inference and the oracle use this same form.
constexpr float kGeluC0 = 0.7978845608028654f;    // sqrt(2/pi)
constexpr float kGeluC1 = 0.0356774081363001f;    // sqrt(2/pi) * 0.044715
__device__ __forceinline__ float tanh_sfu(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu(float z) {
  const float u = z * fmaf(kGeluC1, z * z, kGeluC0);
  const float hz = 0.5f * z;
  return fmaf(hz, tanh_sfu(u), hz);
}
// d gelu / dz = 0.5 (1 + t) + 0.5 z (1 - t^2) du/dz,  du/dz = sqrt(2/pi) (1 + 3 * 0.044715 z^2)
__device__ __forceinline__ float gelu_grad(float z) {
  const float z2 = z * z;
  const float t = tanh_sfu(z * fmaf(kGeluC1, z2, kGeluC0));
  const float du = fmaf(3.0f * kGeluC1, z2, kGeluC0);
  return fmaf(0.5f * z * du, fmaf(-t, t, 1.0f), 0.5f * (1.0f + t));
}

struct GemmArgs {
  const __nv_bfloat16* A;
  const __nv_bfloat16* B;
  int M, N, K;
  int lda, ldb;          // leading dimensions of the stored matrices
  const float* bias;     // [N]
  float* Cf;             // fp32 output (pre-activation or gradient), ld = ldc
  __nv_bfloat16* Cb;     // bf16 output (activation), ld = ldc
  const float* Zin;      // pre-activation for EPI_GELU_BWD, ld = ldc
  int ldc;
};

template <int TA, int TB, int EPI>
__global__ void __launch_bounds__(256) k_gemm(GemmArgs g) {
  __shared__ __align__(16) __nv_bfloat16 As[BM][BK + 8];
  __shared__ __align__(16) __nv_bfloat16 Bs[BN][BK + 8];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 2, wn = warp & 3;   // 2 x 4 warps, warp tile 64 x 32
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  float acc[4][4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.f;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  for (int k0 = 0; k0 < g.K; k0 += BK) {
    // stage A tile (BM x BK) and B tile (BN x BK), bounds-checked
    for (int e = tid; e < BM * BK; e += 256) {
      int mm, kk;
      if (TA == 0) { mm = e / BK; kk = e % BK; } else { kk = e / BM; mm = e % BM; }
      const int gm = m0 + mm, gk = k0 + kk;
      __nv_bfloat16 val = zero;
      if (gm < g.M && gk < g.K) val = TA == 0 ? g.A[(size_t)gm * g.lda + gk] : g.A[(size_t)gk * g.lda + gm];
      As[mm][kk] = val;
    }
    for (int e = tid; e < BN * BK; e += 256) {
      int nn, kk;
      if (TB == 1) { nn = e / BK; kk = e % BK; } else { kk = e / BN; nn = e % BN; }
      const int gn = n0 + nn, gk = k0 + kk;
      __nv_bfloat16 val = zero;
      if (gn < g.N && gk < g.K) val = TB == 1 ? g.B[(size_t)gn * g.ldb + gk] : g.B[(size_t)gk * g.ldb + gn];
      Bs[nn][kk] = val;
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < BK; ks += 16) {
      const int gid = lane >> 2, tig = lane & 3;
      unsigned afr[4][4], bfr[4][2];
#pragma unroll
      for (int fm = 0; fm < 4; ++fm) {
        const int r = wm * 64 + fm * 16 + gid;
        const int c = ks + tig * 2;
        afr[fm][0] = *reinterpret_cast<const unsigned*>(&As[r][c]);
        afr[fm][1] = *reinterpret_cast<const unsigned*>(&As[r + 8][c]);
        afr[fm][2] = *reinterpret_cast<const unsigned*>(&As[r][c + 8]);
        afr[fm][3] = *reinterpret_cast<const unsigned*>(&As[r + 8][c + 8]);
      }
#pragma unroll
      for (int fn = 0; fn < 4; ++fn) {
        const int n = wn * 32 + fn * 8 + gid;
        const int c = ks + tig * 2;
        bfr[fn][0] = *reinterpret_cast<const unsigned*>(&Bs[n][c]);
        bfr[fn][1] = *reinterpret_cast<const unsigned*>(&Bs[n][c + 8]);
      }
#pragma unroll
      for (int fm = 0; fm < 4; ++fm)
#pragma unroll
        for (int fn = 0; fn < 4; ++fn) {
          float* d = acc[fm][fn];
          asm volatile(
              "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
              "{%0,%1,%2,%3};\n"
              : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
              : "r"(afr[fm][0]), "r"(afr[fm][1]), "r"(afr[fm][2]), "r"(afr[fm][3]), "r"(bfr[fn][0]), "r"(bfr[fn][1]));
        }
    }
    __syncthreads();
  }
  // epilogue
  const int gid = lane >> 2, tig = lane & 3;
#pragma unroll
  for (int fm = 0; fm < 4; ++fm)
#pragma unroll
    for (int fn = 0; fn < 4; ++fn)
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const int r = m0 + wm * 64 + fm * 16 + gid + (h >= 2 ? 8 : 0);
        const int cc = n0 + wn * 32 + fn * 8 + tig * 2 + (h & 1);
        if (r >= g.M || cc >= g.N) continue;
        float val = acc[fm][fn][h];
        const size_t o = (size_t)r * g.ldc + cc;
        if (EPI == EPI_STORE_F32) {
          g.Cf[o] = val;
        } else if (EPI == EPI_BIAS) {
          g.Cf[o] = val + g.bias[cc];
        } else if (EPI == EPI_BIAS_GELU) {
          const float z = val + g.bias[cc];
          if (g.Cf) g.Cf[o] = z;
          g.Cb[o] = __float2bfloat16(gelu(z));
        } else {   // EPI_GELU_BWD: dZ = dA * gelu'(Z), stored as bf16 and fp32
          const float dz = val * gelu_grad(g.Zin[o]);
          if (g.Cf) g.Cf[o] = dz;
          g.Cb[o] = __float2bfloat16(dz);
        }
      }
}

template <int TA, int TB, int EPI>
cudaError_t gemm(const GemmArgs& a, cudaStream_t s) {
  dim3 grid((a.N + BN - 1) / BN, (a.M + BM - 1) / BM);
  k_gemm<TA, TB, EPI><<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// ------------------------------------------------------- small kernels ------
__global__ void k_f32_to_bf16(const float* x, __nv_bfloat16* y, long long n) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16(x[i]);
}

// loss gradient for MSE on normalised outputs (first OUT columns)
__global__ void k_mse_grad(const float* out, const float* tgt, int M, float* dout_f, __nv_bfloat16* dout_b,
                           double* loss) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)M * OUTP) return;
  const int c = (int)(i % OUTP);
  const long long r = i / OUTP;
  float d = 0.f;
  if (c < OUT) {
    d = out[i] - tgt[r * OUT + c];
    atomicAdd(loss, (double)(d * d));
  }
  const float gval = c < OUT ? 2.f * d / (float)(M * OUT) : 0.f;
  dout_f[i] = gval;
  dout_b[i] = __float2bfloat16(gval);
}

// column sums (bias gradient): db[n] = sum_m dZ[m][n]
__global__ void k_colsum(const float* dz, int M, int N, float* db) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int m = 0; m < M; ++m) s += dz[(size_t)m * N + n];
  db[n] = s;
}

__global__ void k_adam(float* w, const float* gw, float* mw, float* vw, long long n, float lr, float b1, float b2,
                       float eps, float c1, float c2, __nv_bfloat16* wb) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gr = gw[i];
  const float m = b1 * mw[i] + (1.f - b1) * gr;
  const float v = b2 * vw[i] + (1.f - b2) * gr * gr;
  mw[i] = m;
  vw[i] = v;
  const float wn = w[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
  w[i] = wn;
  if (wb) wb[i] = __float2bfloat16(wn);
}

unsigned g1(long long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

// ------------------------------------------------------------ the model -----
struct izem_mlp {
  // master FP32 parameters and Adam moments; BF16 copies used by the GEMMs
  float* W[NL] = {};
  float* b[NL] = {};
  __nv_bfloat16* Wb[NL] = {};
  float *mW[NL] = {}, *vW[NL] = {}, *mb[NL] = {}, *vb[NL] = {};
  float *gW[NL] = {}, *gb[NL] = {};
  float norm[2 * IN + 2 * OUT] = {};   // in_mean, in_std, out_mean, out_std
  // work buffers for a batch of up to cap rows
  int cap = 0;
  __nv_bfloat16* act[NL + 1] = {};   // act[0] = input (M x INP), act[l+1] = output of layer l
  float* z[NL] = {};                 // pre-activations (FP32)
  float* dzf = nullptr;              // FP32 gradient scratch (M x H)
  __nv_bfloat16* dzb[2] = {};        // BF16 gradients (ping-pong)
  float* out = nullptr;              // network output FP32 (M x OUTP)
  double* d_loss = nullptr;
  int step = 0;
  int device = 0;                    // device current at izem_mlp_create; holds every buffer
  cudaStream_t s = nullptr;
  // inference buffers: BF16 features (rows x 16) and FP32 output (rows x 16)
  long long icap = 0;
  __nv_bfloat16* ib[2] = {};
  float* iout = nullptr;
  float* d_norm = nullptr;
  // tensor-core inference: weights in the tcgen05 operand layout, rebuilt
  // from Wb whenever the parameters change; wait-timeout flag
  __nv_bfloat16* blob[NL] = {};
  bool blob_dirty = true;
  int* d_err = nullptr;
  // error-gate scratch of izem_gpu_psr_batch_mlp (kept across calls)
  int* g_kncf = nullptr;
  int* g_list = nullptr;        // rejected cells of the whole batch
  int g_list_cap = 0;
  unsigned* g_count = nullptr;   // their number
  unsigned* g_counter = nullptr;
  ChemStats* g_stats = nullptr;
};

#include "mlp_tc.cuh"

namespace {

cudaError_t mlp_ensure(izem_mlp* m, int rows) {
  if (rows <= m->cap) return cudaSuccess;
  for (int l = 0; l <= NL; ++l) if (m->act[l]) cudaFree(m->act[l]);
  for (int l = 0; l < NL; ++l) if (m->z[l]) cudaFree(m->z[l]);
  if (m->dzf) cudaFree(m->dzf);
  for (int q = 0; q < 2; ++q) if (m->dzb[q]) cudaFree(m->dzb[q]);
  if (m->out) cudaFree(m->out);
  cudaError_t e;
  const size_t M = rows;
  if ((e = cudaMalloc(&m->act[0], M * INP * sizeof(__nv_bfloat16)))) return e;
  for (int l = 0; l < NL; ++l) {
    if ((e = cudaMalloc(&m->act[l + 1], M * LOUT[l] * sizeof(__nv_bfloat16)))) return e;
    if ((e = cudaMalloc(&m->z[l], M * LOUT[l] * sizeof(float)))) return e;
  }
  if ((e = cudaMalloc(&m->dzf, M * H * sizeof(float)))) return e;
  for (int q = 0; q < 2; ++q)
    if ((e = cudaMalloc(&m->dzb[q], M * H * sizeof(__nv_bfloat16)))) return e;
  if ((e = cudaMalloc(&m->out, M * OUTP * sizeof(float)))) return e;
  m->cap = rows;
  return cudaSuccess;
}

// forward pass for M rows whose normalised inputs (bf16, M x INP) are in
// act[0]; the final layer writes FP32 outputs into m->out (and z[4]).
cudaError_t mlp_forward(izem_mlp* m, int M) {
  cudaError_t e;
  for (int l = 0; l < NL; ++l) {
    GemmArgs a{};
    a.A = m->act[l];
    a.B = m->Wb[l];
    a.M = M; a.N = LOUT[l]; a.K = LIN[l];
    a.lda = LIN[l]; a.ldb = LOUT[l]; a.ldc = LOUT[l];
    a.bias = m->b[l];
    if (l < NL - 1) {
      a.Cf = m->z[l];
      a.Cb = m->act[l + 1];
      if ((e = gemm<0, 0, EPI_BIAS_GELU>(a, m->s))) return e;
    } else {
      a.Cf = m->out;
      if ((e = gemm<0, 0, EPI_BIAS>(a, m->s))) return e;
    }
  }
  return cudaSuccess;
}

// backward pass from dL/dout (FP32 in m->dzf laid out M x OUTP, BF16 copy in
// dzb[0]) to parameter gradients gW/gb.
cudaError_t mlp_backward(izem_mlp* m, int M) {
  cudaError_t e;
  int cur = 0;
  for (int l = NL - 1; l >= 0; --l) {
    // gW[l] = act[l]^T (LIN x M) * dZ (M x LOUT)
    GemmArgs gw{};
    gw.A = m->act[l]; gw.lda = LIN[l];
    gw.B = m->dzb[cur]; gw.ldb = LOUT[l];
    gw.M = LIN[l]; gw.N = LOUT[l]; gw.K = M;
    gw.Cf = m->gW[l]; gw.ldc = LOUT[l];
    if ((e = gemm<1, 0, EPI_STORE_F32>(gw, m->s))) return e;
    k_colsum<<<(LOUT[l] + 127) / 128, 128, 0, m->s>>>(m->dzf, M, LOUT[l], m->gb[l]);
    if (l == 0) break;
    // dA[l-1] = dZ (M x LOUT) * W^T (LOUT x LIN), then * gelu'(z[l-1])
    GemmArgs gx{};
    gx.A = m->dzb[cur]; gx.lda = LOUT[l];
    gx.B = m->Wb[l]; gx.ldb = LOUT[l];   // W stored [LIN][LOUT] = [K... ]: as B^T we read [N=LIN][K=LOUT]
    gx.M = M; gx.N = LIN[l]; gx.K = LOUT[l];
    gx.Zin = m->z[l - 1];
    gx.Cf = m->dzf; gx.Cb = m->dzb[1 - cur]; gx.ldc = LIN[l];
    if ((e = gemm<0, 1, EPI_GELU_BWD>(gx, m->s))) return e;
    cur = 1 - cur;
  }
  return cudaGetLastError();
}

cudaError_t mlp_infer_ensure(izem_mlp* m, long long rows) {
  if (rows <= m->icap) return cudaSuccess;
  if (m->ib[0]) cudaFree(m->ib[0]);
  if (m->iout) cudaFree(m->iout);
  cudaError_t e;
  if ((e = cudaMalloc(&m->ib[0], (size_t)rows * INP * sizeof(__nv_bfloat16)))) return e;
  if ((e = cudaMalloc(&m->iout, (size_t)rows * OUTP * sizeof(float)))) return e;
  m->icap = rows;
  return cudaSuccess;
}

// Inference of M rows on the tensor cores: BF16 features x (M x 16) ->
// FP32 outputs y (M x 16), one persistent CTA per SM (mlp_tc.cuh).
cudaError_t mlp_infer_tc(izem_mlp* m, int M, const __nv_bfloat16* x, float* y, cudaStream_t s) {
  cudaError_t e;
  if (m->blob_dirty) {
    for (int l = 0; l < NL; ++l) {
      const int n = LIN[l] * LOUT[l];
      mlptc::k_tc_blob<<<(n + 255) / 256, 256, 0, s>>>(m->Wb[l], LIN[l], LOUT[l], m->blob[l]);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    m->blob_dirty = false;
  }
  static bool attr = false;
  if (!attr) {
    if ((e = cudaFuncSetAttribute(mlptc::k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)mlptc::SMEM_BYTES)) != cudaSuccess)
      return e;
    attr = true;
  }
  int dev = 0, sms = 0;
  if ((e = cudaGetDevice(&dev)) || (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev))) return e;
  const int ntiles = (M + mlptc::TM - 1) / mlptc::TM;
  mlptc::TcArgs a{};
  a.x = x;
  a.out = y;
  a.M = M;
  for (int l = 0; l < NL; ++l) { a.blob[l] = m->blob[l]; a.bias[l] = m->b[l]; }
  a.err = m->d_err;
  mlptc::k_mlp_tc<<<ntiles < sms ? ntiles : sms, mlptc::THREADS, mlptc::SMEM_BYTES, s>>>(a);
  return cudaGetLastError();
}

// the tensor-core kernel's wait-timeout flag (after the stream is synchronised)
int mlp_tc_status(izem_mlp* m) {
  int h = 0;
  if (cudaMemcpy(&h, m->d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return IZEM_ERR_CUDA;
  return h ? IZEM_ERR_TIMEOUT : IZEM_OK;
}

}  // namespace

// ================================================================ C ABI =====
extern "C" {

int izem_mlp_create(izem_mlp** out) {
  if (!out) return IZEM_ERR_ARG;
  izem_mlp* m = new izem_mlp();
  if (cudaGetDevice(&m->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&m->s, cudaStreamNonBlocking) != cudaSuccess) {
    delete m;
    return IZEM_ERR_CUDA;
  }
  bool ok = true;
  for (int l = 0; l < NL && ok; ++l) {
    const size_t nw = (size_t)LIN[l] * LOUT[l], nb = LOUT[l];
    ok = !(cudaMalloc(&m->W[l], nw * 4) || cudaMalloc(&m->b[l], nb * 4) || cudaMalloc(&m->Wb[l], nw * 2) ||
           cudaMalloc(&m->mW[l], nw * 4) || cudaMalloc(&m->vW[l], nw * 4) || cudaMalloc(&m->mb[l], nb * 4) ||
           cudaMalloc(&m->vb[l], nb * 4) || cudaMalloc(&m->gW[l], nw * 4) || cudaMalloc(&m->gb[l], nb * 4));
    if (ok) {
      cudaMemset(m->mW[l], 0, nw * 4); cudaMemset(m->vW[l], 0, nw * 4);
      cudaMemset(m->mb[l], 0, nb * 4); cudaMemset(m->vb[l], 0, nb * 4);
    }
  }
  ok = ok && cudaMalloc(&m->d_loss, sizeof(double)) == cudaSuccess;
  for (int l = 0; l < NL && ok; ++l) ok = cudaMalloc(&m->blob[l], (size_t)LIN[l] * LOUT[l] * 2) == cudaSuccess;
  ok = ok && cudaMalloc(&m->d_err, sizeof(int)) == cudaSuccess && cudaMemset(m->d_err, 0, sizeof(int)) == cudaSuccess;
  if (!ok) {
    izem_mlp_destroy(m);   // frees what was allocated (cudaFree of a null pointer is a no-op)
    return IZEM_ERR_NOMEM;
  }
  *out = m;
  return IZEM_OK;
}

void izem_mlp_destroy(izem_mlp* m) {
  if (!m) return;
  cudaStreamSynchronize(m->s);
  for (int l = 0; l < NL; ++l) {
    cudaFree(m->W[l]); cudaFree(m->b[l]); cudaFree(m->Wb[l]); cudaFree(m->mW[l]); cudaFree(m->vW[l]);
    cudaFree(m->mb[l]); cudaFree(m->vb[l]); cudaFree(m->gW[l]); cudaFree(m->gb[l]); cudaFree(m->z[l]);
  }
  for (int l = 0; l <= NL; ++l) cudaFree(m->act[l]);
  cudaFree(m->dzf); cudaFree(m->dzb[0]); cudaFree(m->dzb[1]); cudaFree(m->out); cudaFree(m->d_loss);
  cudaFree(m->ib[0]); cudaFree(m->ib[1]); cudaFree(m->iout); cudaFree(m->d_norm);
  for (int l = 0; l < NL; ++l) cudaFree(m->blob[l]);
  cudaFree(m->d_err);
  cudaFree(m->g_kncf); cudaFree(m->g_list); cudaFree(m->g_count); cudaFree(m->g_counter); cudaFree(m->g_stats);
  cudaStreamDestroy(m->s);
  delete m;
}

// Parameters as FP32 host arrays: W_l stored [in][out] row-major (padded
// dimensions 16/256/256/256/256 -> 256/.../16), b_l [out].  The BF16 copies
// used by the tensor-core GEMMs are rounded from these.
int izem_mlp_set_params(izem_mlp* m, const float* const* W, const float* const* b) {
  if (!m || !W || !b) return IZEM_ERR_ARG;
  m->blob_dirty = true;
  for (int l = 0; l < NL; ++l) {
    const size_t nw = (size_t)LIN[l] * LOUT[l];
    if (cudaMemcpy(m->W[l], W[l], nw * 4, cudaMemcpyHostToDevice) != cudaSuccess) return IZEM_ERR_CUDA;
    if (cudaMemcpy(m->b[l], b[l], LOUT[l] * 4, cudaMemcpyHostToDevice) != cudaSuccess) return IZEM_ERR_CUDA;
    k_f32_to_bf16<<<g1(nw), 256, 0, m->s>>>(m->W[l], m->Wb[l], nw);
  }
  return cudaStreamSynchronize(m->s) == cudaSuccess ? IZEM_OK : IZEM_ERR_CUDA;
}

int izem_mlp_get_params(izem_mlp* m, float* const* W, float* const* b) {
  if (!m || !W || !b) return IZEM_ERR_ARG;
  for (int l = 0; l < NL; ++l) {
    const size_t nw = (size_t)LIN[l] * LOUT[l];
    if (cudaMemcpy(W[l], m->W[l], nw * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return IZEM_ERR_CUDA;
    if (cudaMemcpy(b[l], m->b[l], LOUT[l] * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return IZEM_ERR_CUDA;
  }
  return IZEM_OK;
}

int izem_mlp_set_norm(izem_mlp* m, const float* norm) {
  if (!m || !norm) return IZEM_ERR_ARG;
  std::memcpy(m->norm, norm, sizeof(m->norm));
  return IZEM_OK;
}

// Forward on M rows of normalised inputs x (M x 12, FP32, host); writes the
// normalised outputs (M x 10, FP32, host).
int izem_mlp_forward(izem_mlp* m, int M, const float* x, float* y) {
  if (!m || M <= 0 || !x || !y) return IZEM_ERR_ARG;
  if (mlp_infer_ensure(m, M) != cudaSuccess) return IZEM_ERR_NOMEM;
  std::vector<float> xp((size_t)M * INP, 0.f);
  for (int r = 0; r < M; ++r)
    for (int c = 0; c < IN; ++c) xp[(size_t)r * INP + c] = x[(size_t)r * IN + c];
  float* dx = nullptr;
  if (cudaMalloc(&dx, xp.size() * 4) != cudaSuccess) return IZEM_ERR_NOMEM;
  if (cudaMemcpy(dx, xp.data(), xp.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(dx);
    return IZEM_ERR_CUDA;
  }
  k_f32_to_bf16<<<g1(xp.size()), 256, 0, m->s>>>(dx, m->ib[0], (long long)xp.size());
  int rc = cudaGetLastError() == cudaSuccess ? IZEM_OK : IZEM_ERR_CUDA;
  if (rc == IZEM_OK && mlp_infer_tc(m, M, m->ib[0], m->iout, m->s) != cudaSuccess) rc = IZEM_ERR_CUDA;
  std::vector<float> o((size_t)M * OUTP);
  if (cudaMemcpyAsync(o.data(), m->iout, o.size() * 4, cudaMemcpyDeviceToHost, m->s) != cudaSuccess) rc = IZEM_ERR_CUDA;
  if (cudaStreamSynchronize(m->s) != cudaSuccess) rc = IZEM_ERR_CUDA;
  if (rc == IZEM_OK) rc = mlp_tc_status(m);
  cudaFree(dx);
  for (int r = 0; r < M; ++r)
    for (int c = 0; c < OUT; ++c) y[(size_t)r * OUT + c] = o[(size_t)r * OUTP + c];
  return rc;
}

// Loss and parameter gradients of the MSE loss for M rows (normalised x and
// targets t, host FP32); gradients copied to host arrays shaped like the
// parameters.  Used to check the backward kernels against the FP64 oracle.
int izem_mlp_grads(izem_mlp* m, int M, const float* x, const float* t, double* loss, float* const* gW,
                   float* const* gb) {
  if (!m || M <= 0 || !x || !t) return IZEM_ERR_ARG;
  if (mlp_ensure(m, M) != cudaSuccess) return IZEM_ERR_NOMEM;
  std::vector<float> xp((size_t)M * INP, 0.f);
  for (int r = 0; r < M; ++r)
    for (int c = 0; c < IN; ++c) xp[(size_t)r * INP + c] = x[(size_t)r * IN + c];
  float *dx = nullptr, *dt = nullptr;
  if (cudaMalloc(&dx, xp.size() * 4) != cudaSuccess) return IZEM_ERR_NOMEM;
  if (cudaMalloc(&dt, (size_t)M * OUT * 4) != cudaSuccess) {
    cudaFree(dx);
    return IZEM_ERR_NOMEM;
  }
  if (cudaMemcpy(dx, xp.data(), xp.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dt, t, (size_t)M * OUT * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(dx);
    cudaFree(dt);
    return IZEM_ERR_CUDA;
  }
  k_f32_to_bf16<<<g1(xp.size()), 256, 0, m->s>>>(dx, m->act[0], (long long)xp.size());
  int rc = IZEM_OK;
  if (mlp_forward(m, M) != cudaSuccess) rc = IZEM_ERR_CUDA;
  cudaMemsetAsync(m->d_loss, 0, sizeof(double), m->s);
  k_mse_grad<<<g1((long long)M * OUTP), 256, 0, m->s>>>(m->out, dt, M, m->dzf, m->dzb[0], m->d_loss);
  if (rc == IZEM_OK && mlp_backward(m, M) != cudaSuccess) rc = IZEM_ERR_CUDA;
  cudaMemcpyAsync(loss, m->d_loss, sizeof(double), cudaMemcpyDeviceToHost, m->s);
  for (int l = 0; l < NL; ++l) {
    cudaMemcpyAsync(gW[l], m->gW[l], (size_t)LIN[l] * LOUT[l] * 4, cudaMemcpyDeviceToHost, m->s);
    cudaMemcpyAsync(gb[l], m->gb[l], LOUT[l] * 4, cudaMemcpyDeviceToHost, m->s);
  }
  if (cudaStreamSynchronize(m->s) != cudaSuccess) rc = IZEM_ERR_CUDA;
  *loss = *loss / ((double)M * OUT);
  cudaFree(dx);
  cudaFree(dt);
  return rc;
}

// Adam training on n rows of normalised inputs x (n x 12) and targets t
// (n x 10), device FP32 arrays when device_ptrs, else host.  Mini-batches
// of `batch` rows in a fixed seeded permutation per epoch; losses[e] gets
// the mean loss of epoch e.
int izem_mlp_train(izem_mlp* m, long long n, const float* x, const float* t, int device_ptrs, int epochs, int batch,
                   float lr, unsigned seed, double* losses) {
  if (!m || n < batch || !x || !t || epochs <= 0 || batch <= 0) return IZEM_ERR_ARG;
  if (mlp_ensure(m, batch) != cudaSuccess) return IZEM_ERR_NOMEM;
  float *dx = nullptr, *dt = nullptr, *bx = nullptr, *bt = nullptr;
  int rc = IZEM_OK;
  if (device_ptrs) {
    dx = const_cast<float*>(x);
    dt = const_cast<float*>(t);
  } else {
    if (cudaMalloc(&dx, n * IN * 4) || cudaMalloc(&dt, n * OUT * 4)) return IZEM_ERR_NOMEM;
    cudaMemcpy(dx, x, n * IN * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(dt, t, n * OUT * 4, cudaMemcpyHostToDevice);
  }
  if (cudaMalloc(&bx, (size_t)batch * INP * 4) || cudaMalloc(&bt, (size_t)batch * OUT * 4)) return IZEM_ERR_NOMEM;
  cudaMemset(bx, 0, (size_t)batch * INP * 4);
  const long long nb = n / batch;
  std::vector<long long> perm(nb);
  unsigned long long st = seed ? seed : 1ULL;
  for (int ep = 0; ep < epochs; ++ep) {
    for (long long q = 0; q < nb; ++q) perm[q] = q;
    for (long long q = nb - 1; q > 0; --q) {   // Fisher-Yates on batch indices (xorshift)
      st ^= st << 13; st ^= st >> 7; st ^= st << 17;
      long long r = (long long)(st % (unsigned long long)(q + 1));
      long long tmp = perm[q]; perm[q] = perm[r]; perm[r] = tmp;
    }
    cudaMemsetAsync(m->d_loss, 0, sizeof(double), m->s);
    for (long long q = 0; q < nb; ++q) {
      const long long r0 = perm[q] * batch;
      cudaMemcpy2DAsync(bx, INP * 4, dx + r0 * IN, IN * 4, IN * 4, batch, cudaMemcpyDeviceToDevice, m->s);
      cudaMemcpyAsync(bt, dt + r0 * OUT, (size_t)batch * OUT * 4, cudaMemcpyDeviceToDevice, m->s);
      k_f32_to_bf16<<<g1((long long)batch * INP), 256, 0, m->s>>>(bx, m->act[0], (long long)batch * INP);
      if (mlp_forward(m, batch) != cudaSuccess) { rc = IZEM_ERR_CUDA; break; }
      k_mse_grad<<<g1((long long)batch * OUTP), 256, 0, m->s>>>(m->out, bt, batch, m->dzf, m->dzb[0], m->d_loss);
      if (mlp_backward(m, batch) != cudaSuccess) { rc = IZEM_ERR_CUDA; break; }
      m->step += 1;
      m->blob_dirty = true;
      const float b1 = 0.9f, b2 = 0.999f;
      const float c1 = 1.f - powf(b1, (float)m->step), c2 = 1.f - powf(b2, (float)m->step);
      for (int l = 0; l < NL; ++l) {
        const long long nw = (long long)LIN[l] * LOUT[l];
        k_adam<<<g1(nw), 256, 0, m->s>>>(m->W[l], m->gW[l], m->mW[l], m->vW[l], nw, lr, b1, b2, 1e-8f, c1, c2, m->Wb[l]);
        k_adam<<<g1(LOUT[l]), 256, 0, m->s>>>(m->b[l], m->gb[l], m->mb[l], m->vb[l], LOUT[l], lr, b1, b2, 1e-8f, c1, c2,
                                             nullptr);
      }
    }
    double lsum = 0.0;
    cudaMemcpyAsync(&lsum, m->d_loss, sizeof(double), cudaMemcpyDeviceToHost, m->s);
    if (cudaStreamSynchronize(m->s) != cudaSuccess) { rc = IZEM_ERR_CUDA; break; }
    if (losses) losses[ep] = lsum / ((double)nb * batch * OUT);
    if (rc) break;
  }
  cudaFree(bx);
  cudaFree(bt);
  if (!device_ptrs) { cudaFree(dx); cudaFree(dt); }
  return rc;
}

// Surrogate chemistry on n independent reactors (same arrays as
// izem_gpu_psr_batch): MLP inference and the error gate in chunks of 2^20
// rows, the rejected cells of all chunks collected in one list, then one
// BDF launch over that list (one load-balanced pass, so the slowest stiff
// cell is waited for once, not once per chunk).  gate10 = {Tmin, Tmax, dtmin, dtmax,
// tol_el, tol_T_abs, tol_T_rel, tol_ens_abs, tol_ens_rel, dT_cap}; m2 (optional) is
// a second, independently trained network: the prediction is the mean of
// the two, and cells where their dT disagree are rejected;
// kncf = element counts [kk][nele].
// dT_pred (optional, device or host like the other arrays) receives the raw
// network temperature increment.  stats3 = {fallback cells, max BDF steps,
// failed}; ms2 = {total kernel ms, MLP-only ms}.
int izem_gpu_psr_batch_mlp(izem_mlp* m, izem_mlp* m2, const izem_mech* mech, int n, double* T, const double* rho,
                           double* Y, const double* dt, int device_ptrs, const double* gate10, const int* kncf, int nele,
                           double* dT_pred, int* stats3, float* ms2) {
  if (!m || !mech || n <= 0 || !T || !rho || !Y || !dt || !gate10 || !kncf || mech->kk != 9) return IZEM_ERR_ARG;
  if (nele <= 0 || nele > 8) return IZEM_ERR_ARG;
  const int CH = 1 << 20;
  const int chunk = n < CH ? n : CH;
  const int nch = (n + chunk - 1) / chunk;
  cudaStream_t s = m->s;
  if (mlp_infer_ensure(m, chunk) != cudaSuccess) return IZEM_ERR_NOMEM;
  if (m2 && mlp_infer_ensure(m2, chunk) != cudaSuccess) return IZEM_ERR_NOMEM;
  if (!m->d_norm && cudaMalloc(&m->d_norm, sizeof(m->norm)) != cudaSuccess) return IZEM_ERR_NOMEM;
  if (m2 && !m2->d_norm && cudaMalloc(&m2->d_norm, sizeof(m2->norm)) != cudaSuccess) return IZEM_ERR_NOMEM;
  // gate scratch kept in the handle: element counts, fallback list, per-chunk counts
  if (!m->g_kncf && cudaMalloc(&m->g_kncf, IZEM_NSMAX * 8 * sizeof(int)) != cudaSuccess) return IZEM_ERR_NOMEM;
  if (!m->g_counter && (cudaMalloc(&m->g_counter, sizeof(unsigned)) != cudaSuccess ||
                        cudaMalloc(&m->g_count, sizeof(unsigned)) != cudaSuccess ||
                        cudaMalloc(&m->g_stats, sizeof(ChemStats)) != cudaSuccess))
    return IZEM_ERR_NOMEM;
  if (n > m->g_list_cap) {
    cudaFree(m->g_list);
    m->g_list = nullptr;
    if (cudaMalloc(&m->g_list, (size_t)n * sizeof(int)) != cudaSuccess) return IZEM_ERR_NOMEM;
    m->g_list_cap = n;
  }
  if (chem_upload_mech(mech) != cudaSuccess) return IZEM_ERR_CUDA;
  cudaMemcpyAsync(m->d_norm, m->norm, sizeof(m->norm), cudaMemcpyHostToDevice, s);
  if (m2) cudaMemcpyAsync(m2->d_norm, m2->norm, sizeof(m2->norm), cudaMemcpyHostToDevice, s);
  const size_t kk = mech->kk;
  cudaMemcpyAsync(m->g_kncf, kncf, kk * nele * sizeof(int), cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(m->g_stats, 0, sizeof(ChemStats), s);
  cudaMemsetAsync(m->g_count, 0, sizeof(unsigned), s);
  double *dT = nullptr, *drho = nullptr, *dY = nullptr, *ddt = nullptr, *ddTp = nullptr;
  int rc = IZEM_OK;
  if (device_ptrs) {
    dT = T; drho = const_cast<double*>(rho); dY = Y; ddt = const_cast<double*>(dt); ddTp = dT_pred;
  } else {
    const size_t n8 = (size_t)n * 8;
    if (cudaMalloc(&dT, n8) || cudaMalloc(&drho, n8) || cudaMalloc(&dY, n8 * kk) || cudaMalloc(&ddt, n8) ||
        (dT_pred && cudaMalloc(&ddTp, n8))) {
      // cudaFree(nullptr) is a no-op: release whatever the chain allocated
      cudaFree(dT); cudaFree(drho); cudaFree(dY); cudaFree(ddt); cudaFree(ddTp);
      return IZEM_ERR_NOMEM;
    }
    if (cudaMemcpyAsync(dT, T, n8, cudaMemcpyHostToDevice, s) || cudaMemcpyAsync(drho, rho, n8, cudaMemcpyHostToDevice, s) ||
        cudaMemcpyAsync(dY, Y, n8 * kk, cudaMemcpyHostToDevice, s) || cudaMemcpyAsync(ddt, dt, n8, cudaMemcpyHostToDevice, s))
      rc = IZEM_ERR_CUDA;
  }
  std::vector<cudaEvent_t> ev(2 * nch + 2);
  for (auto& e : ev) cudaEventCreate(&e);
  cudaEventRecord(ev[0], s);
  for (int ci = 0; ci < nch && rc == IZEM_OK; ++ci) {
    const int c0 = ci * chunk;
    const int cn = (n - c0) < chunk ? (n - c0) : chunk;
    cudaEventRecord(ev[2 + 2 * ci], s);
    chem_launch_featurize(cn, dT + c0, drho + c0, dY + (size_t)c0 * kk, ddt + c0, m->d_norm, m->ib[0],
                          m2 ? m2->d_norm : nullptr, m2 ? m2->ib[0] : nullptr, s);
    if (mlp_infer_tc(m, cn, m->ib[0], m->iout, s) != cudaSuccess) { rc = IZEM_ERR_CUDA; break; }
    if (m2 && mlp_infer_tc(m2, cn, m2->ib[0], m2->iout, s) != cudaSuccess) { rc = IZEM_ERR_CUDA; break; }
    cudaEventRecord(ev[3 + 2 * ci], s);
    chem_launch_decode_gate(cn, m->iout, m2 ? m2->iout : nullptr, OUTP, m->d_norm, m2 ? m2->d_norm : nullptr, dT + c0,
                            drho + c0, dY + (size_t)c0 * kk, ddt + c0, gate10, m->g_kncf, nele, m->g_list, c0,
                            m->g_count, ddTp ? ddTp + c0 : nullptr, m->g_stats, s);
  }
  if (rc == IZEM_OK && chem_launch_list(m->g_list, m->g_count, dT, drho, dY, ddt, m->g_counter, m->g_stats, s) !=
                           cudaSuccess)
    rc = IZEM_ERR_CUDA;
  cudaEventRecord(ev[1], s);
  ChemStats hs{};
  unsigned nfb = 0;
  cudaMemcpyAsync(&hs, m->g_stats, sizeof(ChemStats), cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(&nfb, m->g_count, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (!device_ptrs) {
    cudaMemcpyAsync(T, dT, (size_t)n * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(Y, dY, (size_t)n * kk * 8, cudaMemcpyDeviceToHost, s);
    if (dT_pred) cudaMemcpyAsync(dT_pred, ddTp, (size_t)n * 8, cudaMemcpyDeviceToHost, s);
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) rc = IZEM_ERR_CUDA;
  if (rc == IZEM_OK) rc = mlp_tc_status(m);
  if (rc == IZEM_OK && m2) rc = mlp_tc_status(m2);
  float ms_tot = 0.f, ms_mlp = 0.f;
  cudaEventElapsedTime(&ms_tot, ev[0], ev[1]);
  for (int ci = 0; ci < nch; ++ci) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ev[2 + 2 * ci], ev[3 + 2 * ci]) == cudaSuccess) ms_mlp += ms;
  }
  if (ms2) { ms2[0] = ms_tot; ms2[1] = ms_mlp; }
  if (stats3) { stats3[0] = (int)nfb; stats3[1] = hs.max_steps; stats3[2] = hs.failed; }
  for (auto& e : ev) cudaEventDestroy(e);
  if (!device_ptrs) { cudaFree(dT); cudaFree(drho); cudaFree(dY); cudaFree(ddt); if (ddTp) cudaFree(ddTp); }
  if (rc == IZEM_OK && hs.failed) rc = IZEM_ERR_CHEM;
  return rc;
}


// The cells the last izem_gpu_psr_batch_mlp call on m sent to the BDF
// integrator, as indices into that call's batch, in no particular order:
// up to cap of them are copied to out (host), *count receives their number.
int izem_mlp_fallback_cells(izem_mlp* m, int* out, int cap, int* count) {
  if (!m || !count || (cap > 0 && !out)) return IZEM_ERR_ARG;
  unsigned nfb = 0;
  if (m->g_count && cudaMemcpy(&nfb, m->g_count, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess)
    return IZEM_ERR_CUDA;
  *count = (int)nfb;
  const int ncopy = (int)nfb < cap ? (int)nfb : cap;
  if (ncopy > 0 && cudaMemcpy(out, m->g_list, (size_t)ncopy * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return IZEM_ERR_CUDA;
  return IZEM_OK;
}

}  // extern "C"

// ===================================================== no-alloc inference ===
// Surrogate inference for callers that cannot allocate device memory while
// they run: a flow solver that hands the whole GPU to its own memory arena
// (or to a framework's caching allocator) at start-up, or that calls the
// surrogate inside its time-step loop, where a cudaMalloc/cudaFree would
// synchronise the whole device and stall its other streams.  The activations
// that izem_mlp_forward keeps in per-handle buffers live here in one
// file-scope device array instead, sized for IZEM_MLP_NOALLOC_MAX_ROWS rows.
//
// The array exists once per device for the life of the process.  Its name,
// used in host code, is only a host-side stand-in: host code passes kernels
// the device address looked up with cudaGetSymbolAddress, once per device.
namespace {

constexpr int NA_ROWS = IZEM_MLP_NOALLOC_MAX_ROWS;
constexpr size_t NA_ACT_BYTES = (size_t)NA_ROWS * H * sizeof(__nv_bfloat16);   // one activation buffer
constexpr size_t NA_OUT_BYTES = (size_t)NA_ROWS * OUTP * sizeof(float);
constexpr size_t NA_BYTES = 2 * NA_ACT_BYTES + NA_OUT_BYTES;                    // 4 MiB + 256 KiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

constexpr int NA_MAX_DEV = 64;
unsigned char* g_noalloc_addr[NA_MAX_DEV] = {};   // device address per device ordinal
std::mutex g_noalloc_mu;

// The array's device address on the current device (looked up on the first
// call per device).
cudaError_t noalloc_scratch(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= NA_MAX_DEV) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    if ((e = cudaGetSymbolAddress(&p, g_noalloc_scratch)) != cudaSuccess) return e;
    g_noalloc_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_noalloc_addr[dev];
  return cudaSuccess;
}

// x (M x 12 FP32) -> BF16 rows padded to 16 columns.  The padding columns are
// written as zeros on every call: the array keeps the previous call's data.
__global__ void k_na_pack(const float* __restrict__ x, int M, __nv_bfloat16* __restrict__ a) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)M * INP) return;
  const int r = (int)(i / INP), c = (int)(i % INP);
  a[i] = __float2bfloat16(c < IN ? x[(size_t)r * IN + c] : 0.0f);
}

// network output (M x 16 FP32) -> y (M x 10 FP32)
__global__ void k_na_unpack(const float* __restrict__ o, int M, float* __restrict__ y) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)M * OUT) return;
  const int r = (int)(i / OUT), c = (int)(i % OUT);
  y[i] = o[(size_t)r * OUTP + c];
}

}  // namespace

extern "C" int izem_mlp_forward_noalloc(izem_mlp* m, int M, const float* d_x, float* d_y, void* stream) {
  if (!m || !d_x || !d_y || M <= 0) return IZEM_ERR_ARG;
  if (M > NA_ROWS) return IZEM_ERR_TOO_LARGE;
  // the weights live on the device the handle was created on; the scratch
  // array is taken from the current device, so the two must be the same
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return IZEM_ERR_CUDA;
  if (dev != m->device) return IZEM_ERR_ARG;
  // an error left by an earlier, unrelated launch is not this call's
  (void)cudaGetLastError();
  unsigned char* base = nullptr;
  if (noalloc_scratch(&base) != cudaSuccess) return IZEM_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  __nv_bfloat16* buf[2] = {reinterpret_cast<__nv_bfloat16*>(base),
                           reinterpret_cast<__nv_bfloat16*>(base + NA_ACT_BYTES)};
  float* out = reinterpret_cast<float*>(base + 2 * NA_ACT_BYTES);
  k_na_pack<<<g1((long long)M * INP), 256, 0, s>>>(d_x, M, buf[0]);
  if (cudaGetLastError() != cudaSuccess) return IZEM_ERR_CUDA;
  int cur = 0;
  for (int l = 0; l < NL; ++l) {
    GemmArgs a{};
    a.A = buf[cur];
    a.B = m->Wb[l];
    a.M = M; a.N = LOUT[l]; a.K = LIN[l];
    a.lda = LIN[l]; a.ldb = LOUT[l]; a.ldc = LOUT[l];
    a.bias = m->b[l];
    cudaError_t e;
    if (l < NL - 1) {
      a.Cb = buf[1 - cur];
      e = gemm<0, 0, EPI_BIAS_GELU>(a, s);
      cur = 1 - cur;
    } else {
      a.Cf = out;
      e = gemm<0, 0, EPI_BIAS>(a, s);
    }
    if (e != cudaSuccess) return IZEM_ERR_CUDA;
  }
  k_na_unpack<<<g1((long long)M * OUT), 256, 0, s>>>(out, M, d_y);
  return cudaGetLastError() == cudaSuccess ? IZEM_OK : IZEM_ERR_CUDA;
}
