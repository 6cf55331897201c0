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
// Every GEMM runs on the 5th-generation tensor cores (tcgen05.mma, BF16 x
// BF16 -> FP32 in tensor memory): inference in one fused persistent kernel
// (mlp_tc.cuh), training in pipelined GEMM kernels whose epilogues fuse
// bias, GELU and its derivative (mlp_train_tc.cuh).
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

// ------------------------------------------------------- small kernels ------
__global__ void k_f32_to_bf16(const float* x, __nv_bfloat16* y, long long n) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16(x[i]);
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
  // training buffers for batches of up to cap rows (a multiple of 128),
  // operands in the K-slab layout of mlp_train_tc.cuh
  int cap = 0;
  uint8_t *xa = nullptr, *xt = nullptr;          // inputs: cap x 16; transposed 128 x cap
  uint8_t *acta[NL - 1] = {}, *actt[NL - 1] = {};   // hidden activations: cap x 256; 256 x cap
  float* z[NL - 1] = {};                         // hidden pre-activations (FP32, cap x 256)
  float* out = nullptr;                          // network output (FP32, cap x 16)
  float* gout = nullptr;                         // output gradient (FP32, cap x 16) ...
  uint8_t *goa = nullptr, *got = nullptr;        // ... as K-slabs: cap x 16; 16 x cap
  float* dzf = nullptr;                          // hidden gradient (FP32, cap x 256) ...
  uint8_t *dza[2] = {}, *dzt = nullptr;          // ... as K-slabs: cap x 256 (two); 256 x cap
  float* part = nullptr;                         // split-K partial weight gradients
  int splits = 0, split_chunks = 0;              // K split of the weight-gradient GEMMs
  uint8_t *wt[NL] = {}, *wn[NL] = {};            // BF16 weights as K-slabs: W^T (forward), W (backward)
  double* d_loss = nullptr;
  int step = 0;
  int residual = 0;                  // trained on the increment minus dt f(y0) (izem_mlp_set_residual)
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
#include "mlp_train_tc.cuh"

namespace {

// Training buffers for batches of up to `rows` rows (rounded up to 128).
cudaError_t mlp_ensure(izem_mlp* m, int rows) {
  rows = (rows + 127) / 128 * 128;
  if (rows <= m->cap) return cudaSuccess;
  cudaFree(m->xa); cudaFree(m->xt); cudaFree(m->out); cudaFree(m->gout); cudaFree(m->goa); cudaFree(m->got);
  cudaFree(m->dzf); cudaFree(m->dza[0]); cudaFree(m->dza[1]); cudaFree(m->dzt); cudaFree(m->part);
  for (int l = 0; l < NL - 1; ++l) { cudaFree(m->acta[l]); cudaFree(m->actt[l]); cudaFree(m->z[l]); }
  m->cap = 0;
  const size_t M = rows;
  // the weight-gradient GEMMs split the batch (K = rows, chunks of 64) over
  // up to 32 CTAs per output tile
  const int nchunks = rows / mlptt::KCMAX;
  m->split_chunks = nchunks / 32 > 1 ? nchunks / 32 : 1;
  m->splits = (nchunks + m->split_chunks - 1) / m->split_chunks;
  cudaError_t e;
  if ((e = cudaMalloc(&m->xa, M * 16 * 2)) || (e = cudaMalloc(&m->xt, 128 * M * 2)) ||
      (e = cudaMemset(m->xt, 0, 128 * M * 2)) || (e = cudaMalloc(&m->out, M * 16 * 4)) ||
      (e = cudaMalloc(&m->gout, M * 16 * 4)) || (e = cudaMalloc(&m->goa, M * 16 * 2)) ||
      (e = cudaMalloc(&m->got, M * 16 * 2)) || (e = cudaMalloc(&m->dzf, M * H * 4)) ||
      (e = cudaMalloc(&m->dza[0], M * H * 2)) || (e = cudaMalloc(&m->dza[1], M * H * 2)) ||
      (e = cudaMalloc(&m->dzt, M * H * 2)) || (e = cudaMalloc(&m->part, (size_t)m->splits * H * H * 4)))
    return e;
  for (int l = 0; l < NL - 1; ++l)
    if ((e = cudaMalloc(&m->acta[l], M * H * 2)) || (e = cudaMalloc(&m->actt[l], M * H * 2)) ||
        (e = cudaMalloc(&m->z[l], M * H * 4)))
      return e;
  m->cap = rows;
  return cudaSuccess;
}

template <int NT, int MODE>
cudaError_t tg_launch(const mlptt::TgArgs& a, int mt, int nt, int splits, cudaStream_t s) {
  static bool attr = false;
  cudaError_t e;
  if (!attr) {
    if ((e = cudaFuncSetAttribute(mlptt::k_tgemm<NT, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)mlptt::tg_smem_bytes(NT))) != cudaSuccess)
      return e;
    attr = true;
  }
  mlptt::k_tgemm<NT, MODE><<<dim3(mt, nt, splits), mlptt::GT_THREADS, mlptt::tg_smem_bytes(NT), s>>>(a);
  return cudaGetLastError();
}

// Forward pass of M rows (a multiple of 128) whose inputs are in m->xa:
// hidden pre-activations and activations of every layer kept for the
// backward pass, FP32 outputs in m->out.
cudaError_t mlp_forward(izem_mlp* m, int M) {
  cudaError_t e;
  for (int l = 0; l < NL; ++l) {
    mlptt::TgArgs a{};
    a.A = l == 0 ? m->xa : m->acta[l - 1];
    a.RA = M;
    a.B = m->wt[l];
    a.RB = LOUT[l];
    a.K = LIN[l];
    a.chunks = LIN[l] / mlptt::kslab_kc(LIN[l]);
    a.N = LOUT[l];
    a.bias = m->b[l];
    a.err = m->d_err;
    if (l < NL - 1) {
      a.outf = m->z[l];
      a.oa = m->acta[l];
      a.ot = m->actt[l];
      a.oaR = M;
      a.otK = M;
      e = tg_launch<128, mlptt::TG_FWD_GELU>(a, M / 128, H / 128, 1, m->s);
    } else {
      a.outf = m->out;
      e = tg_launch<OUTP, mlptt::TG_FWD_OUT>(a, M / 128, 1, 1, m->s);
    }
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Backward pass of M rows from the output gradient in m->gout / m->goa /
// m->got to the parameter gradients gW, gb.
cudaError_t mlp_backward(izem_mlp* m, int M) {
  cudaError_t e;
  const uint8_t* gA = m->goa;   // this layer's output gradient as an A operand
  int nxt = 0;
  for (int l = NL - 1; l >= 0; --l) {
    // gW_l = act_l^T dZ_l: K = the batch, split over CTAs, partials added in order
    mlptt::TgArgs w{};
    w.A = l == 0 ? m->xt : m->actt[l - 1];
    w.RA = l == 0 ? 128 : H;
    w.B = l == NL - 1 ? m->got : m->dzt;
    w.RB = LOUT[l];
    w.K = M;
    w.chunks = m->split_chunks;
    w.N = LOUT[l];
    w.outf = m->part;
    w.err = m->d_err;
    const int splits = (M / mlptt::KCMAX + w.chunks - 1) / w.chunks;
    if (l == NL - 1) e = tg_launch<OUTP, mlptt::TG_WGRAD>(w, w.RA / 128, 1, splits, m->s);
    else e = tg_launch<H, mlptt::TG_WGRAD>(w, w.RA / 128, 1, splits, m->s);
    if (e != cudaSuccess) return e;
    const int nw = LIN[l] * LOUT[l];
    mlptt::k_tg_reduce<<<(nw + 255) / 256, 256, 0, m->s>>>(m->part, splits, w.RA, LIN[l], LOUT[l], m->gW[l]);
    mlptt::k_tg_colsum<<<LOUT[l], 256, 0, m->s>>>(l == NL - 1 ? m->gout : m->dzf, M, LOUT[l], m->gb[l]);
    if (l == 0) break;
    // dZ_{l-1} = (dZ_l W_l^T) gelu'(z_{l-1})
    mlptt::TgArgs d{};
    d.A = gA;
    d.RA = M;
    d.B = m->wn[l];
    d.RB = LIN[l];
    d.K = LOUT[l];
    d.chunks = LOUT[l] / mlptt::kslab_kc(LOUT[l]);
    d.N = H;
    d.zin = m->z[l - 1];
    d.outf = m->dzf;
    d.oa = m->dza[nxt];
    d.ot = m->dzt;
    d.oaR = M;
    d.otK = M;
    d.err = m->d_err;
    if ((e = tg_launch<128, mlptt::TG_BWD_GELU>(d, M / 128, H / 128, 1, m->s)) != cudaSuccess) return e;
    gA = m->dza[nxt];
    nxt ^= 1;
  }
  return cudaGetLastError();
}

// Adam on one parameter array; for weights (lin x lout, wt != nullptr) it
// also writes the BF16 copies the GEMMs read (row-major, W^T and W K-slabs).
__global__ void k_adam(float* w, const float* gw, float* mw, float* vw, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2, int lout, int lin, __nv_bfloat16* wb, uint8_t* wt, uint8_t* wn) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gr = gw[i];
  const float m = b1 * mw[i] + (1.f - b1) * gr;
  const float v = b2 * vw[i] + (1.f - b2) * gr * gr;
  mw[i] = m;
  vw[i] = v;
  const float wv = w[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
  w[i] = wv;
  if (wt) {
    const int r = i / lout, c = i % lout;
    const __nv_bfloat16 b = __float2bfloat16(wv);
    wb[i] = b;
    *reinterpret_cast<__nv_bfloat16*>(wt + mlptt::kslab_off(c, r, lout, lin)) = b;
    *reinterpret_cast<__nv_bfloat16*>(wn + mlptt::kslab_off(r, c, lin, lout)) = b;
  }
}

// The BF16 copies of every weight array after W changed outside Adam.
cudaError_t mlp_weight_copies(izem_mlp* m) {
  for (int l = 0; l < NL; ++l) {
    const int nw = LIN[l] * LOUT[l];
    mlptt::k_tg_weights<<<(nw + 255) / 256, 256, 0, m->s>>>(m->W[l], LIN[l], LOUT[l], m->Wb[l], m->wt[l], m->wn[l]);
  }
  m->blob_dirty = true;
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
  for (int l = 0; l < NL && ok; ++l)
    ok = cudaMalloc(&m->blob[l], (size_t)LIN[l] * LOUT[l] * 2) == cudaSuccess &&
         cudaMalloc(&m->wt[l], (size_t)LIN[l] * LOUT[l] * 2) == cudaSuccess &&
         cudaMalloc(&m->wn[l], (size_t)LIN[l] * LOUT[l] * 2) == cudaSuccess;
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
    cudaFree(m->mb[l]); cudaFree(m->vb[l]); cudaFree(m->gW[l]); cudaFree(m->gb[l]);
    cudaFree(m->wt[l]); cudaFree(m->wn[l]);
  }
  for (int l = 0; l < NL - 1; ++l) { cudaFree(m->acta[l]); cudaFree(m->actt[l]); cudaFree(m->z[l]); }
  cudaFree(m->xa); cudaFree(m->xt); cudaFree(m->out); cudaFree(m->gout); cudaFree(m->goa); cudaFree(m->got);
  cudaFree(m->dzf); cudaFree(m->dza[0]); cudaFree(m->dza[1]); cudaFree(m->dzt); cudaFree(m->part);
  cudaFree(m->d_loss);
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
  }
  if (mlp_weight_copies(m) != cudaSuccess) return IZEM_ERR_CUDA;
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

int izem_mlp_set_residual(izem_mlp* m, int residual) {
  if (!m) return IZEM_ERR_ARG;
  m->residual = residual != 0;
  return IZEM_OK;
}

int izem_gpu_reactor_rhs(const izem_mech* mech, int n, const double* T, const double* rho, const double* Y,
                         double* zdot, int device_ptrs) {
  if (!mech || n <= 0 || !T || !rho || !Y || !zdot || !chem_mech_valid(mech)) return IZEM_ERR_ARG;
  (void)cudaGetLastError();
  if (chem_upload_mech(mech) != cudaSuccess) return IZEM_ERR_CUDA;
  if (device_ptrs) {
    if (chem_launch_rhs(n, T, rho, Y, zdot, 0) != cudaSuccess) return IZEM_ERR_CUDA;
    return cudaStreamSynchronize(0) == cudaSuccess ? IZEM_OK : IZEM_ERR_CUDA;
  }
  const size_t n8 = (size_t)n * 8;
  double *dT = nullptr, *dr = nullptr, *dY = nullptr, *dz = nullptr;
  int rc = IZEM_OK;
  if (cudaMalloc(&dT, n8) || cudaMalloc(&dr, n8) || cudaMalloc(&dY, 9 * n8) || cudaMalloc(&dz, 10 * n8)) {
    rc = IZEM_ERR_NOMEM;
  } else if (cudaMemcpy(dT, T, n8, cudaMemcpyHostToDevice) || cudaMemcpy(dr, rho, n8, cudaMemcpyHostToDevice) ||
             cudaMemcpy(dY, Y, 9 * n8, cudaMemcpyHostToDevice) || chem_launch_rhs(n, dT, dr, dY, dz, 0) ||
             cudaMemcpy(zdot, dz, 10 * n8, cudaMemcpyDeviceToHost)) {
    rc = IZEM_ERR_CUDA;
  }
  cudaFree(dT); cudaFree(dr); cudaFree(dY); cudaFree(dz);
  return rc;
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
  if (!m || M <= 0 || !x || !t || !loss || !gW || !gb) return IZEM_ERR_ARG;
  if (mlp_ensure(m, M) != cudaSuccess) return IZEM_ERR_NOMEM;
  const int Mp = (M + 127) / 128 * 128;
  float *dx = nullptr, *dt = nullptr;
  if (cudaMalloc(&dx, (size_t)M * IN * 4) != cudaSuccess) return IZEM_ERR_NOMEM;
  if (cudaMalloc(&dt, (size_t)M * OUT * 4) != cudaSuccess) {
    cudaFree(dx);
    return IZEM_ERR_NOMEM;
  }
  int rc = IZEM_OK;
  if (cudaMemcpy(dx, x, (size_t)M * IN * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dt, t, (size_t)M * OUT * 4, cudaMemcpyHostToDevice) != cudaSuccess)
    rc = IZEM_ERR_CUDA;
  if (rc == IZEM_OK) {
    mlptt::k_tg_pack_input<<<(Mp * 16 + 255) / 256, 256, 0, m->s>>>(dx, Mp, M, m->xa, m->xt);
    if (cudaGetLastError() != cudaSuccess || mlp_forward(m, Mp) != cudaSuccess) rc = IZEM_ERR_CUDA;
  }
  if (rc == IZEM_OK) {
    cudaMemsetAsync(m->d_loss, 0, sizeof(double), m->s);
    mlptt::k_tg_mse<<<(Mp * 16 + 255) / 256, 256, 0, m->s>>>(m->out, dt, Mp, M, m->gout, m->goa, m->got, m->d_loss);
    if (cudaGetLastError() != cudaSuccess || mlp_backward(m, Mp) != cudaSuccess) rc = IZEM_ERR_CUDA;
  }
  if (rc == IZEM_OK) {
    if (cudaMemcpyAsync(loss, m->d_loss, sizeof(double), cudaMemcpyDeviceToHost, m->s) != cudaSuccess) rc = IZEM_ERR_CUDA;
    for (int l = 0; l < NL && rc == IZEM_OK; ++l)
      if (cudaMemcpyAsync(gW[l], m->gW[l], (size_t)LIN[l] * LOUT[l] * 4, cudaMemcpyDeviceToHost, m->s) != cudaSuccess ||
          cudaMemcpyAsync(gb[l], m->gb[l], LOUT[l] * 4, cudaMemcpyDeviceToHost, m->s) != cudaSuccess)
        rc = IZEM_ERR_CUDA;
  }
  if (cudaStreamSynchronize(m->s) != cudaSuccess) rc = IZEM_ERR_CUDA;
  if (rc == IZEM_OK) rc = mlp_tc_status(m);
  if (rc == IZEM_OK) *loss = *loss / ((double)M * OUT);
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
  const int Mp = (batch + 127) / 128 * 128;
  float *dx = nullptr, *dt = nullptr;
  int rc = IZEM_OK;
  if (device_ptrs) {
    dx = const_cast<float*>(x);
    dt = const_cast<float*>(t);
  } else {
    if (cudaMalloc(&dx, (size_t)n * IN * 4) != cudaSuccess) return IZEM_ERR_NOMEM;
    if (cudaMalloc(&dt, (size_t)n * OUT * 4) != cudaSuccess) {
      cudaFree(dx);
      return IZEM_ERR_NOMEM;
    }
    if (cudaMemcpy(dx, x, (size_t)n * IN * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dt, t, (size_t)n * OUT * 4, cudaMemcpyHostToDevice) != cudaSuccess)
      rc = IZEM_ERR_CUDA;
  }
  const long long nb = n / batch;
  std::vector<long long> perm(nb);
  unsigned long long st = seed ? seed : 1ULL;
  for (int ep = 0; ep < epochs && rc == IZEM_OK; ++ep) {
    for (long long q = 0; q < nb; ++q) perm[q] = q;
    for (long long q = nb - 1; q > 0; --q) {   // Fisher-Yates on batch indices (xorshift)
      st ^= st << 13; st ^= st >> 7; st ^= st << 17;
      long long r = (long long)(st % (unsigned long long)(q + 1));
      long long tmp = perm[q]; perm[q] = perm[r]; perm[r] = tmp;
    }
    cudaMemsetAsync(m->d_loss, 0, sizeof(double), m->s);
    for (long long q = 0; q < nb; ++q) {
      const long long r0 = perm[q] * batch;
      mlptt::k_tg_pack_input<<<(Mp * 16 + 255) / 256, 256, 0, m->s>>>(dx + r0 * IN, Mp, batch, m->xa, m->xt);
      if (mlp_forward(m, Mp) != cudaSuccess) { rc = IZEM_ERR_CUDA; break; }
      mlptt::k_tg_mse<<<(Mp * 16 + 255) / 256, 256, 0, m->s>>>(m->out, dt + r0 * OUT, Mp, batch, m->gout, m->goa,
                                                                 m->got, m->d_loss);
      if (mlp_backward(m, Mp) != cudaSuccess) { rc = IZEM_ERR_CUDA; break; }
      m->step += 1;
      const float b1 = 0.9f, b2 = 0.999f;
      const float c1 = 1.f - powf(b1, (float)m->step), c2 = 1.f - powf(b2, (float)m->step);
      for (int l = 0; l < NL; ++l) {
        const int nw = LIN[l] * LOUT[l];
        k_adam<<<(nw + 255) / 256, 256, 0, m->s>>>(m->W[l], m->gW[l], m->mW[l], m->vW[l], nw, lr, b1, b2, 1e-8f, c1, c2,
                                                   LOUT[l], LIN[l], m->Wb[l], m->wt[l], m->wn[l]);
        k_adam<<<(LOUT[l] + 255) / 256, 256, 0, m->s>>>(m->b[l], m->gb[l], m->mb[l], m->vb[l], LOUT[l], lr, b1, b2,
                                                        1e-8f, c1, c2, 0, 0, nullptr, nullptr, nullptr);
      }
      m->blob_dirty = true;
    }
    if (rc != IZEM_OK) break;
    double lsum = 0.0;
    cudaMemcpyAsync(&lsum, m->d_loss, sizeof(double), cudaMemcpyDeviceToHost, m->s);
    if (cudaStreamSynchronize(m->s) != cudaSuccess) { rc = IZEM_ERR_CUDA; break; }
    if (mlp_tc_status(m) != IZEM_OK) { rc = IZEM_ERR_TIMEOUT; break; }
    if (losses) losses[ep] = lsum / ((double)nb * batch * OUT);
  }
  if (cudaStreamSynchronize(m->s) != cudaSuccess && rc == IZEM_OK) rc = IZEM_ERR_CUDA;
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
  if (!m || !mech || n <= 0 || !T || !rho || !Y || !dt || !gate10 || !kncf || !chem_mech_valid(mech))
    return IZEM_ERR_ARG;
  if (nele <= 0 || nele > 8) return IZEM_ERR_ARG;
  if (m2 && m2->residual != m->residual) return IZEM_ERR_ARG;   // one target form per ensemble
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
                            m->g_count, ddTp ? ddTp + c0 : nullptr, m->g_stats, m->residual, s);
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
constexpr size_t NA_IN_BYTES = (size_t)NA_ROWS * INP * sizeof(__nv_bfloat16);   // BF16 input rows
constexpr size_t NA_OUT_BYTES = (size_t)NA_ROWS * OUTP * sizeof(float);         // FP32 output rows
constexpr size_t NA_BYTES = NA_IN_BYTES + NA_OUT_BYTES;                          // 384 KiB

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
  __nv_bfloat16* in = reinterpret_cast<__nv_bfloat16*>(base);
  float* out = reinterpret_cast<float*>(base + NA_IN_BYTES);
  k_na_pack<<<g1((long long)M * INP), 256, 0, s>>>(d_x, M, in);
  if (cudaGetLastError() != cudaSuccess) return IZEM_ERR_CUDA;
  // the tensor-core inference kernel of izem_mlp_forward; its weight
  // operands and timeout flag live in the handle (allocated at creation)
  if (mlp_infer_tc(m, M, in, out, s) != cudaSuccess) return IZEM_ERR_CUDA;
  k_na_unpack<<<g1((long long)M * OUT), 256, 0, s>>>(out, M, d_y);
  return cudaGetLastError() == cudaSuccess ? IZEM_OK : IZEM_ERR_CUDA;
}

// ------------------------------------------------- bounded-wait self-test --
// The tensor-core kernels poll their mbarriers a bounded number of times and
// give up with an error flag instead of waiting forever.  This kernel waits,
// in the same way, on a barrier that nothing arrives on: one thread
// initialises it for one arrival, polls its first phase `polls` times and
// records whether it gave up.
namespace {
__global__ void k_wait_selftest(int polls, int* gave_up) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  const uint32_t b = mlptc::saddr(&bar);
  mlptc::mbar_init(b, 1);
  mlptc::fence_async_smem();
  int done = 0;
  for (int i = 0; i < polls && !done; ++i) {
    uint32_t d;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(d)
        : "r"(b), "r"(0u)
        : "memory");
    done = (int)d;
  }
  *gave_up = done ? 0 : 1;
}
}  // namespace

extern "C" int izem_gpu_wait_selftest(int polls, int* gave_up) {
  if (polls < 1 || polls > (1 << 20) || !gave_up) return IZEM_ERR_ARG;
  int* d = nullptr;
  if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) return IZEM_ERR_NOMEM;
  int rc = IZEM_OK;
  k_wait_selftest<<<1, 32>>>(polls, d);
  if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
      cudaMemcpy(gave_up, d, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = IZEM_ERR_CUDA;
  cudaFree(d);
  return rc;
}

