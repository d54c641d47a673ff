// Library stand-in for the reference's GPU build (benchmark comparator only).
//
// The reference's chain cannot be compiled here: its correlator (TCC) and
// beamformer (ccglib) are empty submodules.  This file strings together the
// libraries it calls, or their closest stock equivalents, in the reference's
// order, so bench.py can time a "vendor-library GPU chain" on the same GB300:
//   ingest       int8 x int16 scale -> complex fp32 [c][t][pol][r]   (spatial.cuh:423-486,
//                                                                      aligned window)
//   correlate    cuBLAS batched complex GEMM V = X X^H, TF32 tensor cores, fp32 out
//                (in place of TCC, lambda_gpu_pipeline.hpp:649-651)
//   whiten       D^-1/2 V_pp D^-1/2 per (channel, pol)                (spatial.cuh:1068-1093)
//   eigensolve   cusolverDnXsyevBatched, complex fp32, vectors        (lambda_adaptive_..._pipeline.hpp:679-686)
//   projector    P = I - U_K U_K^H from the un-whitened top K         (spatial.cuh:993-1034)
//   W P          cuBLAS batched complex GEMM                          (ccglib, ..._pipeline.hpp:773-794)
//   beamform     cuBLAS batched complex GEMM Y = W_eff X_p, TF32      (ccglib, lambda_gpu_pipeline.hpp:292-299)
//   half output  fp32 -> fp16 [C][Pol][2B][T][2]                      (spatial.cuh:376-418)
// It is not the reference and is never used by the library: only bench.py
// loads it, to report a clearly labelled comparator.
#include <cublas_v2.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <cstdint>
#include <cstdio>
#include <cstring>

namespace {

thread_local char g_err[256] = "";

int fail(const char *what, int code) {
  snprintf(g_err, sizeof(g_err), "%s failed (%d)", what, code);
  return 1;
}

#define CK(call)                                              \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return fail(#call, (int)e_);       \
  } while (0)
#define CB(call)                                              \
  do {                                                        \
    cublasStatus_t e_ = (call);                               \
    if (e_ != CUBLAS_STATUS_SUCCESS) return fail(#call, (int)e_); \
  } while (0)
#define CS(call)                                              \
  do {                                                        \
    cusolverStatus_t e_ = (call);                             \
    if (e_ != CUSOLVER_STATUS_SUCCESS) return fail(#call, (int)e_); \
  } while (0)

// X[c][t][p][r] = samples(window offset Tp) * scale
__global__ void ingest_kernel(const int8_t *samples, const int16_t *scales, float2 *X, int C, int F, int Tp,
                              int Rpp, int P) {
  const int R = F * Rpp, T = P * Tp;
  const size_t total = (size_t)C * T * 2 * R;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i % R);
    const int p = (int)((i / R) & 1);
    const size_t ct = i / (2 * (size_t)R);
    const int t = (int)(ct % T);
    const int c = (int)(ct / T);
    const int q = t + Tp;  // aligned window, no delay
    const int pk = q / Tp, tt = q - pk * Tp;
    const int f = r / Rpp, n = r - f * Rpp;
    const size_t off = (((((size_t)c * (P + 2) + pk) * F + f) * Tp + tt) * Rpp + n) * 4 + 2 * p;
    const int s = scales[(((size_t)c * (P + 2) + pk) * R + r) * 2 + p];
    X[i] = make_float2((float)(samples[off] * s), (float)(samples[off + 1] * s));
  }
}

// A[c][p] (R x R column-major) = d_i conj(d_j) V[c](pR+i, pR+j) / (s_i s_j); s[c][p][i]
__global__ void whiten_kernel(const float2 *V, const float2 *d, float2 *A, float *s, int C, int R) {
  const int cp = blockIdx.x, c = cp >> 1, p = cp & 1;
  const int R2 = 2 * R;
  const float2 *Vc = V + (size_t)c * R2 * R2;
  const float2 *dp = d + (size_t)cp * R;
  __shared__ float ss[256];
  for (int i = threadIdx.x; i < R; i += blockDim.x) {
    const float2 v = Vc[(size_t)(p * R + i) * R2 + p * R + i];
    const float2 di = dp[i];
    ss[i] = sqrtf(fmaxf(v.x * (di.x * di.x + di.y * di.y), 1e-10f));
    s[(size_t)cp * R + i] = ss[i];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
    const int i = e % R, j = e / R;  // row i, column j
    const float2 v = Vc[(size_t)(p * R + j) * R2 + p * R + i];
    const float2 di = dp[i], dj = dp[j];
    // d_i v conj(d_j)
    const float2 t = make_float2(di.x * v.x - di.y * v.y, di.x * v.y + di.y * v.x);
    const float2 u = make_float2(t.x * dj.x + t.y * dj.y, t.y * dj.x - t.x * dj.y);
    const float inv = 1.0f / (ss[i] * ss[j]);
    A[(size_t)cp * R * R + e] = make_float2(u.x * inv, u.y * inv);
  }
}

// P[c][p] = I - sum_k u_k u_k^H, u_k = normalise(s o v_{R-1-k}); W[c][p] (B x R col-major) from fp16
__global__ void projector_kernel(const float2 *A, const float *s, const __half2 *w16, float2 *Pm, float2 *W, int R,
                                 int B, int K) {
  const int cp = blockIdx.x;
  __shared__ float2 u[4][256];
  __shared__ float nrm[4];
  const float2 *V = A + (size_t)cp * R * R;  // eigenvectors in columns, ascending
  for (int k = 0; k < K; ++k)
    for (int i = threadIdx.x; i < R; i += blockDim.x) {
      const float2 v = V[(size_t)(R - 1 - k) * R + i];
      const float si = s[(size_t)cp * R + i];
      u[k][i] = make_float2(v.x * si, v.y * si);
    }
  __syncthreads();
  if (threadIdx.x < K) {
    float a = 0.f;
    for (int i = 0; i < R; ++i) a += u[threadIdx.x][i].x * u[threadIdx.x][i].x + u[threadIdx.x][i].y * u[threadIdx.x][i].y;
    nrm[threadIdx.x] = a > 0.f ? rsqrtf(a) : 0.f;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
    const int i = e % R, j = e / R;
    float2 acc = make_float2(i == j ? 1.f : 0.f, 0.f);
    for (int k = 0; k < K; ++k) {
      const float2 a = u[k][i], b = u[k][j];
      const float q = nrm[k] * nrm[k];
      acc.x -= q * (a.x * b.x + a.y * b.y);
      acc.y -= q * (a.y * b.x - a.x * b.y);
    }
    Pm[(size_t)cp * R * R + e] = acc;
  }
  // W (B x R, column-major: element (b, r) at b + r B) from [c][p][b][r] fp16
  for (int e = threadIdx.x; e < B * R; e += blockDim.x) {
    const int b = e / R, r = e % R;
    W[(size_t)cp * B * R + b + (size_t)r * B] = __half22float2(w16[(size_t)cp * B * R + e]);
  }
}

// W_eff[c][p] (2B x R col-major): rows b = W diag(d), rows B + b = (W P) diag(d)
__global__ void weff_kernel(const float2 *W, const float2 *WP, const float2 *d, float2 *Weff, int R, int B) {
  const int cp = blockIdx.x;
  for (int e = threadIdx.x; e < B * R; e += blockDim.x) {
    const int b = e % B, r = e / B;
    const float2 dr = d[(size_t)cp * R + r];
    const float2 w = W[(size_t)cp * B * R + e], wp = WP[(size_t)cp * B * R + e];
    float2 *o = Weff + (size_t)cp * 2 * B * R + (size_t)r * 2 * B;
    o[b] = make_float2(w.x * dr.x - w.y * dr.y, w.x * dr.y + w.y * dr.x);
    o[B + b] = make_float2(wp.x * dr.x - wp.y * dr.y, wp.x * dr.y + wp.y * dr.x);
  }
}

// Y[c][p] (2B x T col-major) -> fp16 [c][p][2B][T][2]
__global__ void half_output_kernel(const float2 *Y, __half2 *out, int C, int NB, int T) {
  const size_t total = (size_t)C * 2 * NB * T;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int t = (int)(i % T);
    const size_t cpb = i / T;
    const int b = (int)(cpb % NB);
    const size_t cp = cpb / NB;
    out[i] = __float22half2_rn(Y[(cp * T + t) * NB + b]);
  }
}

}  // namespace

struct sfs_ctx {
  int C, F, Tp, R, Rpp, P, B, T;
  cublasHandle_t blas;
  cusolverDnHandle_t solver;
  cusolverDnParams_t params;
  float2 *X, *V, *A, *Pm, *W, *WP, *Weff, *Y, *d;
  float *s, *evals;
  const __half2 *w16;
  int *info;
  void *dwork, *hwork;
  size_t dwork_bytes, hwork_bytes;
};

extern "C" {

const char *sfs_last_error(void) { return g_err; }

int sfs_create(int C, int F, int Tp, int R, int Rpp, int P, int B, sfs_ctx **out) {
  sfs_ctx *x = new sfs_ctx();
  memset(x, 0, sizeof(*x));
  x->C = C; x->F = F; x->Tp = Tp; x->R = R; x->Rpp = Rpp; x->P = P; x->B = B; x->T = P * Tp;
  const size_t T = x->T;
  CB(cublasCreate(&x->blas));
  CS(cusolverDnCreate(&x->solver));
  CS(cusolverDnCreateParams(&x->params));
  CK(cudaMalloc(&x->X, sizeof(float2) * C * T * 2 * R));
  CK(cudaMalloc(&x->V, sizeof(float2) * C * 4 * R * R));
  CK(cudaMalloc(&x->A, sizeof(float2) * C * 2 * R * R));
  CK(cudaMalloc(&x->Pm, sizeof(float2) * C * 2 * R * R));
  CK(cudaMalloc(&x->W, sizeof(float2) * C * 2 * B * R));
  CK(cudaMalloc(&x->WP, sizeof(float2) * C * 2 * B * R));
  CK(cudaMalloc(&x->Weff, sizeof(float2) * C * 2 * 2 * B * R));
  CK(cudaMalloc(&x->Y, sizeof(float2) * C * 2 * 2 * B * T));
  CK(cudaMalloc(&x->d, sizeof(float2) * C * 2 * R));
  CK(cudaMalloc(&x->s, sizeof(float) * C * 2 * R));
  CK(cudaMalloc(&x->evals, sizeof(float) * C * 2 * R));
  CK(cudaMalloc(&x->info, sizeof(int) * C * 2));
  CS(cusolverDnXsyevBatched_bufferSize(x->solver, x->params, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, R,
                                       CUDA_C_32F, x->A, R, CUDA_R_32F, x->evals, CUDA_C_32F, &x->dwork_bytes,
                                       &x->hwork_bytes, 2 * C));
  CK(cudaMalloc(&x->dwork, x->dwork_bytes ? x->dwork_bytes : 16));
  x->hwork = x->hwork_bytes ? malloc(x->hwork_bytes) : nullptr;
  *out = x;
  return 0;
}

// d_weights_f16: [C][2][B][R] half2 (device); d_factors: [C][2][R] float2 (device) or NULL for 1.
int sfs_set_inputs(sfs_ctx *x, const void *d_weights_f16, const void *d_factors) {
  x->w16 = static_cast<const __half2 *>(d_weights_f16);
  if (d_factors) {
    CK(cudaMemcpy(x->d, d_factors, sizeof(float2) * x->C * 2 * x->R, cudaMemcpyDeviceToDevice));
  } else {
    float2 *h = static_cast<float2 *>(malloc(sizeof(float2) * x->C * 2 * x->R));
    for (int i = 0; i < x->C * 2 * x->R; ++i) h[i] = make_float2(1.f, 0.f);
    CK(cudaMemcpy(x->d, h, sizeof(float2) * x->C * 2 * x->R, cudaMemcpyHostToDevice));
    free(h);
  }
  return 0;
}

// The eigensolve alone, on the whitened matrices the last sfs_run_chain built (re-whitened first,
// since cuSOLVER overwrites them with the eigenvectors).
int sfs_run_eig(sfs_ctx *x, void *stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CS(cusolverDnSetStream(x->solver, st));
  whiten_kernel<<<2 * x->C, 256, 0, st>>>(x->V, x->d, x->A, x->s, x->C, x->R);
  CK(cudaGetLastError());
  CS(cusolverDnXsyevBatched(x->solver, x->params, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, x->R, CUDA_C_32F,
                            x->A, x->R, CUDA_R_32F, x->evals, CUDA_C_32F, x->dwork, x->dwork_bytes, x->hwork,
                            x->hwork_bytes, x->info, 2 * x->C));
  return 0;
}

int sfs_run_chain(sfs_ctx *x, const int8_t *d_samples, const int16_t *d_scales, int K, void *d_beams_f16,
                  void *stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int C = x->C, R = x->R, B = x->B, T = x->T, R2 = 2 * R, NB = 2 * B;
  CB(cublasSetStream(x->blas, st));
  ingest_kernel<<<4 * 152, 256, 0, st>>>(d_samples, d_scales, x->X, C, x->F, x->Tp, x->Rpp, x->P);
  CK(cudaGetLastError());
  const float2 one = make_float2(1.f, 0.f), zero = make_float2(0.f, 0.f);
  // V[c] = X[c] X[c]^H, X[c] = (2R x T) column-major
  CB(cublasGemmStridedBatchedEx(x->blas, CUBLAS_OP_N, CUBLAS_OP_C, R2, R2, T, &one, x->X, CUDA_C_32F, R2,
                                (long long)R2 * T, x->X, CUDA_C_32F, R2, (long long)R2 * T, &zero, x->V, CUDA_C_32F,
                                R2, (long long)R2 * R2, C, CUBLAS_COMPUTE_32F_FAST_TF32, CUBLAS_GEMM_DEFAULT));
  if (sfs_run_eig(x, stream)) return 1;
  projector_kernel<<<2 * C, 256, 0, st>>>(x->A, x->s, x->w16, x->Pm, x->W, R, B, K);
  CK(cudaGetLastError());
  // W P: (B x R) (R x R) per (c, p)
  CB(cublasGemmStridedBatchedEx(x->blas, CUBLAS_OP_N, CUBLAS_OP_N, B, R, R, &one, x->W, CUDA_C_32F, B,
                                (long long)B * R, x->Pm, CUDA_C_32F, R, (long long)R * R, &zero, x->WP, CUDA_C_32F,
                                B, (long long)B * R, 2 * C, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT));
  weff_kernel<<<2 * C, 256, 0, st>>>(x->W, x->WP, x->d, x->Weff, R, B);
  CK(cudaGetLastError());
  // Y[c][p] (2B x T) = W_eff[c][p] (2B x R) X_p (R x T, rows p R.. of X[c])
  for (int p = 0; p < 2; ++p)
    CB(cublasGemmStridedBatchedEx(x->blas, CUBLAS_OP_N, CUBLAS_OP_N, NB, T, R, &one, x->Weff + (size_t)p * NB * R,
                                  CUDA_C_32F, NB, (long long)2 * NB * R, x->X + (size_t)p * R, CUDA_C_32F, R2,
                                  (long long)R2 * T, &zero, x->Y + (size_t)p * NB * T, CUDA_C_32F, NB,
                                  (long long)2 * NB * T, C, CUBLAS_COMPUTE_32F_FAST_TF32, CUBLAS_GEMM_DEFAULT));
  half_output_kernel<<<4 * 152, 256, 0, st>>>(x->Y, static_cast<__half2 *>(d_beams_f16), C, NB, T);
  CK(cudaGetLastError());
  return 0;
}

int sfs_destroy(sfs_ctx *x) {
  if (!x) return 0;
  cudaFree(x->X); cudaFree(x->V); cudaFree(x->A); cudaFree(x->Pm); cudaFree(x->W); cudaFree(x->WP);
  cudaFree(x->Weff); cudaFree(x->Y); cudaFree(x->d); cudaFree(x->s); cudaFree(x->evals); cudaFree(x->info);
  cudaFree(x->dwork);
  free(x->hwork);
  cusolverDnDestroyParams(x->params);
  cusolverDnDestroy(x->solver);
  cublasDestroy(x->blas);
  delete x;
  return 0;
}

}  // extern "C"
