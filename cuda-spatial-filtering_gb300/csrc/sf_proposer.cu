// Learned subspace proposer around the adaptive chain: features, the
// proposer object (weights, Adam state, activations), its training step and
// inference through the BF16 tensor-core GEMM of sf_mlp.cu, and the
// warm-started Rayleigh-Ritz refinement with the residual-gated fallback to
// the full eigensolver.
//
// Learned chain per integration (sf_run_adaptive_learned):
//   correlate -> features (whitened covariance / trace, packed upper triangle,
//   bf16) -> MLP -> four complex start vectors per (channel, pol) ->
//   n_iter subspace iterations U <- orth(A U) -> Rayleigh-Ritz on U^H A U
//   (4 x 4 complex Jacobi) -> residuals ||A u_k - theta_k u_k|| -> K (fixed or
//   theta > delta x noise floor, the floor = (tr A - sum theta) / (n - 4)) ->
//   accepted: I - U_K U_K^H on the weights as the full solver does;
//   rejected (a residual above tol x theta_0, K > 4, or the percentile rule,
//   which needs every eigenvalue): the matrix joins a device-side list that
//   the full top-K eigensolver then walks -> beams.
// No counterpart in the reference: its adaptive pipeline always runs the full
// eigensolve (lambda_adaptive_beamformed_spectra_pipeline.hpp:679-686), which
// is this chain's fallback.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>

#include "sf_common.cuh"
#include "sf_plan.cuh"

int sf_internal_set_error(int code, const char *msg);
cudaError_t sf_launch_gemm_bf16(int M, int N, int K, const void *A, int lda, int a_mn, const void *B, int ldb, int b_mn,
                                int mode, const float *bias, const void *mask, int ldm, void *out, int ldo, int splits,
                                uint32_t *status, cudaStream_t stream);
cudaError_t sf_launch_proposer_targets(const int32_t *vis, const float *evals, const float *evecs, int C, int R,
                                       float *targets, float *tw, cudaStream_t stream);
cudaError_t sf_launch_proposer_loss(const float *y, const float *t, const float *tw, int rows, int width, int R,
                                    void *dy, int lddy, float *loss, cudaStream_t stream);
cudaError_t sf_launch_column_sums(const void *dy, int rows, int cols, int ld, float *db, cudaStream_t stream);
cudaError_t sf_launch_adam(float *w, float *g, float *m, float *v, void *w16, int n, float lr, int step,
                           cudaStream_t stream);

namespace {

constexpr int KV = 4;        // proposed vectors per matrix
constexpr int RR_MAX_N = 64;
constexpr int RR_NPL = 2;    // rows per lane (n <= 64)
constexpr int W_B_MAX_RR = 16;  // beams per pol

int fail(int code, const char *fmt, ...) {
  char buf[320];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return sf_internal_set_error(code, buf);
}

int cuda_fail(cudaError_t e, const char *what) { return fail(SF_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e)); }

#define PR_TRY(call, what)                        \
  do {                                            \
    cudaError_t e_ = (call);                      \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

__device__ __forceinline__ float wsum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Features of matrix row = 2 c + p: the whitened covariance (no receiver
// factors) divided by its trace n, packed upper triangle i <= j in baseline
// order, (re, im) per entry, zero-padded to ld.
__global__ void sf_proposer_features_kernel(const int32_t *vis, int R, int NBL, __nv_bfloat16 *x, int ldx) {
  const int row = blockIdx.x, c = row >> 1, p = row & 1;
  __shared__ float s[RR_MAX_N * 2];
  const int32_t *vb = vis + (size_t)c * NBL * 8;
  for (int i = threadIdx.x; i < R; i += blockDim.x)
    s[i] = rsqrtf(fmaxf(static_cast<float>(vb[((size_t)baseline_of(i, i) * 2 + p) * 4 + p * 2]), 1e-10f));
  __syncthreads();
  const float inv_n = 1.0f / static_cast<float>(R);
  __nv_bfloat16 *xr = x + (size_t)row * ldx;
  for (int b = threadIdx.x; b < NBL; b += blockDim.x) {
    int j = static_cast<int>((sqrtf(8.0f * b + 1.0f) - 1.0f) * 0.5f);
    while (j * (j + 1) / 2 > b) --j;
    while ((j + 1) * (j + 2) / 2 <= b) ++j;
    const int i = b - j * (j + 1) / 2;
    const int32_t *v = vb + ((size_t)b * 2 + p) * 4 + p * 2;
    const float sc = s[i] * s[j] * inv_n;
    xr[2 * b] = __float2bfloat16_rn(static_cast<float>(v[0]) * sc);
    xr[2 * b + 1] = __float2bfloat16_rn(static_cast<float>(v[1]) * sc);
  }
  for (int k = 2 * NBL + threadIdx.x; k < ldx; k += blockDim.x) xr[k] = __float2bfloat16_rn(0.0f);
}

// bytes of one warp's region: A n x (n + 1), U and V 4 n, W0 B n, factors n (float2), s and 1 / s n (float)
__host__ __device__ inline size_t rr_region(int n, int B) {
  const size_t per = ((size_t)n * (n + 1) + 2 * (size_t)KV * n + (size_t)B * n + (size_t)n) * 8 + 2 * (size_t)n * 4;
  return (per + 15) & ~size_t(15);
}

struct RRArgs {
  const int32_t *vis;
  const float2 *factors;
  const __half2 *weights;
  const int32_t *fixed_counts;
  const float *y;  // MLP output [rows][ldy]: vector k of row at y + k 2R, (re, im) per component
  int ldy;
  float2 *weff;
  int32_t *counts;
  float *ritz;        // [rows][4] Ritz values (may be NULL)
  int32_t *fb_list, *fb_count;
  int C, R, B, NBL, rows;
  int k_rule;
  float delta;
  int n_iter;
  float tol;
};

// One warp per (channel, pol) matrix; `wpc` matrices per CTA.  Every group of
// independent sums shares one shuffle butterfly (the kernel is bound by the
// latency of its dependent steps, not by arithmetic).
__global__ void __launch_bounds__(128) sf_rr_kernel(const RRArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = blockIdx.x * (blockDim.x >> 5) + warp;
  if (row >= a.rows) return;
  const int n = a.R, ld = n + 1, B = a.B;
  const int c = row >> 1, p = row & 1;
  uint8_t *base = smem + warp * rr_region(n, B);
  float2 *A = reinterpret_cast<float2 *>(base);
  float2 *U = A + n * ld;
  float2 *V = U + KV * n;
  float2 *W0 = V + KV * n;
  float2 *fac = W0 + B * n;
  float *s = reinterpret_cast<float *>(fac + n);
  float *rsd = s + n;  // 1 / s
  // same-pol entry (p, p) of baseline b at vin[8 b], vin[8 b + 1] (layout [b][Pol][Pol][2])
  const int32_t *vin = a.vis + (size_t)c * a.NBL * 8 + 6 * p;
  const float2 *dp = a.factors + (size_t)row * n;
  const bool r0 = lane < n, r1 = lane + 32 < n;  // this lane's rows lane, lane + 32

  // whitened covariance with the receiver factors, both triangles
  for (int i = lane; i < n; i += 32) {
    const float2 d = dp[i];
    fac[i] = d;
    const float sq = fmaxf(static_cast<float>(vin[(size_t)baseline_of(i, i) * 8]) * (d.x * d.x + d.y * d.y), 1e-10f);
    s[i] = sqrtf(sq);
    rsd[i] = rsqrtf(sq);
  }
  __syncwarp();
  {
    const int nb = n * (n + 1) / 2;
    for (int b0 = 0; b0 < nb; b0 += 8 * 32) {
      int2 raw[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int b = b0 + u * 32 + lane;
        raw[u] = b < nb ? *reinterpret_cast<const int2 *>(vin + (size_t)b * 8) : make_int2(0, 0);
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int b = b0 + u * 32 + lane;
        if (b < nb) {
          // b = j (j + 1) / 2 + i: j from an approximate square root, then corrected exactly
          const float t8 = 8.0f * static_cast<float>(b) + 1.0f;
          int j = static_cast<int>((t8 * rsqrtf(t8) - 1.0f) * 0.5f);
          if ((j + 1) * (j + 2) / 2 <= b) ++j;
          if (j * (j + 1) / 2 > b) --j;
          const int i = b - j * (j + 1) / 2;
          float2 x = make_float2(static_cast<float>(raw[u].x), static_cast<float>(raw[u].y));
          x = cmulc(cmul(fac[i], x), fac[j]);  // d_i V(i, j) conj(d_j), element (i, j)
          const float inv = rsd[i] * rsd[j];
          A[i * ld + j] = i == j ? make_float2(x.x * inv, 0.0f) : make_float2(x.x * inv, x.y * inv);
          if (j > i) A[j * ld + i] = make_float2(x.x * inv, -x.y * inv);
        }
      }
    }
  }
  // start vectors: the MLP's (for the factor-free covariance) turned by the factors' phases
  {
    const float2 *yr = reinterpret_cast<const float2 *>(a.y + (size_t)row * a.ldy);  // ldy even
    float2 yv[KV][RR_NPL];
#pragma unroll
    for (int k = 0; k < KV; ++k)
#pragma unroll
      for (int t = 0; t < RR_NPL; ++t) {
        const int i = lane + 32 * t;
        yv[k][t] = i < n ? yr[k * n + i] : make_float2(0.0f, 0.0f);
      }
    const __half2 *w = a.weights + (size_t)row * B * n;
    __half2 wv[(W_B_MAX_RR * RR_MAX_N) / 32];
#pragma unroll
    for (int q = 0; q < (W_B_MAX_RR * RR_MAX_N) / 32; ++q) {
      const int e = lane + 32 * q;
      if (e < B * n) wv[q] = w[e];
    }
#pragma unroll
    for (int t = 0; t < RR_NPL; ++t) {
      const int i = lane + 32 * t;
      if (i < n) {
        const float2 d = fac[i];
        const float dm2 = d.x * d.x + d.y * d.y;
        const float rm = dm2 > 0.0f ? rsqrtf(dm2) : 0.0f;
        const float2 ph = dm2 > 0.0f ? make_float2(d.x * rm, d.y * rm) : make_float2(1.0f, 0.0f);
#pragma unroll
        for (int k = 0; k < KV; ++k) U[k * n + i] = cmul(yv[k][t], ph);
      }
    }
#pragma unroll
    for (int q = 0; q < (W_B_MAX_RR * RR_MAX_N) / 32; ++q) {
      const int e = lane + 32 * q;
      if (e < B * n) W0[e] = __half22float2(wv[q]);
    }
  }
  __syncwarp();

  // orthonormal basis of the four vectors in X (n x 4): classical Gram-Schmidt
  // twice, the dots of vector k with the earlier ones reduced together; a
  // vector that vanishes is replaced by a fixed unit vector and redone
  auto orth = [&](float2 *X) {
#pragma unroll
    for (int k = 0; k < KV; ++k) {
      float2 xl0[KV], xl1[KV];
#pragma unroll
      for (int l = 0; l < KV; ++l) {
        xl0[l] = l < k && r0 ? X[l * n + lane] : make_float2(0.0f, 0.0f);
        xl1[l] = l < k && r1 ? X[l * n + lane + 32] : make_float2(0.0f, 0.0f);
      }
      for (int attempt = 0; attempt < 2; ++attempt) {
        float2 x0 = r0 ? X[k * n + lane] : make_float2(0.0f, 0.0f);
        float2 x1 = r1 ? X[k * n + lane + 32] : make_float2(0.0f, 0.0f);
        if (attempt > 0) {
          const int e1 = (k * 7 + 2 + attempt) % n;
          x0 = make_float2(lane == e1 ? 1.0f : 0.0f, 0.0f);
          x1 = make_float2(lane + 32 == e1 ? 1.0f : 0.0f, 0.0f);
        }
        if (k > 0) {
#pragma unroll
          for (int round = 0; round < 2; ++round) {
            float dr[KV - 1], di[KV - 1];  // <x_l, x_k>
#pragma unroll
            for (int l = 0; l < KV - 1; ++l) {
              dr[l] = xl0[l].x * x0.x + xl0[l].y * x0.y + xl1[l].x * x1.x + xl1[l].y * x1.y;
              di[l] = xl0[l].x * x0.y - xl0[l].y * x0.x + xl1[l].x * x1.y - xl1[l].y * x1.x;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
              for (int l = 0; l < KV - 1; ++l) {
                dr[l] += __shfl_xor_sync(0xffffffffu, dr[l], o);
                di[l] += __shfl_xor_sync(0xffffffffu, di[l], o);
              }
            }
#pragma unroll
            for (int l = 0; l < KV - 1; ++l) {
              if (l < k) {
                x0.x -= dr[l] * xl0[l].x - di[l] * xl0[l].y;
                x0.y -= dr[l] * xl0[l].y + di[l] * xl0[l].x;
                x1.x -= dr[l] * xl1[l].x - di[l] * xl1[l].y;
                x1.y -= dr[l] * xl1[l].y + di[l] * xl1[l].x;
              }
            }
          }
        }
        const float nr = wsum(x0.x * x0.x + x0.y * x0.y + x1.x * x1.x + x1.y * x1.y);
        if (nr > 1e-20f || attempt == 1) {
          const float inv = nr > 1e-20f ? rsqrtf(nr) : 0.0f;
          if (r0) X[k * n + lane] = make_float2(x0.x * inv, x0.y * inv);
          if (r1) X[k * n + lane + 32] = make_float2(x1.x * inv, x1.y * inv);
          break;
        }
      }
      __syncwarp();
    }
  };
  // V = A U (lane: rows lane, lane + 32)
  auto apply = [&]() {
    float2 acc[RR_NPL][KV];
#pragma unroll
    for (int t = 0; t < RR_NPL; ++t)
#pragma unroll
      for (int k = 0; k < KV; ++k) acc[t][k] = make_float2(0.0f, 0.0f);
    int j = 0;
    for (; j + 1 < n; j += 2) {
      float2 uj[2][KV], aij[2][RR_NPL];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
#pragma unroll
        for (int k = 0; k < KV; ++k) uj[h][k] = U[k * n + j + h];
#pragma unroll
        for (int t = 0; t < RR_NPL; ++t) {
          const int i = lane + 32 * t;
          aij[h][t] = i < n ? A[i * ld + j + h] : make_float2(0.0f, 0.0f);
        }
      }
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int t = 0; t < RR_NPL; ++t)
#pragma unroll
          for (int k = 0; k < KV; ++k) {
            const float2 pr = cmul(aij[h][t], uj[h][k]);
            acc[t][k].x += pr.x;
            acc[t][k].y += pr.y;
          }
    }
    if (j < n) {
#pragma unroll
      for (int t = 0; t < RR_NPL; ++t) {
        const int i = lane + 32 * t;
        const float2 aj = i < n ? A[i * ld + j] : make_float2(0.0f, 0.0f);
#pragma unroll
        for (int k = 0; k < KV; ++k) {
          const float2 pr = cmul(aj, U[k * n + j]);
          acc[t][k].x += pr.x;
          acc[t][k].y += pr.y;
        }
      }
    }
#pragma unroll
    for (int t = 0; t < RR_NPL; ++t) {
      const int i = lane + 32 * t;
      if (i < n)
#pragma unroll
        for (int k = 0; k < KV; ++k) V[k * n + i] = acc[t][k];
    }
    __syncwarp();
  };

  orth(U);
  for (int it = 0; it < a.n_iter; ++it) {
    apply();
    for (int e = lane; e < KV * n; e += 32) U[e] = V[e];
    __syncwarp();
    orth(U);
  }
  apply();
  // H = U^H A U (Hermitian 4 x 4), every lane a copy: the 10 entries k <= l in one reduction
  float2 H[KV][KV];
  {
    float hv[2 * KV * KV];
#pragma unroll
    for (int q = 0; q < 2 * KV * KV; ++q) hv[q] = 0.0f;
#pragma unroll
    for (int t = 0; t < RR_NPL; ++t) {
      const int i = lane + 32 * t;
      if (i < n) {
        float2 uk[KV], vl[KV];
#pragma unroll
        for (int k = 0; k < KV; ++k) {
          uk[k] = U[k * n + i];
          vl[k] = V[k * n + i];
        }
#pragma unroll
        for (int k = 0; k < KV; ++k)
#pragma unroll
          for (int l = k; l < KV; ++l) {  // conj(u_k) . v_l
            hv[2 * (k * KV + l)] += uk[k].x * vl[l].x + uk[k].y * vl[l].y;
            hv[2 * (k * KV + l) + 1] += uk[k].x * vl[l].y - uk[k].y * vl[l].x;
          }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int k = 0; k < KV; ++k)
#pragma unroll
        for (int l = k; l < KV; ++l) {
          hv[2 * (k * KV + l)] += __shfl_xor_sync(0xffffffffu, hv[2 * (k * KV + l)], o);
          hv[2 * (k * KV + l) + 1] += __shfl_xor_sync(0xffffffffu, hv[2 * (k * KV + l) + 1], o);
        }
    }
#pragma unroll
    for (int k = 0; k < KV; ++k)
#pragma unroll
      for (int l = k; l < KV; ++l) {
        H[k][l] = make_float2(hv[2 * (k * KV + l)], hv[2 * (k * KV + l) + 1]);
        H[l][k] = make_float2(H[k][l].x, -H[k][l].y);
      }
#pragma unroll
    for (int k = 0; k < KV; ++k) H[k][k].y = 0.0f;
  }
  // cyclic Jacobi on the 4 x 4 Hermitian H: J = I except J_pp = c, J_pq = s,
  // J_qp = -s conj(e), J_qq = c conj(e) with H_pq = g e (|e| = 1),
  // t = sign(tau) / (|tau| + sqrt(1 + tau^2)), tau = (H_qq - H_pp) / (2 g)
  float2 Q[KV][KV];
#pragma unroll
  for (int k = 0; k < KV; ++k)
#pragma unroll
    for (int l = 0; l < KV; ++l) Q[k][l] = make_float2(k == l ? 1.0f : 0.0f, 0.0f);
  for (int sweep = 0; sweep < 10; ++sweep) {
    float off = 0.0f, diag = 0.0f;
#pragma unroll
    for (int k = 0; k < KV; ++k) {
      diag += fabsf(H[k][k].x);
#pragma unroll
      for (int l = 0; l < KV; ++l)
        if (l != k) off += H[k][l].x * H[k][l].x + H[k][l].y * H[k][l].y;
    }
    if (off <= 1e-10f * diag * diag + 1e-30f) break;  // residuals are tested at 1e-3 theta_0
#pragma unroll
    for (int pp = 0; pp < KV - 1; ++pp)
#pragma unroll
      for (int qq = pp + 1; qq < KV; ++qq) {
        const float2 h = H[pp][qq];
        const float g2 = h.x * h.x + h.y * h.y;
        if (!(g2 > 1e-36f)) continue;  // |H_pq| below 1e-18: nothing to rotate
        const float rg = rsqrtf(g2);
        const float2 e = make_float2(h.x * rg, h.y * rg);
        const float tau = (H[qq][qq].x - H[pp][pp].x) * (0.5f * rg);
        const float tau2 = 1.0f + tau * tau;
        const float t = __fdividef(tau >= 0.0f ? 1.0f : -1.0f, fabsf(tau) + tau2 * rsqrtf(tau2));
        const float cs = rsqrtf(1.0f + t * t), sn = t * cs;
        const float2 ce = make_float2(e.x, -e.y);  // conj(e)
        // columns: col p' = c col p - s conj(e) col q ; col q' = s col p + c conj(e) col q
#pragma unroll
        for (int r = 0; r < KV; ++r) {
          const float2 hp = H[r][pp], hq = H[r][qq];
          const float2 sq = cmul(ce, hq);
          H[r][pp] = make_float2(cs * hp.x - sn * sq.x, cs * hp.y - sn * sq.y);
          H[r][qq] = make_float2(sn * hp.x + cs * sq.x, sn * hp.y + cs * sq.y);
          const float2 qp = Q[r][pp], qv = Q[r][qq];
          const float2 sv = cmul(ce, qv);
          Q[r][pp] = make_float2(cs * qp.x - sn * sv.x, cs * qp.y - sn * sv.y);
          Q[r][qq] = make_float2(sn * qp.x + cs * sv.x, sn * qp.y + cs * sv.y);
        }
        // rows: row p' = c row p - s e row q ; row q' = s row p + c e row q
#pragma unroll
        for (int r = 0; r < KV; ++r) {
          const float2 hp = H[pp][r], hq = H[qq][r];
          const float2 eq = cmul(e, hq);
          H[pp][r] = make_float2(cs * hp.x - sn * eq.x, cs * hp.y - sn * eq.y);
          H[qq][r] = make_float2(sn * hp.x + cs * eq.x, sn * hp.y + cs * eq.y);
        }
      }
  }
  // Ritz values descending, Ritz vectors U Q, A U Q (kept in registers for the residuals)
  // (a compare-exchange network on values, so nothing is indexed at run time)
  float theta[KV];
#pragma unroll
  for (int k = 0; k < KV; ++k) theta[k] = H[k][k].x;
#pragma unroll
  for (int pass = 0; pass < KV - 1; ++pass)
#pragma unroll
    for (int l = 0; l < KV - 1; ++l)
      if (theta[l] < theta[l + 1]) {
        const float tt = theta[l];
        theta[l] = theta[l + 1];
        theta[l + 1] = tt;
#pragma unroll
        for (int r = 0; r < KV; ++r) {  // the Ritz vectors' coefficients follow their values
          const float2 tq = Q[r][l];
          Q[r][l] = Q[r][l + 1];
          Q[r][l + 1] = tq;
        }
      }
  // trace and the residuals ||A u_k - theta_k u_k||^2 in one reduction
  float rs[KV + 1];
#pragma unroll
  for (int k = 0; k <= KV; ++k) rs[k] = 0.0f;
#pragma unroll
  for (int t = 0; t < RR_NPL; ++t) {
    const int i = lane + 32 * t;
    if (i >= n) continue;
    rs[KV] += A[i * ld + i].x;
    float2 uo[KV], vo[KV];
#pragma unroll
    for (int k = 0; k < KV; ++k) {
      uo[k] = U[k * n + i];
      vo[k] = V[k * n + i];
    }
#pragma unroll
    for (int k = 0; k < KV; ++k) {
      float2 un = make_float2(0.0f, 0.0f), vn = make_float2(0.0f, 0.0f);
#pragma unroll
      for (int l = 0; l < KV; ++l) {
        const float2 q = Q[l][k];
        const float2 a1 = cmul(uo[l], q), a2 = cmul(vo[l], q);
        un.x += a1.x;
        un.y += a1.y;
        vn.x += a2.x;
        vn.y += a2.y;
      }
      U[k * n + i] = un;
      const float dx = vn.x - theta[k] * un.x, dy = vn.y - theta[k] * un.y;
      rs[k] += dx * dx + dy * dy;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k <= KV; ++k) rs[k] += __shfl_xor_sync(0xffffffffu, rs[k], o);
  }
  __syncwarp();
  const float trace = rs[KV];
  float res[KV];
#pragma unroll
  for (int k = 0; k < KV; ++k) res[k] = sqrtf(rs[k]);
  const float floor_est = (trace - (theta[0] + theta[1] + theta[2] + theta[3])) / static_cast<float>(n - KV);
  int K = 0;
  bool accept = true;
  if (a.k_rule == SF_K_FIXED) {
    K = a.fixed_counts ? a.fixed_counts[c] : 0;
    K = max(0, min(n, K));
    accept = K <= KV;
  } else if (a.k_rule == SF_K_NOISE_FLOOR) {
#pragma unroll
    for (int k = 0; k < KV; ++k) K += theta[k] > a.delta * floor_est;
    accept = K < KV;  // four above the floor: more may be, the full solver decides
  } else {
    accept = false;  // the percentile rule needs every eigenvalue
  }
  const float anorm = fmaxf(theta[0], 1e-30f);
#pragma unroll
  for (int k = 0; k < KV; ++k)
    if (k < K && !(res[k] <= a.tol * anorm)) accept = false;
  if (a.ritz && lane < KV) {
    float tl = theta[0];
#pragma unroll
    for (int k = 1; k < KV; ++k)
      if (lane == k) tl = theta[k];
    a.ritz[(size_t)row * KV + lane] = tl;
  }
  if (!accept) {
    if (lane == 0) {
      const int slot = atomicAdd(a.fb_count, 1);
      a.fb_list[slot] = row;
    }
    return;
  }
  if (lane == 0 && a.counts) a.counts[row] = K;
  // un-whiten and normalise the kept vectors (norms in one reduction), then
  // W' = W - sum_k (W z_k) z_k^H with the coefficients of four beams per reduction
  float2 z0[KV], z1[KV];
  {
    const float s0 = r0 ? s[lane] : 0.0f, s1 = r1 ? s[lane + 32] : 0.0f;
    float nr[KV];
#pragma unroll
    for (int k = 0; k < KV; ++k) {
      z0[k] = k < K && r0 ? U[k * n + lane] : make_float2(0.0f, 0.0f);
      z1[k] = k < K && r1 ? U[k * n + lane + 32] : make_float2(0.0f, 0.0f);
      z0[k] = make_float2(z0[k].x * s0, z0[k].y * s0);
      z1[k] = make_float2(z1[k].x * s1, z1[k].y * s1);
      nr[k] = z0[k].x * z0[k].x + z0[k].y * z0[k].y + z1[k].x * z1[k].x + z1[k].y * z1[k].y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int k = 0; k < KV; ++k) nr[k] += __shfl_xor_sync(0xffffffffu, nr[k], o);
    }
#pragma unroll
    for (int k = 0; k < KV; ++k) {
      const float inv = nr[k] > 0.0f ? rsqrtf(nr[k]) : 0.0f;
      z0[k] = make_float2(z0[k].x * inv, z0[k].y * inv);
      z1[k] = make_float2(z1[k].x * inv, z1[k].y * inv);
    }
  }
  float2 *we = a.weff + (size_t)row * 2 * B * n;
  const float2 f0 = r0 ? fac[lane] : make_float2(0.0f, 0.0f), f1 = r1 ? fac[lane + 32] : make_float2(0.0f, 0.0f);
  for (int m0 = 0; m0 < B; m0 += 4) {
    float cr[4][KV], ci[4][KV];
    float2 wa[4], wb[4];
#pragma unroll
    for (int mm = 0; mm < 4; ++mm) {
      const bool on = m0 + mm < B;
      wa[mm] = on && r0 ? W0[(m0 + mm) * n + lane] : make_float2(0.0f, 0.0f);
      wb[mm] = on && r1 ? W0[(m0 + mm) * n + lane + 32] : make_float2(0.0f, 0.0f);
#pragma unroll
      for (int k = 0; k < KV; ++k) {  // W_m . z_k
        const float2 p0 = cmul(wa[mm], z0[k]), p1 = cmul(wb[mm], z1[k]);
        cr[mm][k] = p0.x + p1.x;
        ci[mm][k] = p0.y + p1.y;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int mm = 0; mm < 4; ++mm)
#pragma unroll
        for (int k = 0; k < KV; ++k) {
          cr[mm][k] += __shfl_xor_sync(0xffffffffu, cr[mm][k], o);
          ci[mm][k] += __shfl_xor_sync(0xffffffffu, ci[mm][k], o);
        }
    }
#pragma unroll
    for (int mm = 0; mm < 4; ++mm) {
      const int m = m0 + mm;
      if (m >= B) continue;
      float2 pa = wa[mm], pb = wb[mm];
#pragma unroll
      for (int k = 0; k < KV; ++k) {
        if (k < K) {
          const float2 cf = make_float2(cr[mm][k], ci[mm][k]);
          const float2 t0 = cmulc(cf, z0[k]), t1 = cmulc(cf, z1[k]);  // c conj(z_i)
          pa.x -= t0.x;
          pa.y -= t0.y;
          pb.x -= t1.x;
          pb.y -= t1.y;
        }
      }
      if (r0) {
        we[m * n + lane] = cmul(wa[mm], f0);
        we[B * n + m * n + lane] = cmul(pa, f0);
      }
      if (r1) {
        we[m * n + lane + 32] = cmul(wb[mm], f1);
        we[B * n + m * n + lane + 32] = cmul(pb, f1);
      }
    }
  }
}

}  // namespace

struct sf_proposer {
  int R, NBL, in, in_ld, hid, out, out_ld, max_rows;
  float *w[3] = {nullptr, nullptr, nullptr}, *b[3] = {nullptr, nullptr, nullptr};
  float *gw[3] = {nullptr, nullptr, nullptr}, *gb[3] = {nullptr, nullptr, nullptr};
  float *mw[3] = {nullptr, nullptr, nullptr}, *vw[3] = {nullptr, nullptr, nullptr};
  float *mb[3] = {nullptr, nullptr, nullptr}, *vb[3] = {nullptr, nullptr, nullptr};
  __nv_bfloat16 *wh[3] = {nullptr, nullptr, nullptr};
  __nv_bfloat16 *x = nullptr, *h1 = nullptr, *h2 = nullptr, *dy = nullptr, *dh2 = nullptr, *dh1 = nullptr;
  float *y = nullptr;
  int32_t *fb_list = nullptr, *fb_count = nullptr;
  uint32_t *status = nullptr;
  int step = 0;
  int rows_in[3], rows_out[3];  // layer l: out x in
};

namespace {

void free_proposer(sf_proposer *q) {
  if (!q) return;
  for (int l = 0; l < 3; ++l) {
    cudaFree(q->w[l]);
    cudaFree(q->b[l]);
    cudaFree(q->gw[l]);
    cudaFree(q->gb[l]);
    cudaFree(q->mw[l]);
    cudaFree(q->vw[l]);
    cudaFree(q->mb[l]);
    cudaFree(q->vb[l]);
    cudaFree(q->wh[l]);
  }
  cudaFree(q->x);
  cudaFree(q->h1);
  cudaFree(q->h2);
  cudaFree(q->dy);
  cudaFree(q->dh2);
  cudaFree(q->dh1);
  cudaFree(q->y);
  cudaFree(q->fb_list);
  cudaFree(q->fb_count);
  cudaFree(q->status);
  delete q;
}

size_t rr_smem_per_warp(int n, int B) { return rr_region(n, B); }

}  // namespace

extern "C" {

int sf_proposer_create(int32_t n_receivers, int32_t hidden, int32_t max_rows, sf_proposer **out) {
  if (!out) return fail(SF_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  if (n_receivers < 8 || n_receivers > RR_MAX_N)
    return fail(SF_ERR_UNSUPPORTED, "the proposer handles 8..%d receivers (got %d)", RR_MAX_N, n_receivers);
  if (hidden < 64 || hidden % 64 != 0) return fail(SF_ERR_INVALID_ARGUMENT, "hidden width must be a multiple of 64");
  if (max_rows < 1) return fail(SF_ERR_INVALID_ARGUMENT, "max_rows must be >= 1");
  sf_proposer *q = new (std::nothrow) sf_proposer();
  if (!q) return fail(SF_ERR_INVALID_ARGUMENT, "out of host memory");
  q->R = n_receivers;
  q->NBL = n_receivers * (n_receivers + 1) / 2;
  q->in = 2 * q->NBL;
  q->in_ld = (q->in + 63) / 64 * 64;
  q->hid = hidden;
  q->out = 2 * KV * n_receivers;
  q->out_ld = (q->out + 63) / 64 * 64;
  q->max_rows = max_rows;
  const int outs[3] = {hidden, hidden, q->out}, ins[3] = {q->in_ld, hidden, hidden};
  cudaError_t e = cudaSuccess;
  for (int l = 0; l < 3 && e == cudaSuccess; ++l) {
    q->rows_out[l] = outs[l];
    q->rows_in[l] = ins[l];
    const size_t nw = (size_t)outs[l] * ins[l], nb = outs[l];
    float **fw[4] = {&q->w[l], &q->gw[l], &q->mw[l], &q->vw[l]};
    for (float **pp : fw)
      if (e == cudaSuccess) e = cudaMalloc(pp, sizeof(float) * nw);
    float **fb[4] = {&q->b[l], &q->gb[l], &q->mb[l], &q->vb[l]};
    for (float **pp : fb)
      if (e == cudaSuccess) e = cudaMalloc(pp, sizeof(float) * nb);
    if (e == cudaSuccess) e = cudaMalloc(&q->wh[l], sizeof(__nv_bfloat16) * nw);
    for (float **pp : fw)
      if (e == cudaSuccess) e = cudaMemset(*pp, 0, sizeof(float) * nw);
    for (float **pp : fb)
      if (e == cudaSuccess) e = cudaMemset(*pp, 0, sizeof(float) * nb);
    if (e == cudaSuccess) e = cudaMemset(q->wh[l], 0, sizeof(__nv_bfloat16) * nw);
  }
  const size_t r = max_rows;
  if (e == cudaSuccess) e = cudaMalloc(&q->x, sizeof(__nv_bfloat16) * r * q->in_ld);
  if (e == cudaSuccess) e = cudaMalloc(&q->h1, sizeof(__nv_bfloat16) * r * hidden);
  if (e == cudaSuccess) e = cudaMalloc(&q->h2, sizeof(__nv_bfloat16) * r * hidden);
  if (e == cudaSuccess) e = cudaMalloc(&q->dh2, sizeof(__nv_bfloat16) * r * hidden);
  if (e == cudaSuccess) e = cudaMalloc(&q->dh1, sizeof(__nv_bfloat16) * r * hidden);
  if (e == cudaSuccess) e = cudaMalloc(&q->dy, sizeof(__nv_bfloat16) * r * q->out_ld);
  if (e == cudaSuccess) e = cudaMalloc(&q->y, sizeof(float) * r * q->out);
  if (e == cudaSuccess) e = cudaMalloc(&q->fb_list, sizeof(int32_t) * r);
  if (e == cudaSuccess) e = cudaMalloc(&q->fb_count, sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&q->status, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(q->dy, 0, sizeof(__nv_bfloat16) * r * q->out_ld);
  if (e == cudaSuccess) e = cudaMemset(q->status, 0, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    free_proposer(q);
    return cuda_fail(e, "proposer create");
  }
  *out = q;
  return SF_OK;
}

int sf_proposer_destroy(sf_proposer *q) {
  if (q) cudaDeviceSynchronize();
  free_proposer(q);
  return SF_OK;
}

int sf_proposer_dims(const sf_proposer *q, int32_t *dims) {
  if (!q || !dims) return fail(SF_ERR_INVALID_ARGUMENT, "NULL argument");
  dims[0] = q->in;
  dims[1] = q->in_ld;
  dims[2] = q->hid;
  dims[3] = q->out;
  dims[4] = q->out_ld;
  dims[5] = q->max_rows;
  return SF_OK;
}

// Host fp32 parameters: layer l weight [out][in] (in = in_ld for layer 0) and bias [out].
int sf_proposer_set_params(sf_proposer *q, const float *w0, const float *b0, const float *w1, const float *b1,
                           const float *w2, const float *b2, void *stream) {
  if (!q || !w0 || !b0 || !w1 || !b1 || !w2 || !b2) return fail(SF_ERR_INVALID_ARGUMENT, "NULL argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const float *ws[3] = {w0, w1, w2}, *bs[3] = {b0, b1, b2};
  for (int l = 0; l < 3; ++l) {
    const size_t nw = (size_t)q->rows_out[l] * q->rows_in[l];
    PR_TRY(cudaMemcpyAsync(q->w[l], ws[l], sizeof(float) * nw, cudaMemcpyHostToDevice, s), "params upload");
    PR_TRY(cudaMemcpyAsync(q->b[l], bs[l], sizeof(float) * q->rows_out[l], cudaMemcpyHostToDevice, s), "params upload");
    PR_TRY(cudaMemsetAsync(q->mw[l], 0, sizeof(float) * nw, s), "params reset");
    PR_TRY(cudaMemsetAsync(q->vw[l], 0, sizeof(float) * nw, s), "params reset");
    PR_TRY(cudaMemsetAsync(q->mb[l], 0, sizeof(float) * q->rows_out[l], s), "params reset");
    PR_TRY(cudaMemsetAsync(q->vb[l], 0, sizeof(float) * q->rows_out[l], s), "params reset");
    // bf16 copy through a zero-learning-rate Adam pass (no gradient, no movement)
    PR_TRY(sf_launch_adam(q->w[l], q->gw[l], q->mw[l], q->vw[l], q->wh[l], (int)nw, 0.0f, 1, s), "params bf16");
  }
  PR_TRY(cudaStreamSynchronize(s), "params upload");
  q->step = 0;
  return SF_OK;
}

int sf_proposer_get_params(const sf_proposer *q, float *w0, float *b0, float *w1, float *b1, float *w2, float *b2,
                           void *stream) {
  if (!q) return fail(SF_ERR_INVALID_ARGUMENT, "proposer is NULL");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  float *ws[3] = {w0, w1, w2}, *bs[3] = {b0, b1, b2};
  for (int l = 0; l < 3; ++l) {
    if (ws[l])
      PR_TRY(cudaMemcpyAsync(ws[l], q->w[l], sizeof(float) * q->rows_out[l] * q->rows_in[l], cudaMemcpyDeviceToHost, s),
             "params download");
    if (bs[l])
      PR_TRY(cudaMemcpyAsync(bs[l], q->b[l], sizeof(float) * q->rows_out[l], cudaMemcpyDeviceToHost, s),
             "params download");
  }
  PR_TRY(cudaStreamSynchronize(s), "params download");
  return SF_OK;
}

int sf_gemm_bf16(int32_t M, int32_t N, int32_t K, const uint16_t *A, int32_t lda, int32_t a_mn_major,
                 const uint16_t *B, int32_t ldb, int32_t b_mn_major, int32_t epilogue, const float *bias,
                 const uint16_t *mask, int32_t ldm, void *out, int32_t ldo, int32_t k_splits, uint32_t *d_status,
                 void *stream) {
  if (!A || !B || !out || !d_status) return fail(SF_ERR_INVALID_ARGUMENT, "NULL buffer");
  if (epilogue < 0 || epilogue > 3) return fail(SF_ERR_INVALID_ARGUMENT, "unknown epilogue %d", epilogue);
  if (epilogue == 2 && !mask) return fail(SF_ERR_INVALID_ARGUMENT, "epilogue 2 needs a mask");
  PR_TRY(sf_launch_gemm_bf16(M, N, K, A, lda, a_mn_major, B, ldb, b_mn_major, epilogue, bias, mask, ldm, out, ldo,
                             k_splits, d_status, static_cast<cudaStream_t>(stream)),
         "bf16 GEMM");
  return SF_OK;
}

int sf_proposer_features(const sf_plan *plan, const int32_t *d_vis, uint16_t *d_x, int32_t ldx, void *stream) {
  if (!plan || !d_vis || !d_x) return fail(SF_ERR_INVALID_ARGUMENT, "NULL argument");
  if (plan->R > RR_MAX_N || ldx < 2 * plan->NBL) return fail(SF_ERR_UNSUPPORTED, "features: shape");
  sf_proposer_features_kernel<<<2 * plan->C, 128, 0, static_cast<cudaStream_t>(stream)>>>(
      d_vis, plan->R, plan->NBL, reinterpret_cast<__nv_bfloat16 *>(d_x), ldx);
  PR_TRY(cudaGetLastError(), "features launch");
  return SF_OK;
}

int sf_proposer_targets(const sf_plan *plan, const int32_t *d_vis, const float *d_evals, const float *d_evecs,
                        float *d_targets, float *d_weights, void *stream) {
  if (!plan || !d_vis || !d_evals || !d_evecs || !d_targets || !d_weights)
    return fail(SF_ERR_INVALID_ARGUMENT, "NULL argument");
  PR_TRY(sf_launch_proposer_targets(d_vis, d_evals, d_evecs, plan->C, plan->R, d_targets, d_weights,
                                    static_cast<cudaStream_t>(stream)),
         "targets launch");
  return SF_OK;
}

int sf_proposer_infer(sf_proposer *q, const uint16_t *d_x, int32_t rows, float *d_y, void *stream) {
  if (!q || !d_x || !d_y) return fail(SF_ERR_INVALID_ARGUMENT, "NULL argument");
  if (rows < 1 || rows > q->max_rows) return fail(SF_ERR_INVALID_ARGUMENT, "rows outside [1, %d]", q->max_rows);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  PR_TRY(sf_launch_gemm_bf16(rows, q->hid, q->in_ld, d_x, q->in_ld, 0, q->wh[0], q->in_ld, 0, 0, q->b[0], nullptr, 0,
                             q->h1, q->hid, 1, q->status, s),
         "layer 1");
  PR_TRY(sf_launch_gemm_bf16(rows, q->hid, q->hid, q->h1, q->hid, 0, q->wh[1], q->hid, 0, 0, q->b[1], nullptr, 0, q->h2,
                             q->hid, 1, q->status, s),
         "layer 2");
  PR_TRY(sf_launch_gemm_bf16(rows, q->out, q->hid, q->h2, q->hid, 0, q->wh[2], q->hid, 0, 1, q->b[2], nullptr, 0, d_y,
                             q->out, 1, q->status, s),
         "layer 3");
  return SF_OK;
}

// One Adam step on a batch: forward, weighted squared error against the
// targets, backward through the three layers (weight gradients by split-K
// GEMMs), Adam.  d_loss (one float) is increased by the batch's loss.
int sf_proposer_train_step(sf_proposer *q, const uint16_t *d_x, const float *d_t, const float *d_tw, int32_t rows,
                           float lr, float *d_loss, void *stream) {
  if (!q || !d_x || !d_t || !d_tw || !d_loss) return fail(SF_ERR_INVALID_ARGUMENT, "NULL argument");
  if (rows < 1 || rows > q->max_rows) return fail(SF_ERR_INVALID_ARGUMENT, "rows outside [1, %d]", q->max_rows);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (int rc = sf_proposer_infer(q, d_x, rows, q->y, stream)) return rc;
  PR_TRY(sf_launch_proposer_loss(q->y, d_t, d_tw, rows, q->out, q->R, q->dy, q->out_ld, d_loss, s), "loss");
  const int splits = rows >= 4096 ? 8 : 1;
  // layer 3: gW3 += dY^T H2, gb3 = colsum dY, dH2 = (dY W3) [H2 > 0]
  PR_TRY(sf_launch_gemm_bf16(q->out, q->hid, rows, q->dy, q->out_ld, 1, q->h2, q->hid, 1, 3, nullptr, nullptr, 0,
                             q->gw[2], q->hid, splits, q->status, s),
         "gW3");
  PR_TRY(sf_launch_column_sums(q->dy, rows, q->out, q->out_ld, q->gb[2], s), "gb3");
  PR_TRY(sf_launch_gemm_bf16(rows, q->hid, q->out, q->dy, q->out_ld, 0, q->wh[2], q->hid, 1, 2, nullptr, q->h2, q->hid,
                             q->dh2, q->hid, 1, q->status, s),
         "dH2");
  // layer 2
  PR_TRY(sf_launch_gemm_bf16(q->hid, q->hid, rows, q->dh2, q->hid, 1, q->h1, q->hid, 1, 3, nullptr, nullptr, 0,
                             q->gw[1], q->hid, splits, q->status, s),
         "gW2");
  PR_TRY(sf_launch_column_sums(q->dh2, rows, q->hid, q->hid, q->gb[1], s), "gb2");
  PR_TRY(sf_launch_gemm_bf16(rows, q->hid, q->hid, q->dh2, q->hid, 0, q->wh[1], q->hid, 1, 2, nullptr, q->h1, q->hid,
                             q->dh1, q->hid, 1, q->status, s),
         "dH1");
  // layer 1
  PR_TRY(sf_launch_gemm_bf16(q->hid, q->in_ld, rows, q->dh1, q->hid, 1, d_x, q->in_ld, 1, 3, nullptr, nullptr, 0,
                             q->gw[0], q->in_ld, splits, q->status, s),
         "gW1");
  PR_TRY(sf_launch_column_sums(q->dh1, rows, q->hid, q->hid, q->gb[0], s), "gb1");
  ++q->step;
  for (int l = 0; l < 3; ++l) {
    PR_TRY(sf_launch_adam(q->w[l], q->gw[l], q->mw[l], q->vw[l], q->wh[l], q->rows_out[l] * q->rows_in[l], lr, q->step,
                          s),
           "adam");
    PR_TRY(sf_launch_adam(q->b[l], q->gb[l], q->mb[l], q->vb[l], nullptr, q->rows_out[l], lr, q->step, s), "adam");
  }
  return SF_OK;
}

int sf_proposer_status(sf_proposer *q, void *stream, uint32_t *out_bits) {
  if (!q) return fail(SF_ERR_INVALID_ARGUMENT, "proposer is NULL");
  uint32_t bits = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  PR_TRY(cudaMemcpyAsync(&bits, q->status, sizeof(bits), cudaMemcpyDeviceToHost, s), "status");
  PR_TRY(cudaMemsetAsync(q->status, 0, sizeof(uint32_t), s), "status");
  PR_TRY(cudaStreamSynchronize(s), "status");
  if (out_bits) *out_bits = bits;
  if (bits) return fail(SF_ERR_DEVICE, "device error bits 0x%x", bits);
  return SF_OK;
}

int sf_covariance_eig_learned(sf_plan *plan, sf_proposer *q, const int32_t *d_vis, int32_t k_rule, float delta,
                              int32_t n_iter, float tol, int32_t *d_counts, float *d_ritz, int32_t *d_fallback_count,
                              void *stream) {
  if (!plan || !q || !d_vis) return fail(SF_ERR_INVALID_ARGUMENT, "NULL argument");
  if (plan->R != q->R) return fail(SF_ERR_INVALID_ARGUMENT, "proposer built for %d receivers, plan has %d", q->R, plan->R);
  const int rows = 2 * plan->C;
  if (rows > q->max_rows) return fail(SF_ERR_UNSUPPORTED, "plan has %d matrices, proposer holds %d", rows, q->max_rows);
  if (plan->B > sf_eig_topk_max_b()) return fail(SF_ERR_UNSUPPORTED, "too many beams");
  if (n_iter < 0 || n_iter > 16) return fail(SF_ERR_INVALID_ARGUMENT, "n_iter outside [0, 16]");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int32_t *counts = d_counts ? d_counts : plan->d_counts;
  if (int rc = sf_proposer_features(plan, d_vis, reinterpret_cast<uint16_t *>(q->x), q->in_ld, stream)) return rc;
  if (int rc = sf_proposer_infer(q, reinterpret_cast<const uint16_t *>(q->x), rows, q->y, stream)) return rc;
  PR_TRY(cudaMemsetAsync(q->fb_count, 0, sizeof(int32_t), s), "fallback reset");
  RRArgs a;
  a.vis = d_vis;
  a.factors = plan->d_factors;
  a.weights = plan->d_weights;
  a.fixed_counts = plan->d_fixed_counts;
  a.y = q->y;
  a.ldy = q->out;
  a.weff = plan->d_weff;
  a.counts = counts;
  a.ritz = d_ritz;
  a.fb_list = q->fb_list;
  a.fb_count = q->fb_count;
  a.C = plan->C;
  a.R = plan->R;
  a.B = plan->B;
  a.NBL = plan->NBL;
  a.rows = rows;
  a.k_rule = k_rule;
  a.delta = delta;
  a.n_iter = n_iter;
  a.tol = tol;
  const size_t per = rr_smem_per_warp(plan->R, plan->B);
  const int wpc = per * 4 <= 200 * 1024 ? 4 : (per * 2 <= 200 * 1024 ? 2 : 1);
  const size_t smem = per * wpc;
  PR_TRY(sf_smem_optin(reinterpret_cast<const void *>(sf_rr_kernel), smem), "RR smem");
  sf_rr_kernel<<<(rows + wpc - 1) / wpc, 32 * wpc, smem, s>>>(a);
  PR_TRY(cudaGetLastError(), "RR launch");
  // the rejected matrices through the full top-K eigensolver
  // (with every eigenvalue, as the plain chain computes them: a rejected matrix gets exactly the
  // plain chain's weights)
  if (sf_eig_small_supported(plan))
    PR_TRY(sf_launch_eig_small(plan, d_vis, k_rule, delta, 0, plan->d_evals, counts, q->fb_list, q->fb_count, s),
           "fallback eig");
  else
    PR_TRY(sf_launch_eig_topk_list(plan, d_vis, q->fb_list, q->fb_count, rows, k_rule, delta, 0, plan->d_evals,
                                   counts, s),
           "fallback eig");
  if (d_fallback_count)
    PR_TRY(cudaMemcpyAsync(d_fallback_count, q->fb_count, sizeof(int32_t), cudaMemcpyDeviceToDevice, s),
           "fallback count");
  return SF_OK;
}

int sf_run_adaptive_learned(sf_plan *plan, sf_proposer *q, const int8_t *d_samples, const int16_t *d_scales,
                            int32_t k_rule, float delta, int32_t n_iter, float tol, int32_t *d_vis, int32_t *d_counts,
                            uint16_t *d_beams_f16, int32_t *d_fallback_count, void *stream) {
  if (!plan) return fail(SF_ERR_INVALID_ARGUMENT, "plan is NULL");
  int32_t *vis = d_vis ? d_vis : plan->d_vis;
  if (int rc = sf_correlate(plan, d_samples, d_scales, SF_WINDOW_ALIGNED, vis, stream)) return rc;
  if (int rc = sf_covariance_eig_learned(plan, q, vis, k_rule, delta, n_iter, tol, d_counts, nullptr, d_fallback_count,
                                         stream))
    return rc;
  return sf_beamform(plan, d_samples, d_scales, SF_WINDOW_ALIGNED, 2, d_beams_f16, stream);
}

}  // extern "C"
