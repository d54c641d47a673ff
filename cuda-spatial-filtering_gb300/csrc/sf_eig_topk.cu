// Adaptive-path eigensolver: one warp per (channel, pol) covariance, all
// eigenvalues + the top-K eigenvectors only (what K selection, I - U U^H and
// the projected weights need).  Used when the caller asks for no eigenvector
// output; the full Jacobi solver (sf_eig.cu) serves the rest.
//
// Per matrix, in shared memory:
//   1. covariance d_i conj(d_j) V(i,j) from the packed int32 upper triangle,
//      diagonal whitening (reference include/spatial/spatial.cuh:1068-1093)
//   2. Householder reduction to a real symmetric tridiagonal T = Q^H A Q
//      (the published LAPACK zhetd2/zlarfg algorithm: reflectors
//      H = I - tau v v^H, subdiagonal made real)
//   3. every eigenvalue by Sturm-sequence bisection, one lane per eigenvalue
//   4. K (fixed, percentile rule of spatial.cuh:900-950, or noise floor)
//   5. the top-K eigenvectors of T by inverse iteration (LU with partial
//      pivoting, three iterations, modified Gram-Schmidt among them), back-
//      transformed through the reflectors, un-whitened and normalised
//      (spatial.cuh:1098-1126)
//   6. effective weights: slot 0 W diag(d), slot 1 (W P) diag(d) with
//      P = I - sum_k w_k u_k u_k^H (null: w = 1 on the un-whitened u;
//      shrink: w = 1 - lambda_bar / lambda_k on the whitened v).
#include <cstdio>

#include "sf_common.cuh"
#include "sf_plan.cuh"

namespace {

constexpr int WARPS = 2;  // the two polarisations of one channel
constexpr int MAX_N = 64;
constexpr int GROUP = 4;  // inverse-iteration vectors solved at once (one lane each)
constexpr int INV_ITERS = 3;

struct TopkArgs {
  const int32_t *vis;
  const float2 *factors;
  const __half2 *weights;
  const int32_t *fixed_counts;
  float *evals;
  int32_t *counts;
  float2 *weff;
  uint32_t *status;
  int C, R, B, NBL;
  int k_rule, shrink;
  float delta;
};

__host__ __device__ inline size_t topk_warp_floats(int n, int B) {
  // A, 4 complex vectors, X (even), LU workspace (GROUP even), Wp, 5 real vectors
  size_t f = (size_t)2 * n * (n + 1) + 8 * (size_t)n + (((size_t)n * n + 1) & ~(size_t)1) +
             5 * GROUP * (size_t)n + 2 * (size_t)B * n + 5 * (size_t)n;
  return (f + 3) & ~(size_t)3;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ float percentile_sorted(const float *v, int n, float quant) {
  if (n <= 0) return 0.0f;
  if (n == 1) return v[0];
  const float qc = fminf(1.0f, fmaxf(0.0f, quant));
  const float pos = qc * static_cast<float>(n - 1);
  const int lo = static_cast<int>(floorf(pos));
  const int hi = static_cast<int>(ceilf(pos));
  if (lo == hi) return v[lo];
  const float frac = pos - static_cast<float>(lo);
  return v[lo] + frac * (v[hi] - v[lo]);
}

// #{eigenvalues of T < x}: Sturm sequence of the LDL^T factorisation.
__device__ __forceinline__ int sturm_count(const float *d, const float *e2, int n, float x,
                                           float pivmin) {
  int cnt = 0;
  float q = d[0] - x;
  if (fabsf(q) < pivmin) q = -pivmin;
  cnt += q < 0.0f;
  for (int i = 1; i < n; ++i) {
    q = d[i] - x - __fdividef(e2[i - 1], q);
    if (fabsf(q) < pivmin) q = -pivmin;
    cnt += q < 0.0f;
  }
  return cnt;
}

__global__ void __launch_bounds__(WARPS * 32) sf_eig_topk_kernel(const TopkArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int n = a.R;
  const int ld = n + 1;
  const int c = blockIdx.x;
  const int p = warp;
  const int bt = c * 2 + p;

  // per-warp carve-up (every float2 array starts on an 8-byte boundary)
  const size_t per_warp_floats = topk_warp_floats(n, a.B);
  float *base = reinterpret_cast<float *>(smem) + warp * per_warp_floats;
  float2 *A = reinterpret_cast<float2 *>(base);  // n x ld
  float2 *vb = A + n * ld;                       // reflector
  float2 *pb = vb + n;                           // A v work vector
  float2 *taus = pb + n;                         // reflector scalars
  float2 *z = taus + n;                          // one back-transformed vector
  float *X = reinterpret_cast<float *>(z + n);   // top-K vectors of T (real), K x n
  float *U0 = X + ((n * n + 1) & ~1);            // LU workspace, GROUP x n each
  float *U1 = U0 + GROUP * n;
  float *U2 = U1 + GROUP * n;
  float *ML = U2 + GROUP * n;
  float *PV = ML + GROUP * n;
  float2 *Wp = reinterpret_cast<float2 *>(PV + GROUP * n);  // projected weights B x n
  float *d = reinterpret_cast<float *>(Wp + a.B * n);
  float *e = d + n;
  float *e2 = e + n;
  float *lam = e2 + n;
  float *sd = lam + n;

  const float2 *dp = a.factors + ((size_t)c * 2 + p) * n;

  // ---- 1. covariance (upper triangle, Hermitian completion), whitening ----
  for (int i = lane; i < n; i += 32) {
    const int32_t *v = a.vis + ((((size_t)c * a.NBL + baseline_of(i, i)) * 2 + p) * 2 + p) * 2;
    float2 x = make_float2(static_cast<float>(v[0]), static_cast<float>(v[1]));
    x = cmulc(cmul(dp[i], x), dp[i]);
    sd[i] = sqrtf(fmaxf(x.x, 1e-10f));
  }
  __syncwarp();
  for (int e0 = lane; e0 < n * n; e0 += 32) {
    const int i = e0 / n, j = e0 - (e0 / n) * n;
    const int lo = min(i, j), hi = max(i, j);
    const int32_t *v = a.vis + ((((size_t)c * a.NBL + baseline_of(lo, hi)) * 2 + p) * 2 + p) * 2;
    float2 x = make_float2(static_cast<float>(v[0]), static_cast<float>(v[1]));
    x = cmulc(cmul(dp[lo], x), dp[hi]);
    const float den = sd[i] * sd[j];
    float2 val;
    if (i == j) val = make_float2(x.x / den, 0.0f);
    else if (i < j) val = make_float2(x.x / den, x.y / den);
    else val = make_float2(x.x / den, -x.y / den);
    A[i * ld + j] = val;
  }
  __syncwarp();

  // ---- 2. Householder tridiagonalisation (lower), T = Q^H A Q ----
  for (int k = 0; k < n - 1; ++k) {
    const int m = n - k - 1;  // length of the reflector
    const float2 alpha = A[(k + 1) * ld + k];
    float part = 0.0f;
    for (int i = 1 + lane; i < m; i += 32) {
      const float2 x = A[(k + 1 + i) * ld + k];
      part += x.x * x.x + x.y * x.y;
    }
    const float xnorm2 = warp_sum(part);
    float2 tau = make_float2(0.0f, 0.0f);
    float beta = alpha.x;
    if (!(xnorm2 == 0.0f && alpha.y == 0.0f)) {
      const float nrm = sqrtf(alpha.x * alpha.x + alpha.y * alpha.y + xnorm2);
      beta = alpha.x >= 0.0f ? -nrm : nrm;
      tau = make_float2((beta - alpha.x) / beta, -alpha.y / beta);
      // scale = 1 / (alpha - beta)
      const float2 am = make_float2(alpha.x - beta, alpha.y);
      const float inv = 1.0f / (am.x * am.x + am.y * am.y);
      const float2 sc = make_float2(am.x * inv, -am.y * inv);
      for (int i = 1 + lane; i < m; i += 32) A[(k + 1 + i) * ld + k] = cmul(A[(k + 1 + i) * ld + k], sc);
    }
    __syncwarp();
    for (int i = lane; i < m; i += 32) vb[i] = i == 0 ? make_float2(1.0f, 0.0f) : A[(k + 1 + i) * ld + k];
    if (lane == 0) {
      taus[k] = tau;
      e[k] = beta;
    }
    __syncwarp();
    if (tau.x != 0.0f || tau.y != 0.0f) {
      // p = tau A22 v
      float dre = 0.0f, dim = 0.0f;
      for (int i = lane; i < m; i += 32) {
        const float2 *row = A + (k + 1 + i) * ld + (k + 1);
        float2 acc = make_float2(0.0f, 0.0f);
        for (int j = 0; j < m; ++j) {
          const float2 t = cmul(row[j], vb[j]);
          acc.x += t.x;
          acc.y += t.y;
        }
        const float2 pi = cmul(tau, acc);
        pb[i] = pi;
        // (p^H v)_i = conj(p_i) v_i
        const float2 t = cmulc(vb[i], pi);
        dre += t.x;
        dim += t.y;
      }
      dre = warp_sum(dre);
      dim = warp_sum(dim);
      // alpha' = -1/2 tau (p^H v)
      const float2 al = cmul(make_float2(-0.5f * tau.x, -0.5f * tau.y), make_float2(dre, dim));
      __syncwarp();
      for (int i = lane; i < m; i += 32) {
        const float2 t = cmul(al, vb[i]);
        pb[i] = make_float2(pb[i].x + t.x, pb[i].y + t.y);
      }
      __syncwarp();
      // A22 -= v p^H + p v^H
      for (int i = lane; i < m; i += 32) {
        float2 *row = A + (k + 1 + i) * ld + (k + 1);
        const float2 vi = vb[i], pi = pb[i];
        for (int j = 0; j < m; ++j) {
          const float2 t1 = cmulc(vi, pb[j]);
          const float2 t2 = cmulc(pi, vb[j]);
          row[j] = make_float2(row[j].x - t1.x - t2.x, row[j].y - t1.y - t2.y);
        }
      }
    }
    __syncwarp();
  }
  for (int i = lane; i < n; i += 32) d[i] = A[i * ld + i].x;
  if (lane == 0) e[n - 1] = 0.0f;
  __syncwarp();
  for (int i = lane; i < n; i += 32) e2[i] = e[i] * e[i];
  __syncwarp();

  // ---- 3. eigenvalues by bisection (Gershgorin bracket) ----
  float glo = 3.0e38f, ghi = -3.0e38f, emax = 0.0f;
  for (int i = lane; i < n; i += 32) {
    const float r = fabsf(e[i]) + (i > 0 ? fabsf(e[i - 1]) : 0.0f);
    glo = fminf(glo, d[i] - r);
    ghi = fmaxf(ghi, d[i] + r);
    emax = fmaxf(emax, e2[i]);
  }
  glo = warp_min(glo);
  ghi = warp_max(ghi);
  emax = warp_max(emax);
  const float tnorm = fmaxf(fabsf(glo), fabsf(ghi));
  const float pivmin = fmaxf(1e-30f, 1e-30f * emax);
  glo -= 2e-7f * tnorm + pivmin;
  ghi += 2e-7f * tnorm + pivmin;
  for (int j = lane; j < n; j += 32) {
    float lo = glo, hi = ghi;
    // absolute tolerance ~ float epsilon x ||T||, the accuracy any backward-
    // stable solver reaches (and what detection and the shifts need)
    const float atol = 2.4e-7f * tnorm + 4.0f * pivmin;
    for (int it = 0; it < 64; ++it) {
      const float mid = 0.5f * (lo + hi);
      if (hi - lo <= atol || mid == lo || mid == hi) break;
      if (sturm_count(d, e2, n, mid, pivmin) > j) hi = mid;
      else lo = mid;
    }
    lam[j] = 0.5f * (lo + hi);
  }
  __syncwarp();
  if (a.evals)
    for (int j = lane; j < n; j += 32) a.evals[(size_t)bt * n + j] = lam[j];

  // ---- 4. K ----
  int K = 0;
  if (a.k_rule == SF_K_DETECT) {
    const float p20 = percentile_sorted(lam, n, 0.2f);
    const float p50 = percentile_sorted(lam, n, 0.5f);
    const float p80 = percentile_sorted(lam, n, 0.8f);
    const float sigma = (p80 - p20) / (2.0f * 0.8416f);
    const float thr = p50 + a.delta * sigma;
    for (int i = 0; i < n; ++i) K += lam[i] > thr;
  } else if (a.k_rule == SF_K_NOISE_FLOOR) {
    const float med = 0.5f * (lam[(n - 1) / 2] + lam[n / 2]);
    for (int i = 0; i < n; ++i) K += lam[i] > a.delta * med;
  } else {
    K = a.fixed_counts ? a.fixed_counts[c] : 0;
  }
  K = max(0, min(n, K));
  if (a.counts && lane == 0) a.counts[bt] = K;

  // ---- 5. top-K eigenvectors of T: inverse iteration + MGS ----
  const float pert = 2.4e-7f * tnorm + pivmin;
  for (int g0 = 0; g0 < K; g0 += GROUP) {
    const int gn = min(GROUP, K - g0);
    // vector r = g0 + lane (lane < gn) belongs to eigenvalue n-1-r
    for (int it = 0; it < INV_ITERS; ++it) {
      if (lane < gn) {
        const int r = g0 + lane;
        float *x = X + r * n;
        float *u0 = U0 + lane * n, *u1 = U1 + lane * n, *u2 = U2 + lane * n, *ml = ML + lane * n,
              *pv = PV + lane * n;
        const float shift = lam[n - 1 - r];
        if (it == 0)
          for (int i = 0; i < n; ++i) x[i] = 1.0f + 0.37f * sinf(0.91f * (i + 1) * (r + 1));
        // LU of (T - shift I) with partial pivoting, applied to x on the fly
        float cd = d[0] - shift, cs = n > 1 ? e[0] : 0.0f;
        for (int i = 0; i < n - 1; ++i) {
          const float sub = e[i];
          const float nd = d[i + 1] - shift;
          const float ns = (i + 1 < n - 1) ? e[i + 1] : 0.0f;
          if (fabsf(cd) >= fabsf(sub)) {
            const float piv = cd == 0.0f ? pert : cd;
            const float l = sub / piv;
            u0[i] = piv;
            u1[i] = cs;
            u2[i] = 0.0f;
            pv[i] = 0.0f;
            ml[i] = l;
            x[i + 1] -= l * x[i];
            cd = nd - l * cs;
            cs = ns;
          } else {
            const float l = cd / sub;
            u0[i] = sub;
            u1[i] = nd;
            u2[i] = ns;
            pv[i] = 1.0f;
            ml[i] = l;
            const float t = x[i];
            x[i] = x[i + 1];
            x[i + 1] = t - l * x[i];
            cd = cs - l * nd;
            cs = -l * ns;
          }
        }
        u0[n - 1] = (fabsf(cd) < pert) ? (cd < 0.0f ? -pert : pert) : cd;
        // back substitution
        x[n - 1] = x[n - 1] / u0[n - 1];
        if (n > 1) x[n - 2] = (x[n - 2] - u1[n - 2] * x[n - 1]) / (fabsf(u0[n - 2]) < pert ? pert : u0[n - 2]);
        for (int i = n - 3; i >= 0; --i) {
          const float piv = fabsf(u0[i]) < pert ? pert : u0[i];
          x[i] = (x[i] - u1[i] * x[i + 1] - u2[i] * x[i + 2]) / piv;
        }
        float s2 = 0.0f;
        for (int i = 0; i < n; ++i) s2 += x[i] * x[i];
        const float inv = s2 > 0.0f ? rsqrtf(s2) : 0.0f;
        for (int i = 0; i < n; ++i) x[i] *= inv;
      }
      __syncwarp();
      // modified Gram-Schmidt of this group's vectors against all earlier ones
      for (int r = g0; r < g0 + gn; ++r) {
        float *x = X + r * n;
        for (int q = 0; q < r; ++q) {
          const float *y = X + q * n;
          float part = 0.0f;
          for (int i = lane; i < n; i += 32) part += x[i] * y[i];
          const float dot = warp_sum(part);
          for (int i = lane; i < n; i += 32) x[i] -= dot * y[i];
          __syncwarp();
        }
        float part = 0.0f;
        for (int i = lane; i < n; i += 32) part += x[i] * x[i];
        const float nrm2 = warp_sum(part);
        const float inv = nrm2 > 0.0f ? rsqrtf(nrm2) : 0.0f;
        for (int i = lane; i < n; i += 32) x[i] *= inv;
        __syncwarp();
      }
    }
  }

  // ---- 6. weights: slot 0 = W diag(d); slot 1 = (W - sum_k w_k (W u_k) u_k^H) diag(d) ----
  const __half2 *w = a.weights + ((size_t)c * 2 + p) * a.B * n;
  for (int e0 = lane; e0 < a.B * n; e0 += 32) Wp[e0] = __half22float2(w[e0]);
  float lam_bar = 0.0f;
  if (a.shrink && K < n) {
    for (int i = 0; i < n - K; ++i) lam_bar += lam[i];
    lam_bar /= static_cast<float>(n - K);
  }
  __syncwarp();
  for (int r = 0; r < K; ++r) {
    // z = Q x: apply the reflectors from the last to the first
    const float *x = X + r * n;
    for (int i = lane; i < n; i += 32) z[i] = make_float2(x[i], 0.0f);
    __syncwarp();
    for (int k = n - 2; k >= 0; --k) {
      const int m = n - k - 1;
      const float2 tau = taus[k];
      if (tau.x == 0.0f && tau.y == 0.0f) continue;
      float dre = 0.0f, dim = 0.0f;
      for (int i = lane; i < m; i += 32) {
        const float2 v = i == 0 ? make_float2(1.0f, 0.0f) : A[(k + 1 + i) * ld + k];
        const float2 t = cmulc(z[k + 1 + i], v);  // conj(v) z
        dre += t.x;
        dim += t.y;
      }
      dre = warp_sum(dre);
      dim = warp_sum(dim);
      const float2 s = cmul(tau, make_float2(dre, dim));
      __syncwarp();
      for (int i = lane; i < m; i += 32) {
        const float2 v = i == 0 ? make_float2(1.0f, 0.0f) : A[(k + 1 + i) * ld + k];
        const float2 t = cmul(s, v);
        z[k + 1 + i] = make_float2(z[k + 1 + i].x - t.x, z[k + 1 + i].y - t.y);
      }
      __syncwarp();
    }
    float wgt = 1.0f;
    if (a.shrink) {
      const float lk = lam[n - 1 - r];
      wgt = 1.0f - (lk > 0.0f ? lam_bar / lk : 0.0f);
    } else {
      // un-whiten and normalise
      float part = 0.0f;
      for (int i = lane; i < n; i += 32) {
        const float2 t = make_float2(z[i].x * sd[i], z[i].y * sd[i]);
        z[i] = t;
        part += t.x * t.x + t.y * t.y;
      }
      const float nrm2 = warp_sum(part);
      const float inv = nrm2 > 0.0f ? rsqrtf(nrm2) : 0.0f;
      for (int i = lane; i < n; i += 32) z[i] = make_float2(z[i].x * inv, z[i].y * inv);
    }
    __syncwarp();
    // P acts on the original weights: Wp_m -= wgt (W_m . z) conj(z)
    for (int m = 0; m < a.B; ++m) {
      float cre = 0.0f, cim = 0.0f;
      for (int i = lane; i < n; i += 32) {
        const float2 t = cmul(__half22float2(w[m * n + i]), z[i]);
        cre += t.x;
        cim += t.y;
      }
      cre = warp_sum(cre);
      cim = warp_sum(cim);
      const float2 cm = make_float2(wgt * cre, wgt * cim);
      for (int i = lane; i < n; i += 32) {
        const float2 t = cmulc(cm, z[i]);  // c_m conj(z_i)
        Wp[m * n + i] = make_float2(Wp[m * n + i].x - t.x, Wp[m * n + i].y - t.y);
      }
    }
    __syncwarp();
  }
  float2 *we = a.weff + ((size_t)c * 2 + p) * 2 * a.B * n;
  for (int e0 = lane; e0 < a.B * n; e0 += 32) {
    const int col = e0 - (e0 / n) * n;
    we[e0] = cmul(__half22float2(w[e0]), dp[col]);
    we[a.B * n + e0] = cmul(Wp[e0], dp[col]);
  }
}

}  // namespace

size_t sf_eig_topk_smem(int n, int B) { return WARPS * topk_warp_floats(n, B) * sizeof(float); }

int sf_eig_topk_supported(const sf_plan *p) { return p->R <= MAX_N && sf_eig_topk_smem(p->R, p->B) <= 200 * 1024; }

cudaError_t sf_launch_eig_topk(const sf_plan *p, const int32_t *vis, int k_rule, float delta, int shrink,
                               float *evals, int32_t *counts, cudaStream_t stream) {
  TopkArgs a;
  a.vis = vis;
  a.factors = p->d_factors;
  a.weights = p->d_weights;
  a.fixed_counts = p->d_fixed_counts;
  a.evals = evals;
  a.counts = counts;
  a.weff = p->d_weff;
  a.status = p->d_status;
  a.C = p->C;
  a.R = p->R;
  a.B = p->B;
  a.NBL = p->NBL;
  a.k_rule = k_rule;
  a.shrink = shrink;
  a.delta = delta;
  const size_t smem = sf_eig_topk_smem(p->R, p->B);
  static int attr_done = 0;
  if (!attr_done) {
    cudaError_t e = cudaFuncSetAttribute(sf_eig_topk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         200 * 1024);
    if (e != cudaSuccess) return e;
    attr_done = 1;
  }
  sf_eig_topk_kernel<<<p->C, WARPS * 32, smem, stream>>>(a);
  return cudaGetLastError();
}
