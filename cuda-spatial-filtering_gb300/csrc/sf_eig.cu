// Covariance -> Hermitian eigendecomposition -> K -> RFI projection -> beam
// weights, one CTA per (channel, pol[, pol]) matrix held in shared memory.
//
// Replaces, for the reference's batched path:
//   unpack_triangular_baseline_batch     include/spatial/spatial.cuh:672-713
//   diagonalWhiten / unwhitenEigenvectors include/spatial/spatial.cuh:1065-1148
//   cusolverDnXsyevBatched               lambda_gpu_pipeline.hpp:494-501,
//                                        lambda_adaptive_beamformed_spectra_pipeline.hpp:679-686
//   detectSignalEigenmodeCounts          include/spatial/spatial.cuh:900-950
//   buildIdentityMinusProjection / shrink include/spatial/spatial.cuh:952-1063
//   ccglib weight projection W' = W P    lambda_adaptive_beamformed_spectra_pipeline.hpp:773-794
//
// Eigensolver: parallel cyclic Jacobi for complex Hermitian matrices.  Each
// step applies n/2 disjoint 2x2 unitary rotations chosen by a round-robin
// tournament; every 2x2 block of A is updated by one thread as J_a^H B J_b,
// so a step is two barriers.  Sweeps stop when no off-diagonal element is
// above max(1e-7 sqrt|a_pp a_qq|, 1e-9 ||A||_F); eigenvalues come out in
// ascending order with eigenvectors in columns (the cuSOLVER contract), each
// vector's largest component made real and positive.
#include <cstdio>

#include "sf_common.cuh"
#include "sf_plan.cuh"

namespace {

constexpr int EIG_THREADS = 256;
constexpr int MAX_N = 64;
constexpr int MAX_SWEEPS = 30;

struct EigArgs {
  const int32_t *vis;
  const float2 *factors;   // [C][2][R]
  const __half2 *weights;  // [C][2][B][R]
  const int32_t *fixed_counts;
  float *evals;
  float2 *evecs;
  int32_t *counts;
  __half2 *proj;
  float2 *weff;  // [C][2][2B][R]
  uint32_t *status;
  int C, R, B, NBL;
  int mode, k_rule, shrink;
  float delta;
};

struct Rot {
  float c, s;
  float2 z;   // e^{-i phi}
  float tw;   // t |w|: diagonal shift
  int on;
};

__device__ __forceinline__ void pair_of(int step, int k, int np, int &a, int &b) {
  const int m1 = np - 1;
  if (k == 0) {
    a = 0;
    b = 1 + (step % m1);
  } else {
    a = 1 + ((step + k) % m1);
    b = 1 + ((step - k + m1 * 4) % m1);
  }
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

__global__ void __launch_bounds__(EIG_THREADS) sf_eig_kernel(const EigArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int n = a.R;
  const int np = (n + 1) & ~1;
  const int h = np / 2;
  const int ld = np + 1;
  float2 *A = reinterpret_cast<float2 *>(smem);  // [np][ld]
  float2 *V = A + np * ld;                       // [np][ld]
  Rot *rot = reinterpret_cast<Rot *>(V + np * ld);
  float *sd = reinterpret_cast<float *>(rot + h);  // whitening sqrt-diagonal
  float *lam = sd + np;                            // sorted eigenvalues
  int *order = reinterpret_cast<int *>(lam + np);  // order[rank] = column
  __shared__ int s_rotations, s_k;
  __shared__ float s_frob2;

  const int tid = threadIdx.x;
  const int bt = blockIdx.x;
  int c, p, q;
  if (a.mode == SF_EIG_ALL_BLOCKS) {
    c = bt >> 2;
    p = (bt >> 1) & 1;
    q = bt & 1;
  } else {
    c = bt >> 1;
    p = q = bt & 1;
  }
  const float2 *dp = a.factors + ((size_t)c * 2 + p) * n;
  const float2 *dq = a.factors + ((size_t)c * 2 + q) * n;

  // ---- covariance from the packed upper triangle (uplo = upper) ----
  if (tid == 0) s_frob2 = 0.0f;
  for (int e = tid; e < np * np; e += EIG_THREADS) {
    const int i = e / np, j = e - (e / np) * np;
    float2 val = make_float2(0.0f, 0.0f);
    if (i < n && j < n) {
      const int lo = min(i, j), hi = max(i, j);
      const int32_t *v = a.vis + ((((size_t)c * a.NBL + baseline_of(lo, hi)) * 2 + p) * 2 + q) * 2;
      float2 x = make_float2(static_cast<float>(v[0]), static_cast<float>(v[1]));
      x = cmulc(cmul(dp[lo], x), dq[hi]);  // d_i conj(d_j) V(i,j)
      if (i == j) val = make_float2(x.x, 0.0f);
      else if (i < j) val = x;
      else val = make_float2(x.x, -x.y);
    }
    A[i * ld + j] = val;
    V[i * ld + j] = make_float2(i == j ? 1.0f : 0.0f, 0.0f);
  }
  __syncthreads();

  const bool whitened = a.mode == SF_EIG_SAME_POL_WHITENED;
  if (whitened) {
    for (int i = tid; i < np; i += EIG_THREADS)
      sd[i] = i < n ? sqrtf(fmaxf(A[i * ld + i].x, 1e-10f)) : 1.0f;
    __syncthreads();
    for (int e = tid; e < n * n; e += EIG_THREADS) {
      const int i = e / n, j = e - (e / n) * n;
      const float den = sd[i] * sd[j];
      float2 x = A[i * ld + j];
      A[i * ld + j] = make_float2(x.x / den, x.y / den);
    }
    __syncthreads();
  }
  {
    float part = 0.0f;
    for (int e = tid; e < np * np; e += EIG_THREADS) {
      const float2 x = A[(e / np) * ld + (e % np)];
      part += x.x * x.x + x.y * x.y;
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((tid & 31) == 0) atomicAdd(&s_frob2, part);
  }
  __syncthreads();
  const float abs_tol = 1e-9f * sqrtf(s_frob2);

  // ---- parallel cyclic Jacobi ----
  bool converged = (np < 2);
  for (int sweep = 0; sweep < MAX_SWEEPS && !converged; ++sweep) {
    if (tid == 0) s_rotations = 0;
    __syncthreads();
    for (int step = 0; step < np - 1; ++step) {
      if (tid < h) {
        int ia, ib;
        pair_of(step, tid, np, ia, ib);
        const float app = A[ia * ld + ia].x;
        const float aqq = A[ib * ld + ib].x;
        const float2 w = A[ia * ld + ib];
        const float aw = sqrtf(w.x * w.x + w.y * w.y);
        Rot r;
        r.c = 1.0f;
        r.s = 0.0f;
        r.z = make_float2(1.0f, 0.0f);
        r.tw = 0.0f;
        r.on = 0;
        if (aw > fmaxf(1e-7f * sqrtf(fabsf(app * aqq)), abs_tol)) {
          const float theta = (aqq - app) / (2.0f * aw);
          float t;
          if (fabsf(theta) > 1e18f) t = 0.5f / theta;
          else t = copysignf(1.0f, theta) / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
          r.c = rsqrtf(t * t + 1.0f);
          r.s = t * r.c;
          r.z = make_float2(w.x / aw, -w.y / aw);
          r.tw = t * aw;
          r.on = 1;
          atomicAdd(&s_rotations, 1);
        }
        rot[tid] = r;
      }
      __syncthreads();
      // 2x2 blocks of A: B <- J_a^H B J_b
      for (int blk = tid; blk < h * h; blk += EIG_THREADS) {
        const int ka = blk / h, kb = blk - (blk / h) * h;
        const Rot ra = rot[ka], rb = rot[kb];
        if (!ra.on && !rb.on) continue;
        int a0, a1, b0, b1;
        pair_of(step, ka, np, a0, a1);
        pair_of(step, kb, np, b0, b1);
        if (ka == kb) {
          A[a0 * ld + a0] = make_float2(A[a0 * ld + a0].x - ra.tw, 0.0f);
          A[a1 * ld + a1] = make_float2(A[a1 * ld + a1].x + ra.tw, 0.0f);
          A[a0 * ld + a1] = make_float2(0.0f, 0.0f);
          A[a1 * ld + a0] = make_float2(0.0f, 0.0f);
          continue;
        }
        float2 x00 = A[a0 * ld + b0], x01 = A[a0 * ld + b1];
        float2 x10 = A[a1 * ld + b0], x11 = A[a1 * ld + b1];
        if (rb.on) {  // columns: (x0, x1) -> (c x0 - s z x1, s x0 + c z x1)
          const float2 zb = rb.z;
          float2 t0 = cmul(zb, x01), t1 = cmul(zb, x11);
          float2 n00 = make_float2(rb.c * x00.x - rb.s * t0.x, rb.c * x00.y - rb.s * t0.y);
          float2 n01 = make_float2(rb.s * x00.x + rb.c * t0.x, rb.s * x00.y + rb.c * t0.y);
          float2 n10 = make_float2(rb.c * x10.x - rb.s * t1.x, rb.c * x10.y - rb.s * t1.y);
          float2 n11 = make_float2(rb.s * x10.x + rb.c * t1.x, rb.s * x10.y + rb.c * t1.y);
          x00 = n00; x01 = n01; x10 = n10; x11 = n11;
        }
        if (ra.on) {  // rows: (y0, y1) -> (c y0 - s conj(z) y1, s y0 + c conj(z) y1)
          const float2 za = make_float2(ra.z.x, -ra.z.y);
          float2 t0 = cmul(za, x10), t1 = cmul(za, x11);
          float2 n00 = make_float2(ra.c * x00.x - ra.s * t0.x, ra.c * x00.y - ra.s * t0.y);
          float2 n10 = make_float2(ra.s * x00.x + ra.c * t0.x, ra.s * x00.y + ra.c * t0.y);
          float2 n01 = make_float2(ra.c * x01.x - ra.s * t1.x, ra.c * x01.y - ra.s * t1.y);
          float2 n11 = make_float2(ra.s * x01.x + ra.c * t1.x, ra.s * x01.y + ra.c * t1.y);
          x00 = n00; x01 = n01; x10 = n10; x11 = n11;
        }
        A[a0 * ld + b0] = x00;
        A[a0 * ld + b1] = x01;
        A[a1 * ld + b0] = x10;
        A[a1 * ld + b1] = x11;
      }
      // eigenvectors: V <- V J
      for (int e = tid; e < np * h; e += EIG_THREADS) {
        const int row = e / h, k = e - (e / h) * h;
        const Rot r = rot[k];
        if (!r.on) continue;
        int c0, c1;
        pair_of(step, k, np, c0, c1);
        const float2 v0 = V[row * ld + c0], v1 = V[row * ld + c1];
        const float2 t = cmul(r.z, v1);
        V[row * ld + c0] = make_float2(r.c * v0.x - r.s * t.x, r.c * v0.y - r.s * t.y);
        V[row * ld + c1] = make_float2(r.s * v0.x + r.c * t.x, r.s * v0.y + r.c * t.y);
      }
      __syncthreads();
    }
    converged = (s_rotations == 0);
    __syncthreads();
  }
  if (!converged && tid == 0) atomicOr(a.status, SF_DEVERR_EIG_NOT_CONVERGED);

  // ---- ascending order (ties by index) ----
  for (int i = tid; i < n; i += EIG_THREADS) {
    const float li = A[i * ld + i].x;
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const float lj = A[j * ld + j].x;
      rank += (lj < li) || (lj == li && j < i);
    }
    lam[rank] = li;
    order[rank] = i;
  }
  __syncthreads();

  const bool null_mode = whitened && !a.shrink;
  // Un-whiten and re-normalise every column (null mode), as the reference's
  // unwhitenAndNormalizeKernel does before building I - U U^H.
  if (null_mode) {
    for (int e = tid; e < n * n; e += EIG_THREADS) {
      const int row = e / n, col = e - (e / n) * n;
      const float2 x = V[row * ld + col];
      V[row * ld + col] = make_float2(x.x * sd[row], x.y * sd[row]);
    }
    __syncthreads();
    for (int col = tid; col < n; col += EIG_THREADS) {
      float s2 = 0.0f;
      for (int row = 0; row < n; ++row) {
        const float2 x = V[row * ld + col];
        s2 += x.x * x.x + x.y * x.y;
      }
      const float inv = s2 > 0.0f ? rsqrtf(s2) : 0.0f;
      for (int row = 0; row < n; ++row) {
        const float2 x = V[row * ld + col];
        V[row * ld + col] = make_float2(x.x * inv, x.y * inv);
      }
    }
    __syncthreads();
  }
  // Phase convention: the largest-magnitude component (lowest index on ties)
  // of each eigenvector is made real and positive.
  for (int col = tid; col < n; col += EIG_THREADS) {
    int best = 0;
    float bm = -1.0f;
    for (int row = 0; row < n; ++row) {
      const float2 x = V[row * ld + col];
      const float m2 = x.x * x.x + x.y * x.y;
      if (m2 > bm) {
        bm = m2;
        best = row;
      }
    }
    const float2 piv = V[best * ld + col];
    const float mag = sqrtf(bm);
    if (mag > 0.0f) {
      const float2 ph = make_float2(piv.x / mag, -piv.y / mag);
      for (int row = 0; row < n; ++row) V[row * ld + col] = cmul(V[row * ld + col], ph);
    }
  }
  __syncthreads();

  if (a.evals)
    for (int k = tid; k < n; k += EIG_THREADS) a.evals[(size_t)bt * n + k] = lam[k];
  if (a.evecs)
    for (int e = tid; e < n * n; e += EIG_THREADS) {
      const int k = e / n, l = e - (e / n) * n;
      a.evecs[(size_t)bt * n * n + e] = V[l * ld + order[k]];
    }
  if (!whitened) return;

  // ---- K ----
  if (tid == 0) {
    int k = 0;
    if (a.k_rule == SF_K_DETECT) {
      const float p20 = percentile_sorted(lam, n, 0.2f);
      const float p50 = percentile_sorted(lam, n, 0.5f);
      const float p80 = percentile_sorted(lam, n, 0.8f);
      const float sigma = (p80 - p20) / (2.0f * 0.8416f);
      const float thr = p50 + a.delta * sigma;
      for (int i = 0; i < n; ++i) k += lam[i] > thr;
    } else if (a.k_rule == SF_K_NOISE_FLOOR) {
      const float med = 0.5f * (lam[(n - 1) / 2] + lam[n / 2]);
      for (int i = 0; i < n; ++i) k += lam[i] > a.delta * med;
    } else {
      k = a.fixed_counts ? a.fixed_counts[c] : 0;
    }
    s_k = max(0, min(n, k));
    if (a.counts) a.counts[bt] = s_k;
  }
  __syncthreads();
  const int K = s_k;

  // ---- projector P (reuses A): null I - sum U_k U_k^H over the top K,
  //      shrink I - sum (1 - d_k) V_k V_k^H with d_k = mean(kept)/lambda_k ----
  float lam_bar = 0.0f;
  if (a.shrink && K < n) {
    for (int i = 0; i < n - K; ++i) lam_bar += lam[i];
    lam_bar /= static_cast<float>(n - K);
  }
  for (int e = tid; e < n * n; e += EIG_THREADS) {
    const int row = e / n, col = e - (e / n) * n;
    float2 acc = make_float2(row == col ? 1.0f : 0.0f, 0.0f);
    for (int r = n - K; r < n; ++r) {
      const int kc = order[r];
      float wgt = 1.0f;
      if (a.shrink) {
        const float lk = lam[r];
        const float dk = lk > 0.0f ? lam_bar / lk : 0.0f;
        wgt = 1.0f - dk;
      }
      const float2 t = cmulc(V[row * ld + kc], V[col * ld + kc]);
      acc.x -= wgt * t.x;
      acc.y -= wgt * t.y;
    }
    A[row * ld + col] = acc;
  }
  __syncthreads();
  if (a.proj)
    for (int e = tid; e < n * n; e += EIG_THREADS) {
      const int col = e / n, row = e - (e / n) * n;  // column-major (row + col * n)
      a.proj[((size_t)c * 2 + p) * n * n + e] = __float22half2_rn(A[row * ld + col]);
    }

  // ---- effective weights: slot 0 = W diag(d), slot 1 = (W P) diag(d) ----
  const __half2 *w = a.weights + ((size_t)c * 2 + p) * a.B * n;
  float2 *we = a.weff + ((size_t)c * 2 + p) * 2 * a.B * n;
  for (int e = tid; e < a.B * n; e += EIG_THREADS) {
    const int m = e / n, col = e - (e / n) * n;
    const float2 wc = __half22float2(w[m * n + col]);
    we[m * n + col] = cmul(wc, dp[col]);
    float2 acc = make_float2(0.0f, 0.0f);
    for (int l = 0; l < n; ++l) {
      const float2 t = cmul(__half22float2(w[m * n + l]), A[l * ld + col]);
      acc.x += t.x;
      acc.y += t.y;
    }
    we[(a.B + m) * n + col] = cmul(acc, dp[col]);
  }
}

}  // namespace

int sf_eig_supported(const sf_plan *p, char *why, size_t why_len) {
  if (p->R > MAX_N) {
    if (why && why_len) snprintf(why, why_len, "eigensolver supports at most %d receivers", MAX_N);
    return 0;
  }
  return 1;
}

cudaError_t sf_launch_eig(const sf_plan *p, const int32_t *vis, int eig_mode, int k_rule,
                          float delta, int shrink, float *evals, float2 *evecs, int32_t *counts,
                          __half2 *proj, cudaStream_t stream) {
  // The adaptive path needs only eigenvalues and the top-K eigenvectors:
  // the tridiagonal solvers serve it unless every eigenvector (or the
  // projector itself) is asked for -- sf_eig_small.cu up to 128 receivers and
  // 16 beams, else sf_eig_topk.cu.
  if (eig_mode == SF_EIG_SAME_POL_WHITENED && evecs == nullptr && proj == nullptr) {
    if (sf_eig_small_supported(p))
      return sf_launch_eig_small(p, vis, k_rule, delta, shrink, evals, counts, nullptr, nullptr, stream);
    if (sf_eig_topk_supported(p))
      return sf_launch_eig_topk(p, vis, k_rule, delta, shrink, evals, counts, stream);
  }
  EigArgs a;
  a.vis = vis;
  a.factors = p->d_factors;
  a.weights = p->d_weights;
  a.fixed_counts = p->d_fixed_counts;
  a.evals = evals;
  a.evecs = evecs;
  a.counts = counts;
  a.proj = proj;
  a.weff = p->d_weff;
  a.status = p->d_status;
  a.C = p->C;
  a.R = p->R;
  a.B = p->B;
  a.NBL = p->NBL;
  a.mode = eig_mode;
  a.k_rule = k_rule;
  a.shrink = shrink;
  a.delta = delta;
  const int np = (p->R + 1) & ~1;
  const size_t smem = (size_t)2 * np * (np + 1) * sizeof(float2) + (size_t)(np / 2) * sizeof(Rot) +
                      (size_t)np * (2 * sizeof(float) + sizeof(int));
  cudaError_t e = sf_smem_optin(reinterpret_cast<const void *>(sf_eig_kernel), smem);
  if (e != cudaSuccess) return e;
  const int batch = eig_mode == SF_EIG_ALL_BLOCKS ? p->C * 4 : p->C * 2;
  sf_eig_kernel<<<batch, EIG_THREADS, smem, stream>>>(a);
  return cudaGetLastError();
}
