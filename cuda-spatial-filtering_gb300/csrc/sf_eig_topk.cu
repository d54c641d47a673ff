// Adaptive-path eigensolver: one CTA (four warps) per (channel, pol)
// covariance, the top-K eigenvectors only (what K selection, I - U U^H and the
// projected weights need) and every eigenvalue only when the K rule, shrink
// mode or the caller needs them.  Used when the caller asks for no
// eigenvector output; the full Jacobi solver (sf_eig.cu) serves the rest.
//
// Per matrix, in shared memory:
//   1. covariance d_i conj(d_j) V(i,j) from the packed int32 upper triangle,
//      diagonal whitening (reference include/spatial/spatial.cuh:1068-1093)
//   2. Householder reduction to a real symmetric tridiagonal T = Q^H A Q
//      (the published LAPACK zhetd2/zlarfg algorithm: reflectors
//      H = I - tau v v^H, subdiagonal made real); the matrix-vector product
//      and the rank-2 update are spread over the CTA
//   3. eigenvalues from Sturm counts: every eigenvalue by 4-way multisection
//      (three lanes each), or only the top K by 33-way multisection (one warp each)
//   4. K (fixed, percentile rule of spatial.cuh:900-950, or noise floor)
//   5. the top-K eigenvectors of T by inverse iteration (LU with partial
//      pivoting, three iterations, modified Gram-Schmidt among them)
//   6. back-transformed through the reflectors (one warp per vector),
//      un-whitened and normalised (spatial.cuh:1098-1126)
//   7. effective weights: slot 0 W diag(d), slot 1 (W P) diag(d) with
//      P = I - sum_k w_k u_k u_k^H (null: w = 1 on the un-whitened u;
//      shrink: w = 1 - lambda_bar / lambda_k on the whitened v).
#include <cstdio>
#include <cstring>

#include "sf_common.cuh"
#include "sf_plan.cuh"

namespace {

constexpr int NT_PLAN = 128;  // threads per matrix on the plan path (six CTAs per SM)
constexpr int MAX_N = 128;   // shared-memory working matrix
constexpr int MAX_N_GLOBAL = 256;  // working matrix in global scratch
constexpr int GROUP = 8;  // inverse-iteration vectors solved at once (one lane of warp 0 each)
constexpr int INV_ITERS = 3;
constexpr int MAX_B = 16;  // beams per pol handled by the projection step
constexpr int MAX_XK = 64;  // eigenvectors of T held at once (K is clamped to this; n <= 64 holds all)

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
  // Batched form (uneven sub-arrays): matrix blockIdx.x is items[first_item + blockIdx.x],
  // with its own size and offsets into the arrays above; NULL for the plan's uniform layout.
  const SfEigItem *items;
  int first_item;
  // Fallback form: the plan-layout matrices list[0 .. *list_count) (device-side count),
  // walked grid-stride; NULL otherwise.
  const int32_t *list;
  const int32_t *list_count;
  // matrices of the launch when CTAs walk them grid-stride (0: one per CTA)
  int n_items;
  // Large matrices: the n x (n+1) working matrix lives in this global scratch
  // (one region of a_ld floats2 per CTA) instead of shared memory.
  float2 *gA;
  long long a_ld;
  // Vectors out: the top-K un-whitened, normalised eigenvectors are written
  // to u_out + (item u_off, or matrix x xk x n) + k n instead of projecting
  // weights (B = 0).
  float2 *u_out;
};

// rows of the eigenvector workspace X for an n x n matrix
__host__ __device__ inline int topk_xk(int n) { return n < MAX_XK ? n : MAX_XK; }

__host__ __device__ inline size_t topk_floats(int n, int B, int NW, bool a_in_smem = true) {
  // float2: A (n x (n+1), unless in global scratch), 2 v, p, tau, Z (NW x n), Wp (B x n), W0 (B x n),
  //         coef (NW x B)
  // float:  X (xk x n), LU workspace (5 GROUP x n), d, e, e2, lam, sd
  const size_t f2 = (a_in_smem ? (size_t)n * (n + 1) : 0) + 4 * (size_t)n + (size_t)NW * n + 2 * (size_t)B * n +
                    (size_t)NW * B;
  const size_t f = (size_t)topk_xk(n) * n + 5 * (size_t)GROUP * n + 5 * (size_t)n;
  return ((2 * f2 + f) + 3) & ~(size_t)3;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// Two independent sums reduced together (their shuffles overlap).
__device__ __forceinline__ void warp_sum2(float &a, float &b) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float ta = __shfl_xor_sync(0xffffffffu, a, o);
    const float tb = __shfl_xor_sync(0xffffffffu, b, o);
    a += ta;
    b += tb;
  }
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
  // unrolled so that the loads of d and e2 run ahead of the recurrence
#pragma unroll 4
  for (int i = 1; i < n; ++i) {
    q = d[i] - x - __fdividef(e2[i - 1], q);
    if (fabsf(q) < pivmin) q = -pivmin;
    cnt += q < 0.0f;
  }
  return cnt;
}

// Reflector of column k (one warp): H = I - tau v v^H with H^H x = beta e_1 for
// x = A[k+1.., k] (LAPACK zlarfg); v (v_0 = 1) is stored below the subdiagonal
// of column k and in vbuf[(k & 1) n ..], tau in taus[k], beta in e[k].
__device__ __forceinline__ void make_reflector(float2 *A, int ld, int n, int k, float2 *vbuf, float2 *taus,
                                               float *e, int lane) {
  const int m = n - k - 1;
  const float2 alpha = A[(k + 1) * ld + k];
  float part = 0.0f;
  for (int i = 1 + lane; i < m; i += 32) {
    const float2 x = A[(k + 1 + i) * ld + k];
    part += x.x * x.x + x.y * x.y;
  }
  const float xnorm2 = warp_sum(part);
  float2 tau = make_float2(0.0f, 0.0f);
  float beta = alpha.x;
  float2 *vb = vbuf + (k & 1) * n;
  if (!(xnorm2 == 0.0f && alpha.y == 0.0f)) {
    const float nrm = sqrtf(alpha.x * alpha.x + alpha.y * alpha.y + xnorm2);
    beta = alpha.x >= 0.0f ? -nrm : nrm;
    const float rb = __frcp_rn(beta);  // == 1.0f / beta, without the division's slow path
    tau = make_float2((beta - alpha.x) * rb, -alpha.y * rb);
    // scale = 1 / (alpha - beta)
    const float2 am = make_float2(alpha.x - beta, alpha.y);
    const float inv = __frcp_rn(am.x * am.x + am.y * am.y);
    const float2 sc = make_float2(am.x * inv, -am.y * inv);
    for (int i = 1 + lane; i < m; i += 32) {
      const float2 v = cmul(A[(k + 1 + i) * ld + k], sc);
      A[(k + 1 + i) * ld + k] = v;
      vb[i] = v;
    }
  } else {
    for (int i = 1 + lane; i < m; i += 32) vb[i] = A[(k + 1 + i) * ld + k];
  }
  if (lane == 0) {
    vb[0] = make_float2(1.0f, 0.0f);
    taus[k] = tau;
    e[k] = beta;
  }
}

// NPL: matrix rows per lane in the register-resident steps (n <= 32 NPL);
// NTT: threads per matrix.
template <int NPL, int NTT>
__global__ void __launch_bounds__(NTT, NTT <= 128 ? (NPL <= 2 ? 6 : 1) : 1) sf_eig_topk_kernel(const TopkArgs a) {
  constexpr int NT = NTT;
  constexpr int NW = NTT / 32;
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ float s_red[4 * NW];
  __shared__ float s_scal[8];
  __shared__ int s_K;
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane = tid & 31;
  const int B = a.B;
  const int count = a.list ? *a.list_count : (a.n_items > 0 ? a.n_items : static_cast<int>(gridDim.x));
  for (int mi = blockIdx.x; mi < count; mi += gridDim.x) {
  if (mi != static_cast<int>(blockIdx.x)) __syncthreads();  // the previous matrix's shared memory is free
  // this matrix: size, packed upper triangle (baseline (i,j) at entry baseline_of(i,j), each entry
  // [Pol][Pol][2] int32), receiver factors, weights [B][n], outputs
  int n, pol, fixedK;
  long long uoff;
  const int32_t *visb;
  const float2 *dp;
  const __half2 *w;
  float2 *we;
  float *ev_out;
  int32_t *cnt_out;
  if (a.items) {
    const SfEigItem it = a.items[a.first_item + mi];
    n = it.n;
    pol = it.pol;
    visb = a.vis + it.vis_off;
    dp = a.factors ? a.factors + it.factor_off : nullptr;
    w = a.weights + it.weight_off;
    we = a.weff ? a.weff + it.weff_off : nullptr;
    uoff = it.u_off;
    ev_out = a.evals ? a.evals + it.eval_off : nullptr;
    cnt_out = a.counts ? a.counts + it.count_idx : nullptr;
    fixedK = a.fixed_counts ? a.fixed_counts[it.count_idx] : 0;
  } else {
    const int bt = a.list ? a.list[mi] : mi;  // c * 2 + p
    const int c = bt >> 1;
    n = a.R;
    pol = bt & 1;
    visb = a.vis + (size_t)c * a.NBL * 8;
    dp = a.factors + (size_t)bt * n;
    w = a.weights + (size_t)bt * B * n;
    we = a.weff ? a.weff + (size_t)bt * 2 * B * n : nullptr;
    uoff = (long long)bt * topk_xk(n) * n;
    ev_out = a.evals ? a.evals + (size_t)bt * n : nullptr;
    cnt_out = a.counts ? a.counts + bt : nullptr;
    fixedK = a.fixed_counts ? a.fixed_counts[c] : 0;
  }
  const int ld = n + 1;
  const int xk = topk_xk(n);

  float2 *A = a.gA ? a.gA + (size_t)blockIdx.x * a.a_ld : reinterpret_cast<float2 *>(smem);  // n x ld
  float2 *vbuf = a.gA ? reinterpret_cast<float2 *>(smem) : A + n * ld;  // reflectors k (even / odd k)
  float2 *pb = vbuf + 2 * n;                     // tau A v
  float2 *taus = pb + n;                         // reflector scalars
  float2 *Z = taus + n;                          // NW back-transformed vectors
  float2 *Wp = Z + NW * n;                       // projected weights B x n
  float2 *W0 = Wp + B * n;                       // the original weights B x n
  float2 *coef = W0 + B * n;                     // NW x B projection coefficients
  float *X = reinterpret_cast<float *>(coef + NW * B);  // top-K vectors of T, K x n
  float *U0 = X + xk * n;                        // LU workspace, GROUP x n each
  float *U1 = U0 + GROUP * n;
  float *U2 = U1 + GROUP * n;
  float *ML = U2 + GROUP * n;
  float *PV = ML + GROUP * n;
  float *d = PV + GROUP * n;
  float *e = d + n;
  float *e2 = e + n;
  float *lam = e2 + n;
  float *sd = lam + n;

  const int p = pol;
  auto factor = [&](int i) { return dp ? dp[i] : make_float2(1.0f, 0.0f); };

  // ---- 1. covariance (upper triangle, Hermitian completion), whitening ----
  for (int i = tid; i < n; i += NT) {
    const int32_t *v = visb + (((size_t)baseline_of(i, i) * 2 + p) * 2 + p) * 2;
    float2 x = make_float2(static_cast<float>(v[0]), static_cast<float>(v[1]));
    x = cmulc(cmul(factor(i), x), factor(i));
    sd[i] = sqrtf(fmaxf(x.x, 1e-10f));
  }
  __syncthreads();
  // both triangles (A[i][j] and A[j][i] = conj(A[i][j])), so that the
  // Householder matrix-vector product reads plain rows
  for (int e0 = tid; e0 < n * n; e0 += NT) {
    const int i = e0 / n, j = e0 - (e0 / n) * n;
    if (j > i) continue;
    const int32_t *v = visb + (((size_t)baseline_of(j, i) * 2 + p) * 2 + p) * 2;
    float2 x = make_float2(static_cast<float>(v[0]), static_cast<float>(v[1]));
    x = cmulc(cmul(factor(j), x), factor(i));  // element (j, i) of the upper triangle
    const float inv = 1.0f / (sd[i] * sd[j]);
    A[i * ld + j] = i == j ? make_float2(x.x * inv, 0.0f) : make_float2(x.x * inv, -x.y * inv);
    if (j < i) A[j * ld + i] = make_float2(x.x * inv, x.y * inv);
  }
  __syncthreads();

  // ---- 2. Householder tridiagonalisation (lower), T = Q^H A Q ----
  // Step k: p = tau A22 v (all threads); then warp 0 applies the rank-2 update
  // to the first column of A22 and at once forms reflector k+1 from it, while
  // warps 1.. update the rest: two block barriers per step.
  if (warp == 0 && n > 1) make_reflector(A, ld, n, 0, vbuf, taus, e, lane);
  __syncthreads();
  for (int k = 0; k < n - 1; ++k) {
    const int m = n - k - 1;  // length of the reflector
    const float2 *vb = vbuf + (k & 1) * n;
    const float2 tau = taus[k];
    float2 *A22 = A + (k + 1) * ld + (k + 1);
    if (tau.x != 0.0f || tau.y != 0.0f) {
      // p = tau A22 v, A22 Hermitian held in both triangles: two threads per
      // row, even / odd columns
      const int h = tid & 1;
      float dre = 0.0f, dim = 0.0f;
      for (int i = tid >> 1; i - (tid >> 1) < m; i += NT / 2) {  // uniform trip count per warp
      float2 acc0 = make_float2(0.0f, 0.0f), acc1 = make_float2(0.0f, 0.0f);
      if (i < m) {
        // four loads in flight before their products
        const float2 *rowp = A22 + i * ld;
        int j = h;
        for (; j + 6 < m; j += 8) {
          float2 x[4], vv[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int jj = j + 2 * u;
            x[u] = rowp[jj];
            vv[u] = vb[jj];
          }
#pragma unroll
          for (int u = 0; u < 4; u += 2) {
            const float2 t0 = cmul(x[u], vv[u]);
            const float2 t1 = cmul(x[u + 1], vv[u + 1]);
            acc0.x += t0.x;
            acc0.y += t0.y;
            acc1.x += t1.x;
            acc1.y += t1.y;
          }
        }
        for (; j < m; j += 2) {
          const float2 t0 = cmul(rowp[j], vb[j]);
          acc0.x += t0.x;
          acc0.y += t0.y;
        }
      }
      float2 acc = make_float2(acc0.x + acc1.x, acc0.y + acc1.y);
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, 1);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, 1);
      if (i < m && h == 0) {
        const float2 pi = cmul(tau, acc);
        pb[i] = pi;
        const float2 t = cmulc(vb[i], pi);  // conj(p_i) v_i
        dre += t.x;
        dim += t.y;
      }
      }
      warp_sum2(dre, dim);
      if (lane == 0) {
        s_red[(k & 1) * 2 * NW + warp] = dre;
        s_red[(k & 1) * 2 * NW + NW + warp] = dim;
      }
      __syncthreads();
      // alpha' = -1/2 tau (p^H v);  A22 -= v p^H + p v^H + 2 Re(alpha') v v^H
      float Dre = 0.0f, Dim = 0.0f;
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        Dre += s_red[(k & 1) * 2 * NW + w];
        Dim += s_red[(k & 1) * 2 * NW + NW + w];
      }
      const float cvv = 2.0f * (-0.5f * (tau.x * Dre - tau.y * Dim));
      if (warp == 0) {
        // column 0 of A22 updated in registers (rows lane, lane + 32), and
        // reflector k+1 formed from it at once (LAPACK zlarfg): alpha is row 1,
        // x the rows below
        const float2 v0 = vb[0], p0 = pb[0];
        float2 col[NPL];
        float part = 0.0f;
#pragma unroll
        for (int t = 0; t < NPL; ++t) {
          const int ii = lane + 32 * t;
          col[t] = make_float2(0.0f, 0.0f);
          if (ii < m) {
            const float2 vi = vb[ii], pi = pb[ii];
            const float2 t1 = cmulc(vi, p0);
            const float2 t2 = cmulc(pi, v0);
            const float2 t3 = cmulc(vi, v0);
            const float2 old = A22[ii * ld];
            col[t] = make_float2(old.x - t1.x - t2.x - cvv * t3.x, old.y - t1.y - t2.y - cvv * t3.y);
            if (ii >= 2) part += col[t].x * col[t].x + col[t].y * col[t].y;
          }
        }
        const float2 alpha = make_float2(__shfl_sync(0xffffffffu, col[0].x, 1), __shfl_sync(0xffffffffu, col[0].y, 1));
        const float xnorm2 = warp_sum(part);
        if (lane < 2 && lane < m) A22[lane * ld] = col[0];  // diagonal element and alpha
        if (k + 1 < n - 1) {
          float2 tau1 = make_float2(0.0f, 0.0f);
          float beta = alpha.x;
          float2 sc = make_float2(1.0f, 0.0f);
          const bool nonzero = !(xnorm2 == 0.0f && alpha.y == 0.0f);
          if (nonzero) {
            const float nrm = sqrtf(alpha.x * alpha.x + alpha.y * alpha.y + xnorm2);
            beta = alpha.x >= 0.0f ? -nrm : nrm;
            const float rb = __frcp_rn(beta);
            tau1 = make_float2((beta - alpha.x) * rb, -alpha.y * rb);
            const float2 am = make_float2(alpha.x - beta, alpha.y);  // scale = 1 / (alpha - beta)
            const float inv = __frcp_rn(am.x * am.x + am.y * am.y);
            sc = make_float2(am.x * inv, -am.y * inv);
          }
          float2 *vn = vbuf + ((k + 1) & 1) * n;
#pragma unroll
          for (int t = 0; t < NPL; ++t) {
            const int ii = lane + 32 * t;
            if (ii >= 2 && ii < m) {
              const float2 v = nonzero ? cmul(col[t], sc) : col[t];
              A22[ii * ld] = v;
              vn[ii - 1] = v;
            }
          }
          if (lane == 0) {
            vn[0] = make_float2(1.0f, 0.0f);
            taus[k + 1] = tau1;
            e[k + 1] = beta;
          }
        } else {
#pragma unroll
          for (int t = 0; t < NPL; ++t) {
            const int ii = lane + 32 * t;
            if (ii >= 2 && ii < m) A22[ii * ld] = col[t];
          }
        }
      } else {
        // rows 1..m-1 of A22, columns 1..row: rows i and m-i (i and m-i
        // elements) share one pass of a warp
        for (int r = warp - 1; r < m / 2; r += NW - 1) {
          const int ia = r + 1, ib = m - 1 - r;
          const int ntot = ia == ib ? ia : m;
          for (int q = lane; q < ntot; q += 32) {
            const int ii = q < ia ? ia : ib;
            const int jj = q < ia ? q + 1 : q - ia + 1;
            const float2 vi = vb[ii], pi = pb[ii], vj = vb[jj], pj = pb[jj];
            const float2 t1 = cmulc(vi, pj);
            const float2 t2 = cmulc(pi, vj);
            const float2 t3 = cmulc(vi, vj);
            float2 *el = A22 + ii * ld + jj;
            const float2 old = *el;
            const float2 nw = make_float2(old.x - t1.x - t2.x - cvv * t3.x, old.y - t1.y - t2.y - cvv * t3.y);
            *el = nw;
            if (jj != ii) A22[jj * ld + ii] = make_float2(nw.x, -nw.y);  // the upper triangle
          }
        }
      }
    } else if (warp == 0 && k + 1 < n - 1) {
      make_reflector(A, ld, n, k + 1, vbuf, taus, e, lane);
    }
    __syncthreads();
  }
  for (int i = tid; i < n; i += NT) {
    d[i] = A[i * ld + i].x;
    if (i == n - 1) e[i] = 0.0f;
  }
  __syncthreads();
  for (int i = tid; i < n; i += NT) e2[i] = e[i] * e[i];
  // K of the fixed rule is known before any eigenvalue
  const bool need_all = a.k_rule != SF_K_FIXED || ev_out != nullptr || a.shrink;
  int Kfix = 0;
  if (!need_all) Kfix = max(0, min(xk, fixedK));
  __syncthreads();

  // ---- 3. eigenvalues (Gershgorin bracket) ----
  if (warp == 0) {
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
    if (lane == 0) {
      s_scal[2] = glo - (2e-7f * tnorm + pivmin);
      s_scal[3] = ghi + (2e-7f * tnorm + pivmin);
      s_scal[4] = tnorm;
      s_scal[5] = pivmin;
    }
  }
  __syncthreads();
  const float glo = s_scal[2], ghi = s_scal[3], tnorm = s_scal[4], pivmin = s_scal[5];
  // absolute tolerance ~ float epsilon x ||T||, the accuracy any backward-
  // stable solver reaches (and what detection and the shifts need)
  const float atol = 2.4e-7f * tnorm + 4.0f * pivmin;
  if (need_all) {
    // every eigenvalue by 4-way multisection, three lanes each (lanes 3 s ..
    // 3 s + 2 of a warp, s < 10), each lane counting at one interior point:
    // two bits of the bracket per Sturm count instead of bisection's one
    const int slot = lane / 3, sub = lane - 3 * slot;
    for (int j0 = 0; j0 < n; j0 += 10 * NW) {
      const int j = j0 + warp * 10 + slot;
      const bool mine = slot < 10 && j < n;
      float lo = glo, hi = ghi;
      bool done = !mine;
      for (int it = 0; it < 64; ++it) {
        if (__all_sync(0xffffffffu, done)) break;
        const float step = (hi - lo) * 0.25f;
        const float x = lo + step * static_cast<float>(sub + 1);
        const bool above = !done && sturm_count(d, e2, n, x, pivmin) > j;
        // eigenvalue j lies in [x_{f-1}, x_f), f = first point with more than j below it
        const unsigned grp = (__ballot_sync(0xffffffffu, above) >> (3 * min(slot, 9))) & 7u;
        if (!done) {
          const int f = grp ? __ffs(grp) - 1 : 3;
          const float nlo = f == 0 ? lo : lo + step * static_cast<float>(f);
          const float nhi = f == 3 ? hi : lo + step * static_cast<float>(f + 1);
          done = !(step > 0.0f) || (nlo == lo && nhi == hi) || nhi - nlo <= atol;
          lo = nlo;
          hi = nhi;
        }
      }
      if (mine && sub == 0) lam[j] = 0.5f * (lo + hi);
    }
  } else {
    // the top K only, one warp each: 33-way multisection (32 interior points)
    for (int r = warp; r < Kfix; r += NW) {
      const int j = n - 1 - r;
      float lo = glo, hi = ghi;
      for (int it = 0; it < 16; ++it) {
        if (hi - lo <= atol) break;
        const float step = (hi - lo) * (1.0f / 33.0f);
        if (!(step > 0.0f)) break;
        const float x = lo + step * static_cast<float>(lane + 1);
        const unsigned above = __ballot_sync(0xffffffffu, sturm_count(d, e2, n, x, pivmin) > j);
        // eigenvalue j lies in (x_{f-1}, x_f], f = first point with more than j below it
        const int f = above ? __ffs(above) - 1 : 32;
        const float nlo = f == 0 ? lo : lo + step * static_cast<float>(f);
        const float nhi = f == 32 ? hi : lo + step * static_cast<float>(f + 1);
        lo = nlo;
        hi = nhi;
      }
      if (lane == 0) lam[j] = 0.5f * (lo + hi);
    }
  }
  __syncthreads();
  if (ev_out)
    for (int j = tid; j < n; j += NT) ev_out[j] = lam[j];

  // ---- 4. K ----
  if (tid == 0) {
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
      K = fixedK;
    }
    K = max(0, min(n, K));
    if (K > xk) {  // more modes than the eigenvector workspace holds: null the top xk
      atomicOr(a.status, SF_DEVERR_BAD_SHAPE);
      K = xk;
    }
    s_K = K;
    if (cnt_out) *cnt_out = K;
  }
  __syncthreads();
  const int K = s_K;

  // ---- 5. top-K eigenvectors of T: inverse iteration + MGS (warp 0) ----
  if (warp == 0) {
    const float pert = 2.4e-7f * tnorm + pivmin;
    for (int g0 = 0; g0 < K; g0 += GROUP) {
      const int gn = min(GROUP, K - g0);
      // vector r = g0 + lane (lane < gn) belongs to eigenvalue n-1-r
      float *u0 = U0 + lane * n, *u1 = U1 + lane * n, *u2 = U2 + lane * n, *ml = ML + lane * n,
            *pv = PV + lane * n;
      if (lane < gn) {
        // LU of (T - shift I) with partial pivoting, once; u0 holds 1 / pivot
        const int r = g0 + lane;
        const float shift = lam[n - 1 - r];
        float cd = d[0] - shift, cs = n > 1 ? e[0] : 0.0f;
#pragma unroll 4
        for (int i = 0; i < n - 1; ++i) {
          const float sub = e[i];
          const float nd = d[i + 1] - shift;
          const float ns = (i + 1 < n - 1) ? e[i + 1] : 0.0f;
          if (fabsf(cd) >= fabsf(sub)) {
            const float piv = fabsf(cd) < pert ? (cd < 0.0f ? -pert : pert) : cd;
            const float rp = __frcp_rn(piv);
            const float l = sub * rp;
            u0[i] = rp;
            u1[i] = cs;
            u2[i] = 0.0f;
            pv[i] = 0.0f;
            ml[i] = l;
            cd = nd - l * cs;
            cs = ns;
          } else {
            const float rs = __frcp_rn(fabsf(sub) < pert ? pert : sub);
            const float l = cd * rs;
            u0[i] = rs;
            u1[i] = nd;
            u2[i] = ns;
            pv[i] = 1.0f;
            ml[i] = l;
            cd = cs - l * nd;
            cs = -l * ns;
          }
        }
        u0[n - 1] = __frcp_rn((fabsf(cd) < pert) ? (cd < 0.0f ? -pert : pert) : cd);
        float *x = X + r * n;
        // a fixed pseudo-random start in [0.5, 1.5): no eigenvector is orthogonal to it
        for (int i = 0; i < n; ++i) {
          const uint32_t hsh = (static_cast<uint32_t>(i + 1) * 2654435761u) ^ (static_cast<uint32_t>(r + 1) * 2246822519u);
          x[i] = 0.5f + static_cast<float>((hsh >> 8) & 0xFFFFu) * (1.0f / 65536.0f);
        }
      }
      for (int it = 0; it < INV_ITERS; ++it) {
        if (lane < gn) {
          const int r = g0 + lane;
          float *x = X + r * n;
          // forward: the row interchanges and multipliers of the factorisation
          // (the running value stays in a register)
          float cur = x[0];
#pragma unroll 4
          for (int i = 0; i < n - 1; ++i) {
            float nxt = x[i + 1];
            if (pv[i] != 0.0f) {
              const float t = cur;
              cur = nxt;
              nxt = t;
            }
            x[i] = cur;
            cur = nxt - ml[i] * cur;
          }
          x[n - 1] = cur;
          // back substitution, x[i+1] and x[i+2] carried in registers
          float x1 = x[n - 1] * u0[n - 1];
          x[n - 1] = x1;
          float x2 = 0.0f;
          if (n > 1) {
            const float v = (x[n - 2] - u1[n - 2] * x1) * u0[n - 2];
            x[n - 2] = v;
            x2 = x1;
            x1 = v;
          }
#pragma unroll 4
          for (int i = n - 3; i >= 0; --i) {
            const float v = (x[i] - u1[i] * x1 - u2[i] * x2) * u0[i];
            x[i] = v;
            x2 = x1;
            x1 = v;
          }
          // no normalisation here: the Gram-Schmidt pass below normalises
          // (one solve grows a unit vector by at most about 1 / pert, far
          // inside the float range)
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
  }

  // ---- 6./7. back-transform (one warp per vector), projected weights ----
  for (int e0 = tid; e0 < B * n; e0 += NT) {
    const float2 x = __half22float2(w[e0]);
    Wp[e0] = x;
    W0[e0] = x;
  }
  float lam_bar = 0.0f;
  if (a.shrink && K < n) {
    for (int i = 0; i < n - K; ++i) lam_bar += lam[i];
    lam_bar /= static_cast<float>(n - K);
  }
  __syncthreads();
  for (int g = 0; g < K; g += NW) {
    const int r = g + warp;
    float2 *z = Z + warp * n;
    if (r < K) {
      // z = Q x: the reflectors from the last to the first, z in registers
      // (lane holds elements lane and lane + 32, n <= 64); reflector k's v is 1
      // at k + 1, A[j][k] below it, 0 above
      const float *x = X + r * n;
      float2 zz[NPL];
#pragma unroll
      for (int t = 0; t < NPL; ++t) {
        const int ii = lane + 32 * t;
        zz[t] = make_float2(ii < n ? x[ii] : 0.0f, 0.0f);
      }
      for (int k = n - 2; k >= 0; --k) {
        const float2 tau = taus[k];
        float2 vv[NPL];
        float dre = 0.0f, dim = 0.0f;  // conj(v) z
#pragma unroll
        for (int t = 0; t < NPL; ++t) {
          const int ii = lane + 32 * t;
          vv[t] = ii > k + 1 && ii < n ? A[ii * ld + k] : make_float2(ii == k + 1 ? 1.0f : 0.0f, 0.0f);
          dre += vv[t].x * zz[t].x + vv[t].y * zz[t].y;
          dim += vv[t].x * zz[t].y - vv[t].y * zz[t].x;
        }
        warp_sum2(dre, dim);
        const float2 sc = cmul(tau, make_float2(dre, dim));
#pragma unroll
        for (int t = 0; t < NPL; ++t)
          zz[t] = make_float2(zz[t].x - (sc.x * vv[t].x - sc.y * vv[t].y), zz[t].y - (sc.x * vv[t].y + sc.y * vv[t].x));
      }
      float wgt = 1.0f;
      if (a.shrink) {
        const float lk = lam[n - 1 - r];
        wgt = 1.0f - (lk > 0.0f ? lam_bar / lk : 0.0f);
      } else {
        // un-whiten and normalise
        float part = 0.0f;
#pragma unroll
        for (int t = 0; t < NPL; ++t) {
          const int ii = lane + 32 * t;
          const float si = ii < n ? sd[ii] : 0.0f;
          zz[t] = make_float2(zz[t].x * si, zz[t].y * si);
          part += zz[t].x * zz[t].x + zz[t].y * zz[t].y;
        }
        const float nrm2 = warp_sum(part);
        const float inv = nrm2 > 0.0f ? rsqrtf(nrm2) : 0.0f;
#pragma unroll
        for (int t = 0; t < NPL; ++t) zz[t] = make_float2(zz[t].x * inv, zz[t].y * inv);
      }
#pragma unroll
      for (int t = 0; t < NPL; ++t)
        if (lane + 32 * t < n) {
          z[lane + 32 * t] = zz[t];
          if (a.u_out) a.u_out[uoff + (long long)r * n + lane + 32 * t] = zz[t];
        }
      // c_m = wgt (W_m . z) against the original weights: all partial sums
      // first, then the reductions
      {
        float cre[MAX_B], cim[MAX_B];
#pragma unroll
        for (int mm = 0; mm < MAX_B; ++mm) {
          cre[mm] = 0.0f;
          cim[mm] = 0.0f;
          if (mm < B) {
#pragma unroll
            for (int t = 0; t < NPL; ++t) {
              const int ii = lane + 32 * t;
              const float2 wa = ii < n ? W0[mm * n + ii] : make_float2(0.0f, 0.0f);
              cre[mm] += wa.x * zz[t].x - wa.y * zz[t].y;
              cim[mm] += wa.x * zz[t].y + wa.y * zz[t].x;
            }
          }
        }
#pragma unroll
        for (int mm = 0; mm < MAX_B; ++mm) {
          if (mm < B) {
            warp_sum2(cre[mm], cim[mm]);
            if (lane == 0) coef[warp * B + mm] = make_float2(wgt * cre[mm], wgt * cim[mm]);
          }
        }
      }
    }
    __syncthreads();
    // P acts on the original weights: Wp_m -= sum_r c_m,r conj(z_r)
    const int gv = min(NW, K - g);
    for (int e0 = tid; e0 < B * n; e0 += NT) {
      const int mm = e0 / n, i = e0 - (e0 / n) * n;
      float2 acc = Wp[e0];
      for (int q = 0; q < gv; ++q) {
        const float2 t = cmulc(coef[q * B + mm], Z[q * n + i]);  // c conj(z_i)
        acc.x -= t.x;
        acc.y -= t.y;
      }
      Wp[e0] = acc;
    }
    __syncthreads();
  }
  if (we)
    for (int e0 = tid; e0 < B * n; e0 += NT) {
      const int col = e0 - (e0 / n) * n;
      we[e0] = cmul(W0[e0], factor(col));
      we[B * n + e0] = cmul(Wp[e0], factor(col));
    }
  }  // matrices of this CTA
}

}  // namespace

size_t sf_eig_topk_smem(int n, int B) { return topk_floats(n, B, NT_PLAN / 32) * sizeof(float); }

int sf_eig_topk_supported(const sf_plan *p) {
  return p->R <= 64 && p->B <= MAX_B && sf_eig_topk_smem(p->R, p->B) <= 200 * 1024;
}

int sf_eig_topk_max_n() { return MAX_N; }

// Shared memory of one matrix of at most n_max receivers in the batched form
// (the launch picks 128 / 256 / 512 threads for n_max <= 32 / 64 / 128).
size_t sf_eig_topk_items_smem(int n_max, int B) {
  const int nw = n_max <= 32 ? 4 : (n_max <= 64 ? 8 : 16);
  return topk_floats(n_max, B, nw) * sizeof(float);
}
int sf_eig_topk_max_b() { return MAX_B; }

cudaError_t sf_launch_eig_topk_items(const SfEigItem *items, int first, int count, int n_max, int B,
                                     const int32_t *vis, const float2 *factors, const __half2 *weights,
                                     const int32_t *fixed_counts, int k_rule, float delta, int shrink, float *evals,
                                     int32_t *counts, float2 *weff, uint32_t *status, cudaStream_t stream) {
  if (count <= 0) return cudaSuccess;
  if (n_max > MAX_N || B > MAX_B) return cudaErrorInvalidValue;
  TopkArgs a;
  a.vis = vis;
  a.factors = factors;
  a.weights = weights;
  a.fixed_counts = fixed_counts;
  a.evals = evals;
  a.counts = counts;
  a.weff = weff;
  a.status = status;
  a.C = 0;
  a.R = n_max;
  a.B = B;
  a.NBL = 0;
  a.k_rule = k_rule;
  a.shrink = shrink;
  a.delta = delta;
  a.items = items;
  a.first_item = first;
  a.list = nullptr;
  a.list_count = nullptr;
  a.n_items = 0;
  a.gA = nullptr;
  a.a_ld = 0;
  a.u_out = nullptr;
  // large matrices take more threads: the rank-2 update is spread over all warps but one
  cudaError_t e;
  if (n_max <= 32) {
    const size_t smem = topk_floats(n_max, B, 4) * sizeof(float);
    e = sf_smem_optin(reinterpret_cast<const void *>(sf_eig_topk_kernel<1, 128>), smem);
    if (e != cudaSuccess) return e;
    sf_eig_topk_kernel<1, 128><<<count, 128, smem, stream>>>(a);
  } else if (n_max <= 64) {
    const size_t smem = topk_floats(n_max, B, 8) * sizeof(float);
    e = sf_smem_optin(reinterpret_cast<const void *>(sf_eig_topk_kernel<2, 256>), smem);
    if (e != cudaSuccess) return e;
    sf_eig_topk_kernel<2, 256><<<count, 256, smem, stream>>>(a);
  } else {
    const size_t smem = topk_floats(n_max, B, 16) * sizeof(float);
    e = sf_smem_optin(reinterpret_cast<const void *>(sf_eig_topk_kernel<4, 512>), smem);
    if (e != cudaSuccess) return e;
    sf_eig_topk_kernel<4, 512><<<count, 512, smem, stream>>>(a);
  }
  return cudaGetLastError();
}

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
  a.items = nullptr;
  a.first_item = 0;
  a.list = nullptr;
  a.list_count = nullptr;
  a.n_items = 0;
  a.gA = nullptr;
  a.a_ld = 0;
  a.u_out = nullptr;
  const size_t smem = sf_eig_topk_smem(p->R, p->B);
  cudaError_t e = sf_smem_optin(reinterpret_cast<const void *>(sf_eig_topk_kernel<2, NT_PLAN>), smem);
  if (e != cudaSuccess) return e;
  sf_eig_topk_kernel<2, NT_PLAN><<<p->C * 2, NT_PLAN, smem, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t sf_launch_eig_topk_list(const sf_plan *p, const int32_t *vis, const int32_t *list, const int32_t *list_count,
                                    int max_count, int k_rule, float delta, int shrink, float *evals, int32_t *counts,
                                    cudaStream_t stream) {
  if (max_count <= 0) return cudaSuccess;
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
  a.items = nullptr;
  a.first_item = 0;
  a.list = list;
  a.list_count = list_count;
  a.n_items = 0;
  a.gA = nullptr;
  a.a_ld = 0;
  a.u_out = nullptr;
  const size_t smem = sf_eig_topk_smem(p->R, p->B);
  cudaError_t e = sf_smem_optin(reinterpret_cast<const void *>(sf_eig_topk_kernel<2, NT_PLAN>), smem);
  if (e != cudaSuccess) return e;
  const int grid = max_count < 6 * p->num_sms ? max_count : 6 * p->num_sms;
  sf_eig_topk_kernel<2, NT_PLAN><<<grid, NT_PLAN, smem, stream>>>(a);
  return cudaGetLastError();
}

// Eigenvectors out, for matrices of up to 256 receivers (the working matrix in
// global scratch above 128): per item the top-K un-whitened normalised
// eigenvectors at u_out + item.u_off, K at counts, eigenvalues at evals;
// no weight projection.  scratch holds min(count, grid) x n_max x (n_max + 1)
// float2; returns the grid used (<= max_grid).
cudaError_t sf_launch_eig_topk_vectors(const SfEigItem *items, int first, int count, int n_max, const int32_t *vis,
                                       const int32_t *fixed_counts, int k_rule, float delta, float *evals,
                                       int32_t *counts, float2 *u_out, float2 *scratch, int max_grid,
                                       uint32_t *status, cudaStream_t stream) {
  if (count <= 0) return cudaSuccess;
  if (n_max > MAX_N_GLOBAL) return cudaErrorInvalidValue;
  TopkArgs a;
  memset(&a, 0, sizeof(a));
  a.vis = vis;
  a.fixed_counts = fixed_counts;
  a.evals = evals;
  a.counts = counts;
  a.status = status;
  a.R = n_max;
  a.B = 0;
  a.k_rule = k_rule;
  a.delta = delta;
  a.items = items;
  a.first_item = first;
  a.u_out = u_out;
  cudaError_t e;
  if (n_max <= 128) {
    const size_t smem = topk_floats(n_max, 0, 16) * sizeof(float);
    e = sf_smem_optin(reinterpret_cast<const void *>(sf_eig_topk_kernel<4, 512>), smem);
    if (e != cudaSuccess) return e;
    sf_eig_topk_kernel<4, 512><<<count, 512, smem, stream>>>(a);
  } else {
    const int grid = count < max_grid ? count : max_grid;
    a.gA = scratch;
    a.a_ld = (long long)n_max * (n_max + 1);
    a.n_items = count;
    const size_t smem = topk_floats(n_max, 0, 16, false) * sizeof(float);
    e = sf_smem_optin(reinterpret_cast<const void *>(sf_eig_topk_kernel<8, 512>), smem);
    if (e != cudaSuccess) return e;
    sf_eig_topk_kernel<8, 512><<<grid, 512, smem, stream>>>(a);
  }
  return cudaGetLastError();
}
