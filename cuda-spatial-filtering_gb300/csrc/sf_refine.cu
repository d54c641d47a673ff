// FP64 Rayleigh-quotient refinement of the nulled subspace and FP64
// re-projection of the beam weights (the precision form of the batched
// chain).
//
// Input per (unit, pol) matrix: the exact int32 visibilities and the FP32
// eigensolver's top-K eigenvectors u_k (un-whitened, normalised).  In FP64:
//   v_k = normalise(D^{-1/2} u_k)                   (back to the whitened problem)
//   `steps` times: X = A V, V <- orth(X) (modified Gram-Schmidt), then
//   Rayleigh-Ritz: H = V^H A V (K x K, cyclic Jacobi), V <- V Y, theta = diag
//   residuals max_k ||A v_k - theta_k v_k|| / theta_max before and after
//   u_k = D^{1/2} v_k; Q = orth(U) (orthogonal re-projection) or the u_k
//   normalised one by one (the reference's I - U U^H convention);
//   W' = W - sum_k (W q_k) q_k^H
// A = D^{-1/2} V D^{-1/2} is formed on the fly from the int32 visibilities
// (exact in FP64).  Effective weights are stored in FP32 for the beamformer:
// slot 0 = W, slot 1 = W'.  No counterpart in the reference, whose nulling
// is FP32 cuSOLVER vectors into an fp16 projector
// (lambda_adaptive_beamformed_spectra_pipeline.hpp:679-757).
#include <cstdio>

#include "sf_common.cuh"
#include "sf_plan.cuh"

namespace {

constexpr int RF_THREADS = 256;
constexpr int RF_KMAX = 8;   // refined vectors per matrix (K is clamped to this)
constexpr int RF_NMAX = 256;

struct RefineArgs {
  const int32_t *vis;
  const SfEigItem *items;   // weff_off: effective weights out [2B][n]; u_off: the FP32 vectors
  const float2 *u32;        // FP32 vectors: item i at u32 + item.u_off, vector k at + k n
  const int32_t *counts;    // K per matrix (count_idx)
  const __half2 *weights;   // [B][n] at item.weight_off
  float2 *weff;
  double *ritz;             // [item][RF_KMAX] (may be NULL)
  float *resid;             // [item][2] residual before / after (may be NULL)
  uint32_t *status;
  int B, steps, orthogonal;
};

struct dcplx {
  double x, y;
};
__device__ __forceinline__ dcplx dmul(dcplx a, dcplx b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ dcplx dmulc(dcplx a, dcplx b) { return {a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y}; }

__device__ __forceinline__ double block_sum(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < RF_THREADS / 32; ++i) s += red[i];
  return s;
}

__global__ void __launch_bounds__(RF_THREADS) sf_refine64_kernel(const RefineArgs a) {
  extern __shared__ __align__(16) uint8_t rf_smem[];
  dcplx *Vb = reinterpret_cast<dcplx *>(rf_smem);  // [RF_KMAX][RF_NMAX]
  dcplx *Xb = Vb + RF_KMAX * RF_NMAX;              // [RF_KMAX][RF_NMAX]
  __shared__ double s[RF_NMAX];
  __shared__ double red[RF_THREADS / 32];
  __shared__ dcplx H[RF_KMAX][RF_KMAX], Y[RF_KMAX][RF_KMAX];
  __shared__ double theta[RF_KMAX];
#define V(k, i) Vb[(k) * RF_NMAX + (i)]
#define X(k, i) Xb[(k) * RF_NMAX + (i)]
  const SfEigItem it = a.items[blockIdx.x];
  const int n = it.n, p = it.pol, tid = threadIdx.x, B = a.B;
  int K = a.counts[it.count_idx];
  if (K > RF_KMAX) {
    if (tid == 0) atomicOr(a.status, SF_DEVERR_BAD_SHAPE);
    K = RF_KMAX;
  }
  K = K < 0 ? 0 : K;
  const int32_t *vb = a.vis + it.vis_off;
  auto vis_at = [&](int i, int j) -> dcplx {  // V(i, j) = sum_t x_i conj(x_j), from the packed upper triangle
    const int lo = i < j ? i : j, hi = i < j ? j : i;
    const int32_t *e = vb + ((long long)baseline_of(lo, hi) * 2 + p) * 4 + p * 2;
    dcplx v = {static_cast<double>(e[0]), static_cast<double>(e[1])};
    if (i > j) v.y = -v.y;
    return v;
  };
  for (int i = tid; i < n; i += RF_THREADS) s[i] = sqrt(fmax(static_cast<double>(vb[((long long)baseline_of(i, i) * 2 + p) * 4 + p * 2]), 1e-10));
  __syncthreads();
  // whitened start vectors from the FP32 un-whitened ones
  const float2 *u = a.u32 + it.u_off;
  for (int k = 0; k < K; ++k) {
    double part = 0.0;
    for (int i = tid; i < n; i += RF_THREADS) {
      const float2 x = u[(long long)k * n + i];
      V(k, i) = {x.x / s[i], x.y / s[i]};
      part += V(k, i).x * V(k, i).x + V(k, i).y * V(k, i).y;
    }
    const double inv = 1.0 / sqrt(fmax(block_sum(part, red), 1e-300));
    for (int i = tid; i < n; i += RF_THREADS) V(k, i) = {V(k, i).x * inv, V(k, i).y * inv};
  }
  __syncthreads();
  auto apply = [&]() {  // X = A V, A = D^{-1/2} V D^{-1/2}
    for (int i = tid; i < n; i += RF_THREADS) {
      dcplx acc[RF_KMAX];
      for (int k = 0; k < RF_KMAX; ++k) acc[k] = {0.0, 0.0};
      for (int j = 0; j < n; ++j) {
        const dcplx aij0 = vis_at(i, j);
        const double sc = 1.0 / (s[i] * s[j]);
        const dcplx aij = {aij0.x * sc, aij0.y * sc};
        for (int k = 0; k < K; ++k) {
          const dcplx t = dmul(aij, V(k, j));
          acc[k].x += t.x;
          acc[k].y += t.y;
        }
      }
      for (int k = 0; k < K; ++k) X(k, i) = acc[k];
    }
    __syncthreads();
  };
  auto orth = [&](dcplx *Zb) {  // modified Gram-Schmidt, two rounds, of the vectors Zb[k * RF_NMAX + i]
    for (int k = 0; k < K; ++k) {
      for (int round = 0; round < 2; ++round)
        for (int l = 0; l < k; ++l) {
          double cr = 0.0, ci = 0.0;
          for (int i = tid; i < n; i += RF_THREADS) {
            const dcplx t = dmulc(Zb[(k) * RF_NMAX + (i)], Zb[(l) * RF_NMAX + (i)]);  // conj(z_l) z_k
            cr += t.x;
            ci += t.y;
          }
          cr = block_sum(cr, red);
          ci = block_sum(ci, red);
          for (int i = tid; i < n; i += RF_THREADS) {
            const dcplx t = dmul({cr, ci}, Zb[(l) * RF_NMAX + (i)]);
            Zb[(k) * RF_NMAX + (i)].x -= t.x;
            Zb[(k) * RF_NMAX + (i)].y -= t.y;
          }
          __syncthreads();
        }
      double part = 0.0;
      for (int i = tid; i < n; i += RF_THREADS) part += Zb[(k) * RF_NMAX + (i)].x * Zb[(k) * RF_NMAX + (i)].x + Zb[(k) * RF_NMAX + (i)].y * Zb[(k) * RF_NMAX + (i)].y;
      const double inv = 1.0 / sqrt(fmax(block_sum(part, red), 1e-300));
      for (int i = tid; i < n; i += RF_THREADS) Zb[(k) * RF_NMAX + (i)] = {Zb[(k) * RF_NMAX + (i)].x * inv, Zb[(k) * RF_NMAX + (i)].y * inv};
      __syncthreads();
    }
  };
  // Rayleigh-Ritz on span(V) with X = A V: H = V^H X, eig(H) by cyclic Jacobi
  // (thread 0), V <- V Y, X <- X Y; returns max_k ||x_k - theta_k v_k|| / theta_max
  auto ritz = [&]() -> double {
    for (int k = 0; k < K; ++k)
      for (int l = 0; l < K; ++l) {
        double hr = 0.0, hi = 0.0;
        for (int i = tid; i < n; i += RF_THREADS) {
          const dcplx t = dmulc(X(l, i), V(k, i));  // conj(v_k) x_l
          hr += t.x;
          hi += t.y;
        }
        hr = block_sum(hr, red);
        hi = block_sum(hi, red);
        if (tid == 0) H[k][l] = {hr, hi};
      }
    __syncthreads();
    if (tid == 0) {
      for (int k = 0; k < K; ++k)
        for (int l = 0; l < K; ++l) Y[k][l] = {k == l ? 1.0 : 0.0, 0.0};
      for (int sweep = 0; sweep < 30; ++sweep) {
        double off = 0.0, dg = 0.0;
        for (int k = 0; k < K; ++k) {
          dg += fabs(H[k][k].x);
          for (int l = 0; l < K; ++l)
            if (l != k) off += H[k][l].x * H[k][l].x + H[k][l].y * H[k][l].y;
        }
        if (off <= 1e-30 * dg * dg + 1e-300) break;
        for (int pp = 0; pp < K - 1; ++pp)
          for (int qq = pp + 1; qq < K; ++qq) {
            const dcplx h = H[pp][qq];
            const double g = sqrt(h.x * h.x + h.y * h.y);
            if (g < 1e-300) continue;
            const dcplx e = {h.x / g, h.y / g}, ce = {e.x, -e.y};
            const double tau = (H[qq][qq].x - H[pp][pp].x) / (2.0 * g);
            const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            const double cs = 1.0 / sqrt(1.0 + t * t), sn = t * cs;
            for (int r = 0; r < K; ++r) {  // columns p, q of H and Y
              const dcplx hp = H[r][pp], sq = dmul(ce, H[r][qq]);
              H[r][pp] = {cs * hp.x - sn * sq.x, cs * hp.y - sn * sq.y};
              H[r][qq] = {sn * hp.x + cs * sq.x, sn * hp.y + cs * sq.y};
              const dcplx yp = Y[r][pp], sy = dmul(ce, Y[r][qq]);
              Y[r][pp] = {cs * yp.x - sn * sy.x, cs * yp.y - sn * sy.y};
              Y[r][qq] = {sn * yp.x + cs * sy.x, sn * yp.y + cs * sy.y};
            }
            for (int r = 0; r < K; ++r) {  // rows p, q of H
              const dcplx hp = H[pp][r], eq = dmul(e, H[qq][r]);
              H[pp][r] = {cs * hp.x - sn * eq.x, cs * hp.y - sn * eq.y};
              H[qq][r] = {sn * hp.x + cs * eq.x, sn * hp.y + cs * eq.y};
            }
          }
      }
      // descending order of the Ritz values
      int ord[RF_KMAX];
      for (int k = 0; k < K; ++k) ord[k] = k;
      for (int k = 0; k < K; ++k)
        for (int l = 0; l + 1 < K; ++l)
          if (H[ord[l]][ord[l]].x < H[ord[l + 1]][ord[l + 1]].x) {
            const int tmp = ord[l];
            ord[l] = ord[l + 1];
            ord[l + 1] = tmp;
          }
      dcplx Ys[RF_KMAX][RF_KMAX];
      for (int k = 0; k < K; ++k) {
        theta[k] = H[ord[k]][ord[k]].x;
        for (int r = 0; r < K; ++r) Ys[r][k] = Y[r][ord[k]];
      }
      for (int r = 0; r < K; ++r)
        for (int k = 0; k < K; ++k) Y[r][k] = Ys[r][k];
    }
    __syncthreads();
    for (int i = tid; i < n; i += RF_THREADS) {
      dcplx vo[RF_KMAX], xo[RF_KMAX];
      for (int k = 0; k < K; ++k) {
        vo[k] = V(k, i);
        xo[k] = X(k, i);
      }
      for (int k = 0; k < K; ++k) {
        dcplx vn = {0.0, 0.0}, xn = {0.0, 0.0};
        for (int l = 0; l < K; ++l) {
          const dcplx a1 = dmul(vo[l], Y[l][k]), a2 = dmul(xo[l], Y[l][k]);
          vn.x += a1.x;
          vn.y += a1.y;
          xn.x += a2.x;
          xn.y += a2.y;
        }
        V(k, i) = vn;
        X(k, i) = xn;
      }
    }
    __syncthreads();
    double worst = 0.0;
    for (int k = 0; k < K; ++k) {
      double part = 0.0;
      for (int i = tid; i < n; i += RF_THREADS) {
        const double dx = X(k, i).x - theta[k] * V(k, i).x, dy = X(k, i).y - theta[k] * V(k, i).y;
        part += dx * dx + dy * dy;
      }
      worst = fmax(worst, sqrt(block_sum(part, red)));
    }
    return K > 0 ? worst / fmax(fabs(theta[0]), 1e-300) : 0.0;
  };

  double r_before = 0.0, r_after = 0.0;
  if (K > 0) {
    apply();
    r_before = ritz();
    r_after = r_before;
    for (int st = 0; st < a.steps; ++st) {
      for (int k = 0; k < K; ++k)
        for (int i = tid; i < n; i += RF_THREADS) V(k, i) = X(k, i);
      __syncthreads();
      orth(Vb);
      apply();
      r_after = ritz();
    }
  }
  if (tid == 0) {
    if (a.resid) {
      a.resid[blockIdx.x * 2] = static_cast<float>(r_before);
      a.resid[blockIdx.x * 2 + 1] = static_cast<float>(r_after);
    }
    if (a.ritz)
      for (int k = 0; k < RF_KMAX; ++k) a.ritz[(long long)blockIdx.x * RF_KMAX + k] = k < K ? theta[k] : 0.0;
  }
  // un-whiten; orthonormal basis of the nulled subspace (or each vector normalised)
  for (int k = 0; k < K; ++k) {
    for (int i = tid; i < n; i += RF_THREADS) V(k, i) = {V(k, i).x * s[i], V(k, i).y * s[i]};
    __syncthreads();
  }
  if (a.orthogonal) {
    orth(Vb);
  } else {
    for (int k = 0; k < K; ++k) {
      double part = 0.0;
      for (int i = tid; i < n; i += RF_THREADS) part += V(k, i).x * V(k, i).x + V(k, i).y * V(k, i).y;
      const double inv = 1.0 / sqrt(fmax(block_sum(part, red), 1e-300));
      for (int i = tid; i < n; i += RF_THREADS) V(k, i) = {V(k, i).x * inv, V(k, i).y * inv};
      __syncthreads();
    }
  }
  // W' = W - sum_k (W q_k) q_k^H, one beam at a time
  const __half2 *w = a.weights + it.weight_off;
  float2 *we = a.weff + it.weff_off;
  for (int m = 0; m < B; ++m) {
    double cr[RF_KMAX], ci[RF_KMAX];
    for (int k = 0; k < K; ++k) {
      double pr = 0.0, pi = 0.0;
      for (int i = tid; i < n; i += RF_THREADS) {
        const float2 wf = __half22float2(w[(long long)m * n + i]);
        const dcplx t = dmul({wf.x, wf.y}, V(k, i));
        pr += t.x;
        pi += t.y;
      }
      cr[k] = block_sum(pr, red);
      ci[k] = block_sum(pi, red);
    }
    for (int i = tid; i < n; i += RF_THREADS) {
      const float2 wf = __half22float2(w[(long long)m * n + i]);
      dcplx wp = {wf.x, wf.y};
      for (int k = 0; k < K; ++k) {
        const dcplx t = dmulc({cr[k], ci[k]}, V(k, i));  // c conj(q_i)
        wp.x -= t.x;
        wp.y -= t.y;
      }
      we[(long long)m * n + i] = wf;
      we[(long long)(B + m) * n + i] = make_float2(static_cast<float>(wp.x), static_cast<float>(wp.y));
    }
  }
#undef V
#undef X
}

}  // namespace

int sf_refine64_kmax() { return RF_KMAX; }

cudaError_t sf_launch_refine64(const SfEigItem *items, int count, const int32_t *vis, const float2 *u32,
                               const int32_t *counts, const __half2 *weights, float2 *weff,
                               int B, int steps, int orthogonal, double *ritz, float *resid, uint32_t *status,
                               cudaStream_t stream) {
  if (count <= 0) return cudaSuccess;
  RefineArgs a;
  a.vis = vis;
  a.items = items;
  a.u32 = u32;
  a.counts = counts;
  a.weights = weights;
  a.weff = weff;
  a.ritz = ritz;
  a.resid = resid;
  a.status = status;
  a.B = B;
  a.steps = steps;
  a.orthogonal = orthogonal;
  const size_t smem = 2 * sizeof(dcplx) * RF_KMAX * RF_NMAX;
  cudaError_t e = sf_smem_optin(reinterpret_cast<const void *>(sf_refine64_kernel), smem);
  if (e != cudaSuccess) return e;
  sf_refine64_kernel<<<count, RF_THREADS, smem, stream>>>(a);
  return cudaGetLastError();
}
