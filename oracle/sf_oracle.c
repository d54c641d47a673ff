/*
 * sf_oracle.c - C restatement of the spatial-filtering chain (CPU oracle).
 *
 * TEST INFRASTRUCTURE ONLY: the checker and the timed CPU baseline.  Only the
 * tests, __graft_entry__.smoke() and bench.py's CPU legs load it; the product
 * path never does.
 *
 * Same algorithm and layouts as oracle/sf_oracle.py (which cites the
 * reference file:line for every step): exact integer correlation in int64 of
 * the scaled int8 samples (spatial.cuh:423-486, TCC packed triangle
 * baseline(i,j)=j(j+1)/2+i with value sum_t x_ip conj(x_jq)), same-pol
 * covariance with gain/phasor factors, diagonal whitening
 * (spatial.cuh:1068-1148), FP64 cyclic Jacobi eigendecomposition (ascending,
 * vectors in columns, the cusolverDnXsyevBatched contract), K (fixed /
 * spatial.cuh:900-950 percentile rule / noise floor), I - U U^H or shrink
 * (spatial.cuh:952-1063), W' = W P (adaptive pipeline :773-794) and the
 * beams Y = W_eff x (no conjugation).  OpenMP over channels.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct sfo_shape {
  int32_t C, F, Tp, R, Rpp, P, B;
} sfo_shape;

typedef struct {
  double re, im;
} cd;

static inline cd cmul(cd a, cd b) { return (cd){a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
static inline cd cmulc(cd a, cd b) { return (cd){a.re * b.re + a.im * b.im, a.im * b.re - a.re * b.im}; }
static inline int bl(int i, int j) { return j * (j + 1) / 2 + i; }

/* x[p][r][t] (re, im) scaled integers for one channel */
static void aligned_channel(const sfo_shape *sh, const int8_t *samples, const int16_t *scales,
                            const int32_t *offsets, int c, int32_t *xre, int32_t *xim) {
  const int T = sh->P * sh->Tp, R = sh->R;
  const size_t slot = (size_t)R * sh->Tp * 4;
  const int8_t *chan = samples + (size_t)c * (sh->P + 2) * slot;
  const int16_t *csc = scales + (size_t)c * (sh->P + 2) * R * 2;
  for (int r = 0; r < R; ++r) {
    const int f = r / sh->Rpp, n = r % sh->Rpp;
    for (int t = 0; t < T; ++t) {
      const int q = t + offsets[f];
      const int pkt = q / sh->Tp, tt = q % sh->Tp;
      const int8_t *s = chan + (size_t)pkt * slot + ((size_t)(f * sh->Tp + tt) * sh->Rpp + n) * 4;
      for (int p = 0; p < 2; ++p) {
        const int sc = csc[((size_t)pkt * R + r) * 2 + p];
        xre[((size_t)p * R + r) * T + t] = (int32_t)s[2 * p] * sc;
        xim[((size_t)p * R + r) * T + t] = (int32_t)s[2 * p + 1] * sc;
      }
    }
  }
}

static void correlate_channel(const sfo_shape *sh, const int32_t *xre, const int32_t *xim,
                              int64_t *vis /* [NBL][2][2][2] */) {
  const int T = sh->P * sh->Tp, R = sh->R;
  for (int j = 0; j < R; ++j)
    for (int i = 0; i <= j; ++i)
      for (int p = 0; p < 2; ++p)
        for (int q = 0; q < 2; ++q) {
          const int32_t *ar = xre + ((size_t)p * R + i) * T, *ai = xim + ((size_t)p * R + i) * T;
          const int32_t *br = xre + ((size_t)q * R + j) * T, *bi = xim + ((size_t)q * R + j) * T;
          int64_t sr = 0, si = 0;
          for (int t = 0; t < T; ++t) {
            sr += (int64_t)ar[t] * br[t] + (int64_t)ai[t] * bi[t];
            si += (int64_t)ai[t] * br[t] - (int64_t)ar[t] * bi[t];
          }
          int64_t *o = vis + (((size_t)bl(i, j) * 2 + p) * 2 + q) * 2;
          o[0] = sr;
          o[1] = si;
        }
}

/* Cyclic Jacobi for a complex Hermitian n x n matrix a (row-major), FP64.
 * On return w[] ascending and v column k = eigenvector k (row-major n x n). */
static void jacobi_herm(int n, cd *a, double *w, cd *v) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) v[i * n + j] = (cd){i == j ? 1.0 : 0.0, 0.0};
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        const double m2 = a[i * n + j].re * a[i * n + j].re + a[i * n + j].im * a[i * n + j].im;
        tot += m2;
        if (i != j) off += m2;
      }
    if (off <= 1e-30 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const cd apq = a[p * n + q];
        const double aw = hypot(apq.re, apq.im);
        if (aw <= 1e-300) continue;
        const double app = a[p * n + p].re, aqq = a[q * n + q].re;
        const double theta = (aqq - app) / (2.0 * aw);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
        const cd z = {apq.re / aw, -apq.im / aw}; /* e^{-i phi} */
        const cd zc = {z.re, -z.im};
        /* columns: A <- A J */
        for (int k = 0; k < n; ++k) {
          const cd xp = a[k * n + p], xq = a[k * n + q];
          const cd tz = cmul(z, xq);
          a[k * n + p] = (cd){cs * xp.re - sn * tz.re, cs * xp.im - sn * tz.im};
          a[k * n + q] = (cd){sn * xp.re + cs * tz.re, sn * xp.im + cs * tz.im};
          const cd vp = v[k * n + p], vq = v[k * n + q];
          const cd tv = cmul(z, vq);
          v[k * n + p] = (cd){cs * vp.re - sn * tv.re, cs * vp.im - sn * tv.im};
          v[k * n + q] = (cd){sn * vp.re + cs * tv.re, sn * vp.im + cs * tv.im};
        }
        /* rows: A <- J^H A */
        for (int k = 0; k < n; ++k) {
          const cd yp = a[p * n + k], yq = a[q * n + k];
          const cd tz = cmul(zc, yq);
          a[p * n + k] = (cd){cs * yp.re - sn * tz.re, cs * yp.im - sn * tz.im};
          a[q * n + k] = (cd){sn * yp.re + cs * tz.re, sn * yp.im + cs * tz.im};
        }
        a[p * n + q] = (cd){0, 0};
        a[q * n + p] = (cd){0, 0};
      }
  }
  /* sort ascending (insertion sort of indices) */
  int *idx = (int *)malloc(sizeof(int) * n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  for (int i = 1; i < n; ++i) {
    int k = idx[i], j = i - 1;
    while (j >= 0 && a[idx[j] * n + idx[j]].re > a[k * n + k].re) {
      idx[j + 1] = idx[j];
      --j;
    }
    idx[j + 1] = k;
  }
  cd *tmp = (cd *)malloc(sizeof(cd) * n * n);
  memcpy(tmp, v, sizeof(cd) * n * n);
  for (int k = 0; k < n; ++k) {
    w[k] = a[idx[k] * n + idx[k]].re;
    for (int r = 0; r < n; ++r) v[r * n + k] = tmp[r * n + idx[k]];
  }
  free(tmp);
  free(idx);
}

static double pct_f64(const double *v, int n, double q) {
  if (n <= 0) return 0.0;
  if (n == 1) return v[0];
  const double pos = (q < 0 ? 0 : q > 1 ? 1 : q) * (n - 1);
  const int lo = (int)floor(pos), hi = (int)ceil(pos);
  if (lo == hi) return v[lo];
  return v[lo] + (pos - lo) * (v[hi] - v[lo]);
}

int sfo_correlate(const sfo_shape *sh, const int8_t *samples, const int16_t *scales,
                  const int32_t *offsets, int nthreads, int64_t *vis_out) {
  const int T = sh->P * sh->Tp, R = sh->R, NBL = R * (R + 1) / 2;
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
  for (int c = 0; c < sh->C; ++c) {
    int32_t *xre = (int32_t *)malloc(sizeof(int32_t) * 2 * R * T);
    int32_t *xim = (int32_t *)malloc(sizeof(int32_t) * 2 * R * T);
    aligned_channel(sh, samples, scales, offsets, c, xre, xim);
    correlate_channel(sh, xre, xim, vis_out + (size_t)c * NBL * 8);
    free(xre);
    free(xim);
  }
  return 0;
}

/* Whole adaptive chain.  weights float [C][2][B][R][2]; factors double
 * [C][2][R][2] (gain x phasor); fixed_k [C]; k_rule 0 fixed, 1 percentile
 * detect (delta), 2 noise floor (delta x median).  Outputs (any may be NULL):
 * vis int64 [C][NBL][2][2][2], evals [C][2][R], counts [C][2], beams double
 * [C][2][2B][T][2] (slot 0 original, slot 1 projected). */
int sfo_adaptive_chain(const sfo_shape *sh, const int8_t *samples, const int16_t *scales,
                       const int32_t *offsets, const float *weights, const double *factors,
                       const int32_t *fixed_k, int k_rule, double delta, int shrink, int nthreads,
                       int64_t *vis_out, double *evals_out, int32_t *counts_out,
                       double *beams_out) {
  const int T = sh->P * sh->Tp, R = sh->R, B = sh->B, NBL = R * (R + 1) / 2;
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
  for (int c = 0; c < sh->C; ++c) {
    int32_t *xre = (int32_t *)malloc(sizeof(int32_t) * 2 * R * T);
    int32_t *xim = (int32_t *)malloc(sizeof(int32_t) * 2 * R * T);
    int64_t *vis = (int64_t *)malloc(sizeof(int64_t) * NBL * 8);
    cd *a = (cd *)malloc(sizeof(cd) * R * R);
    cd *v = (cd *)malloc(sizeof(cd) * R * R);
    cd *pm = (cd *)malloc(sizeof(cd) * R * R);
    cd *weff = (cd *)malloc(sizeof(cd) * 2 * B * R);
    double *w = (double *)malloc(sizeof(double) * R);
    double *sd = (double *)malloc(sizeof(double) * R);
    aligned_channel(sh, samples, scales, offsets, c, xre, xim);
    correlate_channel(sh, xre, xim, vis);
    if (vis_out) memcpy(vis_out + (size_t)c * NBL * 8, vis, sizeof(int64_t) * NBL * 8);
    for (int p = 0; p < 2; ++p) {
      const double *d = factors + ((size_t)c * 2 + p) * R * 2;
      for (int i = 0; i < R; ++i)
        for (int j = 0; j < R; ++j) {
          const int lo = i < j ? i : j, hi = i < j ? j : i;
          const int64_t *x = vis + (((size_t)bl(lo, hi) * 2 + p) * 2 + p) * 2;
          cd val = {(double)x[0], (double)x[1]};
          const cd dl = {d[2 * lo], d[2 * lo + 1]}, dh = {d[2 * hi], d[2 * hi + 1]};
          val = cmulc(cmul(dl, val), dh);
          if (i == j) val.im = 0.0;
          else if (i > j) val.im = -val.im;
          a[i * R + j] = val;
        }
      for (int i = 0; i < R; ++i) sd[i] = sqrt(a[i * R + i].re > 1e-10 ? a[i * R + i].re : 1e-10);
      for (int i = 0; i < R; ++i)
        for (int j = 0; j < R; ++j) {
          a[i * R + j].re /= sd[i] * sd[j];
          a[i * R + j].im /= sd[i] * sd[j];
        }
      jacobi_herm(R, a, w, v);
      int k = 0;
      if (k_rule == 1) {
        const double s = (pct_f64(w, R, 0.8) - pct_f64(w, R, 0.2)) / (2.0 * 0.8416);
        const double thr = pct_f64(w, R, 0.5) + delta * s;
        for (int i = 0; i < R; ++i) k += w[i] > thr;
      } else if (k_rule == 2) {
        const double med = 0.5 * (w[(R - 1) / 2] + w[R / 2]);
        for (int i = 0; i < R; ++i) k += w[i] > delta * med;
      } else {
        k = fixed_k ? fixed_k[c] : 0;
      }
      if (k < 0) k = 0;
      if (k > R) k = R;
      if (evals_out) memcpy(evals_out + ((size_t)c * 2 + p) * R, w, sizeof(double) * R);
      if (counts_out) counts_out[c * 2 + p] = k;
      double lam_bar = 0.0;
      if (shrink) {
        if (k < R) {
          for (int i = 0; i < R - k; ++i) lam_bar += w[i];
          lam_bar /= (R - k);
        }
      } else {
        /* un-whiten and normalise every column */
        for (int col = 0; col < R; ++col) {
          double s2 = 0.0;
          for (int r = 0; r < R; ++r) {
            v[r * R + col].re *= sd[r];
            v[r * R + col].im *= sd[r];
            s2 += v[r * R + col].re * v[r * R + col].re + v[r * R + col].im * v[r * R + col].im;
          }
          const double inv = s2 > 0 ? 1.0 / sqrt(s2) : 0.0;
          for (int r = 0; r < R; ++r) {
            v[r * R + col].re *= inv;
            v[r * R + col].im *= inv;
          }
        }
      }
      for (int r = 0; r < R; ++r)
        for (int cc = 0; cc < R; ++cc) {
          cd acc = {r == cc ? 1.0 : 0.0, 0.0};
          if (shrink) {
            /* M = V diag(d) V^H */
            acc = (cd){0, 0};
            for (int kk = 0; kk < R; ++kk) {
              double dk = 1.0;
              if (kk >= R - k) dk = w[kk] > 0 ? lam_bar / w[kk] : 0.0;
              const cd t = cmulc(v[r * R + kk], v[cc * R + kk]);
              acc.re += dk * t.re;
              acc.im += dk * t.im;
            }
          } else {
            for (int kk = R - k; kk < R; ++kk) {
              const cd t = cmulc(v[r * R + kk], v[cc * R + kk]);
              acc.re -= t.re;
              acc.im -= t.im;
            }
          }
          pm[r * R + cc] = acc;
        }
      for (int m = 0; m < B; ++m)
        for (int col = 0; col < R; ++col) {
          const float *wm = weights + ((((size_t)c * 2 + p) * B + m) * R) * 2;
          const cd dc = {d[2 * col], d[2 * col + 1]};
          const cd w0 = {wm[2 * col], wm[2 * col + 1]};
          weff[(size_t)m * R + col] = cmul(w0, dc);
          cd acc = {0, 0};
          for (int l = 0; l < R; ++l) {
            const cd t = cmul((cd){wm[2 * l], wm[2 * l + 1]}, pm[l * R + col]);
            acc.re += t.re;
            acc.im += t.im;
          }
          weff[(size_t)(B + m) * R + col] = cmul(acc, dc);
        }
      if (beams_out) {
        for (int m = 0; m < 2 * B; ++m) {
          double *yo = beams_out + ((((size_t)c * 2 + p) * 2 * B + m) * T) * 2;
          for (int t = 0; t < T; ++t) {
            yo[2 * t] = 0.0;
            yo[2 * t + 1] = 0.0;
          }
          for (int r = 0; r < R; ++r) {
            const cd we = weff[(size_t)m * R + r];
            const int32_t *xr = xre + ((size_t)p * R + r) * T, *xi = xim + ((size_t)p * R + r) * T;
            for (int t = 0; t < T; ++t) {
              yo[2 * t] += we.re * xr[t] - we.im * xi[t];
              yo[2 * t + 1] += we.re * xi[t] + we.im * xr[t];
            }
          }
        }
      }
    }
    free(xre);
    free(xim);
    free(vis);
    free(a);
    free(v);
    free(pm);
    free(weff);
    free(w);
    free(sd);
  }
  return 0;
}

int sfo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
