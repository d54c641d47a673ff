// Adaptive-path eigensolver for up to 128 receivers and 16 beams: one CTA per
// (channel, pol) covariance -- four warps with two rows per lane up to 64
// receivers, sixteen warps with four rows per lane up to 128.  Same algorithm as
// sf_eig_topk.cu -- whitening, Householder tridiagonalisation, Sturm counts
// with multisection, K, inverse iteration for the top K, back-transform,
// un-whitening, projected weights -- laid out so that no thread walks a long
// serial chain:
//
// * Householder: each row of the trailing matrix is split over four lanes
//   (columns j = s mod 4), so a thread touches about m / 4 elements per
//   step, with its shared-memory loads issued in batches of four.  Warp 0
//   updates column 0 of the trailing matrix in registers and forms the next
//   reflector from them while the other warps do the rest of the rank-2 update, so
//   a step costs two CTA barriers (after tau A v, after the update).  The scaled reflector
//   is kept in the dead upper triangle (row k), where the back-transform
//   reads it with unit stride.
// * Eigenvalues: the tridiagonal is scaled by a power of two to norm <= 1 and
//   the Sturm count uses the three-term determinant recurrence
//   p_i = (d_i - x) p_(i-1) - e_(i-1)^2 p_(i-2) (sign changes counted, both
//   terms rescaled every eight steps, a zero pivot replaced as in the ratio
//   form), so the dependent chain per step is one FMA and a select instead of
//   a reciprocal.  Each thread carries four points: a 512-point grid first,
//   then multisection with g threads (4 g points) per eigenvalue.
// * Inverse iteration: the LU factors and solves load their operands eight
//   steps ahead and pivot with selects, not branches.
//
// The matrix is row-major in both triangles with a leading dimension
// ld = 4 (mod 16), so the four segments of the eight rows a half-warp touches
// fall in distinct banks.
//
// Published algorithms restated: LAPACK zhetd2 / zlarfg (Householder
// tridiagonalisation of a Hermitian matrix), Sturm sequences (eigenvalue
// counts of a symmetric tridiagonal) with bisection / multisection, inverse
// iteration with partial pivoting and modified Gram-Schmidt.
#include <algorithm>
#include <cstdio>

#include "sf_common.cuh"
#include "sf_plan.cuh"

namespace {

constexpr int SN_MAX = 128;
constexpr int SB_MAX = 16;
constexpr int S_GROUP = 8;          // inverse-iteration vectors per pass (lanes 0..7 of warp 0)
constexpr int S_INV_ITERS = 3;
constexpr int S_COARSE = 512;       // coarse Sturm grid points (four per thread of the first 128)
constexpr int S_VEC = 4;            // eigenvectors back-transformed per pass (one per warp of warps 0-3)
constexpr int S_RED = 32;           // float2 slots of the cross-warp partials (16 warps) and scalars
constexpr unsigned FULL = 0xffffffffu;

// top-K eigenvectors of T kept in shared memory: every one up to 64 receivers, 32 beyond
__host__ __device__ inline int small_xk(int n) { return n <= 64 ? n : 32; }

struct SmallEigArgs {
  const int32_t *vis;
  const float2 *factors;
  const __half2 *weights;
  const int32_t *fixed_counts;
  float *evals;
  int32_t *counts;
  float2 *weff;
  uint32_t *status;  // SF_DEVERR_BAD_SHAPE when K exceeds the kept eigenvectors (K is clamped)
  int C, R, B, NBL;
  int k_rule, shrink;
  float delta;
  // matrices list[0 .. *list_count) instead of all 2C (the learned chain's fallback), or NULL
  const int32_t *list;
  const int32_t *list_count;
  // batched form: matrices items[first_item .. first_item + n_items) (R = their largest n), or NULL
  const SfEigItem *items;
  int first_item, n_items;
};

// one matrix's inputs and outputs
struct SmallMat {
  int n;
  const int32_t *vin;   // same-pol entry (p, p) of packed baseline b at vin[8 b], vin[8 b + 1]
  const float2 *fac;    // receiver factors [n], or NULL for unit factors
  const __half2 *w;     // weights [B][n]
  float2 *we;           // effective weights [2B][n] (slot 0 original, slot 1 projected)
  float *ev;            // eigenvalues [n], or NULL
  int32_t *cnt;         // K, or NULL
  int kfix;             // K of the fixed rule (clamped to [0, n] here)
};

// leading dimension (float2) of the matrix: the smallest ld >= n with ld = 4 (mod 16)
__host__ __device__ inline int small_ld(int n) { return n + ((4 - n) & 15); }

// byte offsets of the CTA's shared-memory region
struct SRegion {
  size_t vp, de, A, taus, fac, W0, Wp, Z, coef, red, X, LU, dvec, cnt, total;
};
__host__ __device__ inline SRegion s_region(int n, int B) {
  SRegion r;
  size_t o = 0;
  r.vp = o;    o += 16 * 2 * (size_t)n;             // float4 {v, tau A v}, two buffers
  r.de = o;    o += 8 * (size_t)n;                  // float2 {d_i, e_(i-1)^2}, scaled
  r.A = o;     o += 8 * (size_t)n * small_ld(n);    // float2
  r.taus = o;  o += 8 * (size_t)n;
  r.fac = o;   o += 8 * (size_t)n;
  r.W0 = o;    o += 8 * (size_t)B * n;
  r.Wp = o;    o += 8 * (size_t)B * n;
  r.Z = o;     o += 8 * (size_t)S_VEC * n;
  r.coef = o;  o += 8 * (size_t)S_VEC * SB_MAX;
  r.red = o;   o += 8 * (size_t)S_RED;               // cross-warp partials and scalars
  r.X = o;     o += 4 * (size_t)small_xk(n) * n;    // float: top-K eigenvectors of T
  r.LU = o;    o += 4 * 5 * (size_t)S_GROUP * n;    // float: inverse-iteration factors
  r.dvec = o;  o += 4 * 5 * (size_t)n;              // float: d, e, e2, lam, sd
  r.cnt = o;   o += 4 * (size_t)S_COARSE;           // int: coarse-grid counts
  r.total = (o + 15) & ~size_t(15);
  return r;
}

__device__ __forceinline__ float wsum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}
__device__ __forceinline__ void wsum2(float &a, float &b) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float ta = __shfl_xor_sync(FULL, a, o), tb = __shfl_xor_sync(FULL, b, o);
    a += ta;
    b += tb;
  }
}
__device__ __forceinline__ float wmax(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(FULL, v, o));
  return v;
}
__device__ __forceinline__ float wmin(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(FULL, v, o));
  return v;
}
__device__ __forceinline__ float fast_rcp(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ float2 vpart(const float4 &q) { return make_float2(q.x, q.y); }

// value at quantile `quant` of ascending v[0..n), linear interpolation between
// order statistics (the reference's detection rule, spatial.cuh:900-917)
__device__ __forceinline__ float pct_sorted(const float *v, int n, float quant) {
  if (n <= 0) return 0.0f;
  if (n == 1) return v[0];
  const float qc = fminf(1.0f, fmaxf(0.0f, quant));
  const float pos = qc * static_cast<float>(n - 1);
  const int lo = static_cast<int>(floorf(pos)), hi = static_cast<int>(ceilf(pos));
  if (lo == hi) return v[lo];
  return v[lo] + (pos - static_cast<float>(lo)) * (v[hi] - v[lo]);
}

// one Sturm step of the three-term recurrence for four points
__device__ __forceinline__ void sturm_step(float2 f, const float (&x)[4], float pivmin, float (&p0)[4], float (&p1)[4],
                                           int (&cnt)[4]) {
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float pn = fmaf(f.x - x[c], p1[c], -f.y * p0[c]);
    // a pivot q = p_i / p_(i-1) below pivmin in magnitude becomes -pivmin (the ratio form's rule)
    pn = fabsf(pn) < pivmin * fabsf(p1[c]) ? -pivmin * p1[c] : pn;
    cnt[c] += (__float_as_uint(pn) ^ __float_as_uint(p1[c])) >> 31;
    p0[c] = p1[c];
    p1[c] = pn;
  }
}
__device__ __forceinline__ void sturm_rescale(float (&p0)[4], float (&p1)[4]) {
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int ex = max((__float_as_int(p0[c]) >> 23) & 0xff, (__float_as_int(p1[c]) >> 23) & 0xff);
    const float s = __int_as_float((254 - ex) << 23);  // 2^(127 - ex): the larger term into [1, 2)
    p0[c] *= s;
    p1[c] *= s;
  }
}

// #{eigenvalues of T < x_c} for four points: sign changes of the leading
// principal minors det(T_i - x_c I), T scaled to norm <= 1 (so a term grows
// at most 3x per step and eight steps stay far from overflow)
__device__ __forceinline__ void sturm4(const float2 *de, int n, const float (&x)[4], float pivmin, int (&cnt)[4]) {
  float p0[4], p1[4];
  const float d0 = de[0].x;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    p0[c] = 1.0f;
    p1[c] = d0 - x[c];
    if (fabsf(p1[c]) < pivmin) p1[c] = -pivmin;
    cnt[c] = __float_as_uint(p1[c]) >> 31;
  }
  int i = 1;
  for (; i + 7 < n; i += 8) {
    float2 f[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) f[u] = de[i + u];
#pragma unroll
    for (int u = 0; u < 8; ++u) sturm_step(f[u], x, pivmin, p0, p1, cnt);
    sturm_rescale(p0, p1);
  }
  for (; i < n; ++i) sturm_step(de[i], x, pivmin, p0, p1, cnt);
}

// grid point P of `npts` interior points of [lo, hi]: one expression wherever a
// point is formed, so brackets taken from a point equal the point counted
__device__ __forceinline__ float grid_point(float lo, float hi, int P, int npts) {
  return lo + (hi - lo) * (static_cast<float>(P + 1) / static_cast<float>(npts + 1));
}

// Warp-wide: the reflector of column kk (zlarfg) from values in registers:
// lane l holds rows kk + l + 32 q (r[q], q < NPL) of the column, so the
// entries c_i = A[kk+1+i][kk], i < mm = n - kk - 1, are r[q] of lane i + 1 - 32 q.
// H^H c = beta e_1 with H = I - tau v v^H, v_0 = 1.  Writes v to vb[i].xy
// (i < mm), the scaled entries v_i (i >= 1) into the dead upper triangle
// A[kk][kk+1+i], taus[kk] and e[kk] = beta.
template <int NPL>
__device__ __forceinline__ void make_reflector(const float2 (&r)[NPL], float2 *A, int ld, int n, int kk, float4 *vb,
                                               float2 *taus, float *e, int lane) {
  const int mm = n - kk - 1;
  const float2 alpha = make_float2(__shfl_sync(FULL, r[0].x, 1), __shfl_sync(FULL, r[0].y, 1));
  float2 c[NPL];
  bool h[NPL];
  float part = 0.0f;
#pragma unroll
  for (int q = 0; q < NPL; ++q) {
    const int row = lane + 32 * q;  // entry row - 1
    h[q] = row >= 2 && row <= mm;
    c[q] = h[q] ? r[q] : make_float2(0.0f, 0.0f);
    part += c[q].x * c[q].x + c[q].y * c[q].y;
  }
  const float xnorm2 = wsum(part);
  float2 tau = make_float2(0.0f, 0.0f);
  float beta = alpha.x;
  if (!(xnorm2 == 0.0f && alpha.y == 0.0f)) {
    const float nrm2 = alpha.x * alpha.x + alpha.y * alpha.y + xnorm2;  // > 0 here
    const float nrm = nrm2 * rsqrtf(nrm2);
    beta = alpha.x >= 0.0f ? -nrm : nrm;
    const float rb = fast_rcp(beta);
    tau = make_float2((beta - alpha.x) * rb, -alpha.y * rb);
    const float2 am = make_float2(alpha.x - beta, alpha.y);  // |am| >= nrm > 0
    const float inv = fast_rcp(am.x * am.x + am.y * am.y);
    const float2 sc = make_float2(am.x * inv, -am.y * inv);
#pragma unroll
    for (int q = 0; q < NPL; ++q) c[q] = cmul(c[q], sc);
  }
  float2 *urow = A + (size_t)kk * ld + (kk + 1);  // entry i at urow[i]
#pragma unroll
  for (int q = 0; q < NPL; ++q) {
    if (h[q]) {
      const int i = lane + 32 * q - 1;
      *reinterpret_cast<float2 *>(&vb[i]) = c[q];
      urow[i] = c[q];
    }
  }
  if (lane == 0) {
    *reinterpret_cast<float2 *>(&vb[0]) = make_float2(1.0f, 0.0f);
    taus[kk] = tau;
    e[kk] = beta;
  }
}

// a_ij -= v_i conj(p_j + cvv v_j) + p_i conj(v_j) for one element
__device__ __forceinline__ float2 rank2(float2 r, const float4 &qi, const float4 &qj, float cvv) {
  const float wx = qj.z + cvv * qj.x, wy = qj.w + cvv * qj.y;
  r.x -= qi.x * wx + qi.y * wy + qi.z * qj.x + qi.w * qj.y;
  r.y -= qi.y * wx - qi.x * wy + qi.w * qj.x - qi.z * qj.y;
  return r;
}

// the whole solve of one matrix by the CTA of NT threads, NPL rows per lane (n <= 32 NPL)
template <int NT, int NPL>
__device__ __forceinline__ void eig_small_one(const SmallEigArgs &a, const SmallMat &mt, uint8_t *smem) {
  constexpr int NWARP = NT / 32;
  constexpr int RS = NT / 4;  // row slots of the row-split loops (four lanes per row)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int rs = tid >> 2, sg = tid & 3;  // row slot, column segment
  const int n = mt.n, B = a.B, ld = small_ld(n);
  const SRegion L = s_region(n, B);
  float4 *vp = reinterpret_cast<float4 *>(smem + L.vp);
  float2 *de = reinterpret_cast<float2 *>(smem + L.de);
  float2 *A = reinterpret_cast<float2 *>(smem + L.A);
  float2 *taus = reinterpret_cast<float2 *>(smem + L.taus);
  float2 *fac = reinterpret_cast<float2 *>(smem + L.fac);
  float2 *W0 = reinterpret_cast<float2 *>(smem + L.W0);
  float2 *Wp = reinterpret_cast<float2 *>(smem + L.Wp);
  float2 *Z = reinterpret_cast<float2 *>(smem + L.Z);
  float2 *coef = reinterpret_cast<float2 *>(smem + L.coef);
  float2 *red = reinterpret_cast<float2 *>(smem + L.red);
  float *redf = reinterpret_cast<float *>(smem + L.red);
  float *X = reinterpret_cast<float *>(smem + L.X);
  float *U0 = reinterpret_cast<float *>(smem + L.LU);
  float *U1 = U0 + S_GROUP * n;
  float *U2 = U1 + S_GROUP * n;
  float *ML = U2 + S_GROUP * n;
  float *PV = ML + S_GROUP * n;
  float *d = reinterpret_cast<float *>(smem + L.dvec);
  float *e = d + n;
  float *e2 = e + n;
  float *lam = e2 + n;
  float *sd = lam + n;
  int *cnt = reinterpret_cast<int *>(smem + L.cnt);
  // same-pol entry (p, p) of baseline b at vin[8 b], vin[8 b + 1] (layout [b][Pol][Pol][2])
  const int32_t *vin = mt.vin;

  // ---- 1. covariance d_i V conj(d_j), both triangles, whitened ----
  for (int i = tid; i < n; i += NT) {
    const float2 di = mt.fac ? mt.fac[i] : make_float2(1.0f, 0.0f);
    fac[i] = di;
    const float v = static_cast<float>(vin[(size_t)baseline_of(i, i) * 8]);
    sd[i] = sqrtf(fmaxf(v * (di.x * di.x + di.y * di.y), 1e-10f));
  }
  {
    const __half2 *w = mt.w;
    for (int ee = tid; ee < B * n; ee += NT) {
      const float2 x = __half22float2(w[ee]);
      W0[ee] = x;
      Wp[ee] = x;
    }
  }
  __syncthreads();
  {
    const int nb = n * (n + 1) / 2;
    for (int b0 = 0; b0 < nb; b0 += 4 * NT) {
      int2 raw[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int b = b0 + u * NT + tid;
        raw[u] = b < nb ? *reinterpret_cast<const int2 *>(vin + (size_t)b * 8) : make_int2(0, 0);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int b = b0 + u * NT + tid;
        if (b < nb) {
          // b = j (j + 1) / 2 + i, i <= j
          int j = static_cast<int>((sqrtf(8.0f * static_cast<float>(b) + 1.0f) - 1.0f) * 0.5f);
          if ((j + 1) * (j + 2) / 2 <= b) ++j;
          if (j * (j + 1) / 2 > b) --j;
          const int i = b - j * (j + 1) / 2;
          float2 x = make_float2(static_cast<float>(raw[u].x), static_cast<float>(raw[u].y));
          x = cmulc(cmul(fac[i], x), fac[j]);  // element (i, j), i <= j
          const float inv = 1.0f / (sd[i] * sd[j]);
          A[(size_t)i * ld + j] = i == j ? make_float2(x.x * inv, 0.0f) : make_float2(x.x * inv, x.y * inv);
          if (j > i) A[(size_t)j * ld + i] = make_float2(x.x * inv, -x.y * inv);
        }
      }
    }
  }
  __syncthreads();

  // ---- 2. Householder tridiagonalisation T = Q^H A Q (lower) ----
  if (warp == 0) {
    float2 r[NPL];
#pragma unroll
    for (int q = 0; q < NPL; ++q) r[q] = lane + 32 * q < n ? A[(size_t)(lane + 32 * q) * ld] : make_float2(0.0f, 0.0f);
    make_reflector<NPL>(r, A, ld, n, 0, vp, taus, e, lane);
  }
  __syncthreads();
  for (int k = 0; k < n - 1; ++k) {
    const int m = n - k - 1;  // order of the trailing matrix A22 = A[k+1.., k+1..]
    float4 *vb = vp + (k & 1) * n;
    float4 *vnext = vp + ((k + 1) & 1) * n;
    const float2 tau = taus[k];
    const bool act = !(tau.x == 0.0f && tau.y == 0.0f);  // the same in every thread
    float2 *A22 = A + (size_t)(k + 1) * ld + (k + 1);
    float cvv = 0.0f;
    if (act) {
      // p = tau A22 v: thread (rs, sg) sums the columns j = sg (mod 4) of rows rs, rs + RS, ...
      float pr = 0.0f, pim = 0.0f;  // this thread's part of p^H v
      for (int q = 0; RS * q < m; ++q) {  // uniform
        const int i = rs + RS * q;
        const int jm = i < m ? m : 0;
        const float2 *row = A22 + (size_t)i * ld;
        const float2 vi = sg == 0 && i < m ? vpart(vb[i]) : make_float2(0.0f, 0.0f);
        float2 a0 = make_float2(0.0f, 0.0f), a1 = make_float2(0.0f, 0.0f);
        int j = sg;
        for (; j + 12 < jm; j += 16) {
          float2 r[4], v[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            r[u] = row[j + 4 * u];
            v[u] = vpart(vb[j + 4 * u]);
          }
#pragma unroll
          for (int u = 0; u < 4; u += 2) {
            a0.x += r[u].x * v[u].x - r[u].y * v[u].y;
            a0.y += r[u].x * v[u].y + r[u].y * v[u].x;
            a1.x += r[u + 1].x * v[u + 1].x - r[u + 1].y * v[u + 1].y;
            a1.y += r[u + 1].x * v[u + 1].y + r[u + 1].y * v[u + 1].x;
          }
        }
        for (; j < jm; j += 4) {
          const float2 r = row[j], v = vpart(vb[j]);
          a0.x += r.x * v.x - r.y * v.y;
          a0.y += r.x * v.y + r.y * v.x;
        }
        float sx = a0.x + a1.x, sy = a0.y + a1.y;
        sx += __shfl_xor_sync(FULL, sx, 1);
        sy += __shfl_xor_sync(FULL, sy, 1);
        sx += __shfl_xor_sync(FULL, sx, 2);
        sy += __shfl_xor_sync(FULL, sy, 2);
        if (sg == 0 && i < m) {
          const float2 pi = cmul(tau, make_float2(sx, sy));
          *reinterpret_cast<float2 *>(&vb[i].z) = pi;
          const float2 t = cmulc(vi, pi);  // conj(p_i) v_i
          pr += t.x;
          pim += t.y;
        }
      }
#pragma unroll
      for (int o = 4; o < 32; o <<= 1) {
        pr += __shfl_xor_sync(FULL, pr, o);
        pim += __shfl_xor_sync(FULL, pim, o);
      }
      if (lane == 0) red[warp] = make_float2(pr, pim);
      __syncthreads();  // p and the partials of p^H v
      float2 pv = red[0];
#pragma unroll
      for (int w = 1; w < NWARP; ++w) {
        pv.x += red[w].x;
        pv.y += red[w].y;
      }
      // A22 -= v p^H + p v^H + 2 Re(alpha') v v^H, alpha' = -1/2 tau (p^H v)
      cvv = -(tau.x * pv.x - tau.y * pv.y);
    }
    if (warp == 0) {
      // column 0 of A22 (rows lane + 32 q): the next diagonal entry and the next reflector,
      // formed while the other warps update the rest
      float2 r[NPL];
#pragma unroll
      for (int q = 0; q < NPL; ++q) r[q] = lane + 32 * q < m ? A22[(size_t)(lane + 32 * q) * ld] : make_float2(0.0f, 0.0f);
      if (act) {
        const float4 q0 = vb[0];
#pragma unroll
        for (int q = 0; q < NPL; ++q)
          if (lane + 32 * q < m) r[q] = rank2(r[q], vb[lane + 32 * q], q0, cvv);
      }
      if (lane == 0) A22[0] = r[0];
      if (k + 1 < n - 1) make_reflector<NPL>(r, A, ld, n, k + 1, vnext, taus, e, lane);
    } else if (act) {
      // rows 1.. and columns 1.. of A22 (row 0 is the dead mirror of column 0): RS - 8 row slots
      const int rs3 = rs - 8;
      for (int i = 1 + rs3; i < m; i += RS - 8) {
        float2 *row = A22 + (size_t)i * ld;
        const float4 qi = vb[i];
        int j = 1 + sg;
        for (; j + 12 < m; j += 16) {
          float2 r[4];
          float4 qq[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            r[u] = row[j + 4 * u];
            qq[u] = vb[j + 4 * u];
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) r[u] = rank2(r[u], qi, qq[u], cvv);
#pragma unroll
          for (int u = 0; u < 4; ++u) row[j + 4 * u] = r[u];
        }
        for (; j < m; j += 4) row[j] = rank2(row[j], qi, vb[j], cvv);
      }
    }
    __syncthreads();  // the trailing matrix and the next reflector
  }

  // ---- 3. eigenvalues: Gershgorin bracket, scaled T, coarse grid, multisection ----
  for (int i = tid; i < n; i += NT) {
    d[i] = A[(size_t)i * ld + i].x;
    if (i == n - 1) e[i] = 0.0f;
  }
  __syncthreads();
  if (warp == 0) {
    float glo = 3.0e38f, ghi = -3.0e38f, emax = 0.0f;
    for (int i = lane; i < n; i += 32) {
      e2[i] = e[i] * e[i];
      const float r = fabsf(e[i]) + (i > 0 ? fabsf(e[i - 1]) : 0.0f);
      glo = fminf(glo, d[i] - r);
      ghi = fmaxf(ghi, d[i] + r);
      emax = fmaxf(emax, e[i] * e[i]);
    }
    glo = wmin(glo);
    ghi = wmax(ghi);
    emax = wmax(emax);
    const float tnorm = fmaxf(fabsf(glo), fabsf(ghi));
    // scale by 2^-ex with tnorm < 2^ex: exact, and |d|, |e| <= 1 afterwards
    const int ex = ((__float_as_int(tnorm) >> 23) & 0xff) - 126;
    const float sc = __int_as_float((127 - ex) << 23);
    for (int i = lane; i < n; i += 32) {
      const float es = i > 0 ? e[i - 1] * sc : 0.0f;
      de[i] = make_float2(d[i] * sc, es * es);
    }
    if (lane == 0) {
      const float tn = tnorm * sc, pivs = fmaxf(1e-30f, 1e-30f * emax * sc * sc);
      redf[40] = glo * sc - (2e-7f * tn + pivs);                  // scaled bracket low
      redf[41] = ghi * sc + (2e-7f * tn + pivs);                  // scaled bracket high
      redf[42] = 2.4e-7f * tn + 4.0f * pivs;                     // scaled absolute tolerance
      redf[43] = pivs;                                           // scaled pivmin
      redf[44] = __int_as_float((127 + ex) << 23);               // 1 / sc
      redf[45] = 2.4e-7f * tnorm + fmaxf(1e-30f, 1e-30f * emax);  // inverse-iteration pivot floor
    }
  }
  __syncthreads();
  const float glo = redf[40], ghi = redf[41], atol = redf[42], pivs = redf[43], unsc = redf[44], pert = redf[45];
  const int Kfix = max(0, min(n, mt.kfix));
  const bool need_all = a.k_rule != SF_K_FIXED || mt.ev != nullptr || a.shrink || Kfix > 32;
  if (tid < S_COARSE / 4) {
    float xs[4];
    int cn[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) xs[s] = grid_point(glo, ghi, 4 * tid + s, S_COARSE);
    sturm4(de, n, xs, pivs, cn);
#pragma unroll
    for (int s = 0; s < 4; ++s) cnt[4 * tid + s] = cn[s];
  }
  __syncthreads();
  {
    const int ne = need_all ? n : Kfix;
    // threads per eigenvalue: a power of two, so a group lies in one warp; at most 128 threads in
    // all (the passes are issue-bound beyond four warps: 16 warps on 128 eigenvalues measured 3x
    // the cycles of 4)
    int g = 1;
    while (g < 32 && 2 * g * ne <= (NT < 128 ? NT : 128)) g *= 2;
    const int r = tid / g, sub = tid - r * g;
    const bool mine = r < ne;
    const int j = need_all ? r : n - 1 - r;
    const int gbase = lane - sub;
    const unsigned gmask = (g == 32 ? FULL : ((1u << g) - 1u)) << gbase;
    float lo = glo, hi = ghi;
    if (mine) {
      // first coarse point with more than j eigenvalues below it
      int t0 = 0, t1 = S_COARSE;
      while (t0 < t1) {
        const int mid = (t0 + t1) >> 1;
        if (cnt[mid] > j) t1 = mid;
        else t0 = mid + 1;
      }
      if (t0 > 0) lo = grid_point(glo, ghi, t0 - 1, S_COARSE);
      if (t0 < S_COARSE) hi = grid_point(glo, ghi, t0, S_COARSE);
    }
    bool done = !mine || hi - lo <= atol;
    const int npts = 4 * g;
    for (int it = 0; it < 40; ++it) {
      if (__all_sync(FULL, done)) break;
      float xs[4];
      int cn[4];
#pragma unroll
      for (int s = 0; s < 4; ++s) xs[s] = grid_point(lo, hi, 4 * sub + s, npts);
      sturm4(de, n, xs, pivs, cn);
      int fl = 4;  // this thread's first point with more than j below it
#pragma unroll
      for (int s = 3; s >= 0; --s)
        if (cn[s] > j) fl = s;
      const unsigned bal = __ballot_sync(FULL, fl < 4) & gmask;
      const int ft = bal ? __ffs(bal) - 1 : lane;
      const int f = __shfl_sync(FULL, fl, ft);
      // lambda_j in [x_(P-1), x_P), P = the group's first point above
      const int P = bal ? 4 * (ft - gbase) + f : npts;
      const float nlo = P == 0 ? lo : grid_point(lo, hi, P - 1, npts);
      const float nhi = P == npts ? hi : grid_point(lo, hi, P, npts);
      if (!done) {
        done = (nlo == lo && nhi == hi) || nhi - nlo <= atol;
        lo = nlo;
        hi = nhi;
      }
    }
    if (mine && sub == 0) lam[j] = 0.5f * (lo + hi) * unsc;
  }
  __syncthreads();
  if (mt.ev)
    for (int j = tid; j < n; j += NT) mt.ev[j] = lam[j];

  // ---- 4. K ----
  int *sK = reinterpret_cast<int *>(redf + 46);
  if (tid == 0) {
    int K = 0;
    if (a.k_rule == SF_K_DETECT) {
      const float p20 = pct_sorted(lam, n, 0.2f), p50 = pct_sorted(lam, n, 0.5f), p80 = pct_sorted(lam, n, 0.8f);
      const float thr = p50 + a.delta * ((p80 - p20) / (2.0f * 0.8416f));
      for (int i = 0; i < n; ++i) K += lam[i] > thr;
    } else if (a.k_rule == SF_K_NOISE_FLOOR) {
      const float med = 0.5f * (lam[(n - 1) / 2] + lam[n / 2]);
      for (int i = 0; i < n; ++i) K += lam[i] > a.delta * med;
    } else {
      K = Kfix;
    }
    K = max(0, min(n, K));
    if (K > small_xk(n)) {  // more modes than the kept eigenvectors: null the top ones kept
      if (a.status) atomicOr(a.status, SF_DEVERR_BAD_SHAPE);
      K = small_xk(n);
    }
    *sK = K;
    if (mt.cnt) *mt.cnt = K;
  }
  __syncthreads();
  const int K = *sK;

  // ---- 5. top-K eigenvectors of T: inverse iteration (lanes 0..7 of warp 0) + MGS ----
  if (warp == 0) {
    for (int g0 = 0; g0 < K; g0 += S_GROUP) {
      const int gn = min(S_GROUP, K - g0);
      float *u0 = U0 + lane * n, *u1 = U1 + lane * n, *u2 = U2 + lane * n, *ml = ML + lane * n, *pv = PV + lane * n;
      if (lane < gn) {
        // LU of T - lambda I with partial pivoting (U has two superdiagonals), operands loaded 8 steps ahead
        const int r = g0 + lane;
        const float shift = lam[n - 1 - r];
        float cd = d[0] - shift, cs = n > 1 ? e[0] : 0.0f;
        for (int i0 = 0; i0 < n - 1; i0 += 8) {
          float dd[8], ee[9];
#pragma unroll
          for (int u = 0; u < 8; ++u) dd[u] = i0 + 1 + u < n ? d[i0 + 1 + u] : 0.0f;
#pragma unroll
          for (int u = 0; u < 9; ++u) ee[u] = i0 + u < n ? e[i0 + u] : 0.0f;
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int i = i0 + u;
            if (i < n - 1) {
              const float sub = ee[u], nd = dd[u] - shift, ns = ee[u + 1];  // e[n-1] = 0
              const bool sw = fabsf(cd) < fabsf(sub);
              const float piv0 = sw ? sub : cd;
              const float piv = fabsf(piv0) < pert ? (sw ? pert : (piv0 < 0.0f ? -pert : pert)) : piv0;
              const float rp = fast_rcp(piv);
              const float l = (sw ? cd : sub) * rp;
              u0[i] = rp;
              u1[i] = sw ? nd : cs;
              u2[i] = sw ? ns : 0.0f;
              pv[i] = sw ? 1.0f : 0.0f;
              ml[i] = l;
              const float ncd = sw ? cs - l * nd : nd - l * cs;
              cs = sw ? -l * ns : ns;
              cd = ncd;
            }
          }
        }
        u0[n - 1] = fast_rcp((fabsf(cd) < pert) ? (cd < 0.0f ? -pert : pert) : cd);
        float *x = X + r * n;
        for (int i = 0; i < n; ++i) {
          const uint32_t hsh = (static_cast<uint32_t>(i + 1) * 2654435761u) ^ (static_cast<uint32_t>(r + 1) * 2246822519u);
          x[i] = 0.5f + static_cast<float>((hsh >> 8) & 0xFFFFu) * (1.0f / 65536.0f);
        }
      }
      for (int it = 0; it < S_INV_ITERS; ++it) {
        if (lane < gn) {
          float *x = X + (g0 + lane) * n;
          // forward: row interchanges and L
          float cur = x[0];
          for (int i0 = 0; i0 < n - 1; i0 += 8) {
            float xn[8], pw[8], mw[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const bool in = i0 + u < n - 1;
              xn[u] = in ? x[i0 + u + 1] : 0.0f;
              pw[u] = in ? pv[i0 + u] : 0.0f;
              mw[u] = in ? ml[i0 + u] : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              if (i0 + u < n - 1) {
                const bool sw = pw[u] != 0.0f;
                const float lo_ = sw ? xn[u] : cur, hi_ = sw ? cur : xn[u];
                x[i0 + u] = lo_;
                cur = hi_ - mw[u] * lo_;
              }
            }
          }
          x[n - 1] = cur;
          // backward: U (diagonal stored inverted)
          float x1 = cur * u0[n - 1], x2 = 0.0f;
          x[n - 1] = x1;
          for (int i0 = n - 2; i0 >= 0; i0 -= 8) {
            float xv[8], a0[8], a1[8], a2[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const bool in = i0 - u >= 0;
              xv[u] = in ? x[i0 - u] : 0.0f;
              a0[u] = in ? u0[i0 - u] : 0.0f;
              a1[u] = in ? u1[i0 - u] : 0.0f;
              a2[u] = in ? u2[i0 - u] : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              if (i0 - u >= 0) {
                const float v = (xv[u] - a1[u] * x1 - a2[u] * x2) * a0[u];
                x[i0 - u] = v;
                x2 = x1;
                x1 = v;
              }
            }
          }
        }
        __syncwarp();
        for (int r = g0; r < g0 + gn; ++r) {
          float *x = X + r * n;
          for (int q = 0; q < r; ++q) {
            const float *y = X + q * n;
            float part2 = 0.0f;
            for (int i = lane; i < n; i += 32) part2 += x[i] * y[i];
            const float dot = wsum(part2);
            for (int i = lane; i < n; i += 32) x[i] -= dot * y[i];
            __syncwarp();
          }
          float part2 = 0.0f;
          for (int i = lane; i < n; i += 32) part2 += x[i] * x[i];
          const float nrm2 = wsum(part2);
          const float inv = nrm2 > 0.0f ? rsqrtf(nrm2) : 0.0f;
          for (int i = lane; i < n; i += 32) x[i] *= inv;
          __syncwarp();
        }
      }
    }
  }
  __syncthreads();

  // ---- 6./7. back-transform (one vector per warp), un-whiten, projected weights ----
  float lam_bar = 0.0f;
  if (a.shrink && K < n) {
    for (int i = 0; i < n - K; ++i) lam_bar += lam[i];
    lam_bar /= static_cast<float>(n - K);
  }
  for (int r0 = 0; r0 < K; r0 += S_VEC) {
    const int rn = min(S_VEC, K - r0);
    if (warp < rn) {
      const float *x = X + (r0 + warp) * n;
      float2 z[NPL];
#pragma unroll
      for (int q = 0; q < NPL; ++q) z[q] = make_float2(lane + 32 * q < n ? x[lane + 32 * q] : 0.0f, 0.0f);
      for (int k = n - 2; k >= 0; --k) {
        const float2 tau = taus[k];
        if (tau.x == 0.0f && tau.y == 0.0f) continue;
        // v_(k+1) = 1, v_i = A[k][i] for i > k + 1 (kept in the upper triangle)
        const float2 *urow = A + (size_t)k * ld;
        float2 v[NPL];
        float dre = 0.0f, dim = 0.0f;  // conj(v) z
#pragma unroll
        for (int q = 0; q < NPL; ++q) {
          const int i = lane + 32 * q;
          v[q] = i > k + 1 && i < n ? urow[i] : make_float2(i == k + 1 ? 1.0f : 0.0f, 0.0f);
          dre += v[q].x * z[q].x + v[q].y * z[q].y;
          dim += v[q].x * z[q].y - v[q].y * z[q].x;
        }
        wsum2(dre, dim);
        const float2 sc = cmul(tau, make_float2(dre, dim));
#pragma unroll
        for (int q = 0; q < NPL; ++q)
          z[q] = make_float2(z[q].x - (sc.x * v[q].x - sc.y * v[q].y), z[q].y - (sc.x * v[q].y + sc.y * v[q].x));
      }
      if (!a.shrink) {
        // u = D^1/2 z / |D^1/2 z| (un-whitened, unit norm)
        float part = 0.0f;
#pragma unroll
        for (int q = 0; q < NPL; ++q) {
          const float sq = lane + 32 * q < n ? sd[lane + 32 * q] : 0.0f;
          z[q] = make_float2(z[q].x * sq, z[q].y * sq);
          part += z[q].x * z[q].x + z[q].y * z[q].y;
        }
        const float nrm2 = wsum(part);
        const float inv = nrm2 > 0.0f ? rsqrtf(nrm2) : 0.0f;
#pragma unroll
        for (int q = 0; q < NPL; ++q) z[q] = make_float2(z[q].x * inv, z[q].y * inv);
      }
#pragma unroll
      for (int q = 0; q < NPL; ++q)
        if (lane + 32 * q < n) Z[warp * n + lane + 32 * q] = z[q];
    }
    __syncthreads();
    // c_(v,m) = wgt_v (W_m . z_v) for the pass's vectors and every beam: g2 lanes per
    // (v, m), each summing i = sub (mod g2), reduced by shuffles
    {
      const int npair = rn * B;
      int g2 = 1;
      while (g2 < 32 && 2 * g2 * npair <= NT) g2 *= 2;
      for (int pbase = 0; pbase < npair * g2; pbase += NT) {
        const int pt = (pbase + tid) / g2, sub2 = (pbase + tid) - pt * g2;
        float2 acc = make_float2(0.0f, 0.0f);
        if (pt < npair) {
          const int v = pt / B, mm = pt - v * B;
          const float2 *wr = W0 + mm * n, *zv = Z + v * n;
          for (int i = sub2; i < n; i += g2) {
            const float2 t = cmul(wr[i], zv[i]);
            acc.x += t.x;
            acc.y += t.y;
          }
        }
        for (int o = 1; o < g2; o <<= 1) {
          acc.x += __shfl_xor_sync(FULL, acc.x, o);
          acc.y += __shfl_xor_sync(FULL, acc.y, o);
        }
        if (pt < npair && sub2 == 0) {
          const int v = pt / B, mm = pt - v * B;
          float wgt = 1.0f;
          if (a.shrink) {
            const float lk = lam[n - 1 - (r0 + v)];
            wgt = 1.0f - (lk > 0.0f ? lam_bar / lk : 0.0f);
          }
          coef[v * SB_MAX + mm] = make_float2(wgt * acc.x, wgt * acc.y);
        }
      }
    }
    __syncthreads();
    // Wp_m -= sum_v c_(v,m) conj(z_v)
    {
      int mm = tid / n, i = tid - (tid / n) * n;  // element ee = mm n + i, advanced by NT
      const int dm = NT / n, dii = NT - (NT / n) * n;
      for (int ee = tid; ee < B * n; ee += NT) {
        float2 w = Wp[ee];
        for (int v = 0; v < rn; ++v) {
          const float2 t = cmulc(coef[v * SB_MAX + mm], Z[v * n + i]);  // c conj(z_i)
          w.x -= t.x;
          w.y -= t.y;
        }
        Wp[ee] = w;
        i += dii;
        mm += dm;
        if (i >= n) {
          i -= n;
          ++mm;
        }
      }
    }
    __syncthreads();
  }
  float2 *we = mt.we;
  for (int ee = tid; ee < B * n; ee += NT) {
    const int col = ee - (ee / n) * n;
    we[ee] = cmul(W0[ee], fac[col]);
    we[B * n + ee] = cmul(Wp[ee], fac[col]);
  }
}

// One CTA per matrix, or a grid of at most one resident wave walking the
// device list (its count is known only on the device) or the item range
template <int NT, int NPL>
__global__ void __launch_bounds__(NT, NT == 128 ? 6 : 1) sf_eig_small_kernel(const SmallEigArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int count = a.list ? *a.list_count : (a.items ? a.n_items : 2 * a.C);
  for (int slot = blockIdx.x; slot < count; slot += gridDim.x) {
    SmallMat mt;
    if (a.items) {
      const SfEigItem it = a.items[a.first_item + slot];
      mt.n = it.n;
      mt.vin = a.vis + it.vis_off + 6 * it.pol;
      mt.fac = a.factors ? a.factors + it.factor_off : nullptr;
      mt.w = a.weights + it.weight_off;
      mt.we = a.weff + it.weff_off;
      mt.ev = a.evals ? a.evals + it.eval_off : nullptr;
      mt.cnt = a.counts ? a.counts + it.count_idx : nullptr;
      mt.kfix = a.fixed_counts ? a.fixed_counts[it.count_idx] : 0;
    } else {
      const int bt = a.list ? a.list[slot] : slot;  // c * 2 + p
      const int c = bt >> 1, n = a.R;
      mt.n = n;
      mt.vin = a.vis + (size_t)c * a.NBL * 8 + 6 * (bt & 1);
      mt.fac = a.factors + (size_t)bt * n;
      mt.w = a.weights + (size_t)bt * a.B * n;
      mt.we = a.weff + (size_t)bt * 2 * a.B * n;
      mt.ev = a.evals ? a.evals + (size_t)bt * n : nullptr;
      mt.cnt = a.counts ? a.counts + bt : nullptr;
      mt.kfix = a.fixed_counts ? a.fixed_counts[c] : 0;
    }
    eig_small_one<NT, NPL>(a, mt, smem);
    __syncthreads();  // the next matrix reuses the shared memory
  }
}

}  // namespace

namespace {

// the configuration for matrices of at most n_max receivers: four warps and two rows per lane up
// to 64, sixteen warps and four rows per lane up to 128
struct SmallLaunch {
  const void *fn;
  int nt;
};
SmallLaunch small_config(int n_max) {
  if (n_max <= 64) return {reinterpret_cast<const void *>(sf_eig_small_kernel<128, 2>), 128};
  return {reinterpret_cast<const void *>(sf_eig_small_kernel<512, 4>), 512};
}

bool small_fits(int n_max, int B) {
  return n_max >= 2 && n_max <= SN_MAX && B <= SB_MAX && s_region(n_max, B).total <= (size_t)sf_device_max_smem();
}

// grid: every matrix its own CTA (count_hint > 0 and no cap), or at most one resident wave
cudaError_t launch_small(const SmallEigArgs &a, int n_max, int count, bool one_wave, int num_sms, cudaStream_t stream) {
  const SmallLaunch cfg = small_config(n_max);
  const size_t smem = s_region(n_max, a.B).total;
  cudaError_t e = sf_smem_optin(cfg.fn, smem);
  if (e != cudaSuccess) return e;
  int grid = count;
  if (one_wave) {
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cfg.fn, cfg.nt, smem);
    if (e != cudaSuccess) return e;
    grid = std::min(count, std::max(1, per_sm) * num_sms);
  }
  if (grid <= 0) return cudaSuccess;
  if (cfg.nt == 128)
    sf_eig_small_kernel<128, 2><<<grid, 128, smem, stream>>>(a);
  else
    sf_eig_small_kernel<512, 4><<<grid, 512, smem, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace

int sf_eig_small_supported(const sf_plan *p) { return small_fits(p->R, p->B); }

cudaError_t sf_launch_eig_small(const sf_plan *p, const int32_t *vis, int k_rule, float delta, int shrink,
                                float *evals, int32_t *counts, const int32_t *list, const int32_t *list_count,
                                cudaStream_t stream) {
  SmallEigArgs a;
  a.list = list;
  a.list_count = list_count;
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
  a.n_items = 0;
  // one CTA per matrix; the device list (whose count only the device knows) by one resident wave
  return launch_small(a, p->R, 2 * p->C, list != nullptr, p->num_sms, stream);
}

int sf_eig_small_items_supported(int n_max, int B) { return small_fits(n_max, B); }

cudaError_t sf_launch_eig_small_items(const SfEigItem *items, int first, int count, int n_max, int B,
                                      const int32_t *vis, const float2 *factors, const __half2 *weights,
                                      const int32_t *fixed_counts, int k_rule, float delta, int shrink,
                                      float *evals, int32_t *counts, float2 *weff, uint32_t *status, int num_sms,
                                      cudaStream_t stream) {
  if (count <= 0) return cudaSuccess;
  if (!small_fits(n_max, B)) return cudaErrorInvalidValue;
  SmallEigArgs a;
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
  a.list = nullptr;
  a.list_count = nullptr;
  a.items = items;
  a.first_item = first;
  a.n_items = count;
  return launch_small(a, n_max, count, true, num_sms, stream);
}
