// Learned subspace proposer: the hand-written BF16 tensor-core kernels that
// train and run a 3-layer MLP (1344 -> 512 -> 512 -> 288) mapping a whitened,
// trace-normalised covariance to k <= 4 complex 36-vectors (a warm start for
// the interference subspace), plus its feature, target, loss, bias-gradient
// and Adam kernels.  The warm-started Rayleigh-Ritz refinement and the
// residual-gated fallback live in sf_proposer.cu.
//
// GEMM: C[M][N] = sum_k A(m, k) B(n, k), A and B bf16, each stored K-major
// ([M][K] / [N][K]) or MN-major ([K][M] / [K][N]) -- the forward pass is
// X W^T (both K-major), the data-gradient passes dY W (B MN-major) and the
// weight-gradient passes dY^T H (both MN-major).  One CTA per 128 x 128 output
// tile (split over K for the weight gradients): warp 0 streams 64-deep K
// blocks of both operands by 2-D TMA (128-byte swizzle) into a four-stage
// ring, warp 1 issues tcgen05.mma kind::f16 (bf16 in, fp32 accumulation in
// tensor memory), warps 4-7 drain the accumulator through a fused epilogue:
//   0  bf16 out = relu(acc + bias)          (hidden layers)
//   1  fp32 out = acc + bias                (output layer)
//   2  bf16 out = acc x [mask > 0]          (back through a ReLU)
//   3  fp32 out += acc (atomic)             (split-K weight gradients)
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cstdio>
#include <cstring>

#include "sf_common.cuh"
#include "sf_plan.cuh"

namespace {

constexpr int GT = 128;       // output tile edge (M and N)
constexpr int GK = 64;        // K block (one 128-byte swizzle row of bf16)
constexpr int GSTAGES = 4;
constexpr int GTHREADS = 256;
constexpr uint32_t TILE_BYTES = GT * GK * 2;  // 16 KB per operand per stage
constexpr uint32_t GHEADER = 1024;

struct GemmArgs {
  int M, N, K;
  int a_mn, b_mn;
  int k_per_split;
  int mode;
  const float *bias;
  const __nv_bfloat16 *mask;
  int ldm;
  void *out;
  int ldo;
  uint32_t *status;
};

struct __align__(8) GemmHeader {
  uint64_t full[GSTAGES], empty[GSTAGES];
  uint64_t acc_full;
  uint32_t tmem_base;
  int abort;
};

__device__ __forceinline__ uint64_t gdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((addr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
  d |= static_cast<uint64_t>(1u) << 46;
  d |= static_cast<uint64_t>(2u) << 61;
  return d;
}

// one operand's K block: K-major = one [128 rows][64 k] box; MN-major = two
// [64 k rows][64 mn] boxes (mn atoms 8 KB apart)
__device__ __forceinline__ void load_operand(uint8_t *dst, const void *tmap, bool mn_major, int mn0, int k0,
                                             uint64_t *bar) {
  if (mn_major) {
    tma_load_2d(dst, tmap, mn0, k0, bar);
    tma_load_2d(dst + TILE_BYTES / 2, tmap, mn0 + 64, k0, bar);
  } else {
    tma_load_2d(dst, tmap, k0, mn0, bar);
  }
}

__global__ void __launch_bounds__(GTHREADS, 1)
    sf_gemm_bf16_kernel(const __grid_constant__ CUtensorMap tma, const __grid_constant__ CUtensorMap tmb,
                        const GemmArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  GemmHeader &h = *reinterpret_cast<GemmHeader *>(smem);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t sbase = smem_u32(smem);
  const uint32_t ring = (sbase + GHEADER + 1023u) & ~1023u;
  uint8_t *ring_ptr = smem + (ring - sbase);
  const int n0 = blockIdx.x * GT, m0 = blockIdx.y * GT;
  const int kb0 = blockIdx.z * a.k_per_split;
  const int kb1 = min(a.K, kb0 + a.k_per_split);
  const int nkb = kb1 > kb0 ? (kb1 - kb0 + GK - 1) / GK : 0;

  if (tid == 0) {
    for (int s = 0; s < GSTAGES; ++s) {
      mbar_init(&h.full[s], 1);
      mbar_init(&h.empty[s], 1);
    }
    mbar_init(&h.acc_full, 1);
    h.abort = 0;
    fence_mbarrier_init();
  }
  if (warp == 1) {
    tmem_alloc(&h.tmem_base, GT);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  volatile int *abort_flag = &h.abort;

  if (warp == 0) {
    if (lane == 0) {
      bool ok = true;
      for (int kb = 0; kb < nkb && ok; ++kb) {
        const int s = kb % GSTAGES;
        ok = mbar_wait(&h.empty[s], ((kb / GSTAGES) & 1) ^ 1, abort_flag, 20000);
        if (!ok) break;
        mbar_arrive_expect_tx(&h.full[s], 2 * TILE_BYTES);
        uint8_t *st = ring_ptr + s * 2 * TILE_BYTES;
        load_operand(st, &tma, a.a_mn, m0, kb0 + kb * GK, &h.full[s]);
        load_operand(st + TILE_BYTES, &tmb, a.b_mn, n0, kb0 + kb * GK, &h.full[s]);
      }
      const int begin = nkb > GSTAGES ? nkb - GSTAGES : 0;
      for (int kb = begin; kb < nkb; ++kb) mbar_wait_drain(&h.full[kb % GSTAGES], (kb / GSTAGES) & 1);
      if (!ok) atomicOr(a.status, SF_DEVERR_TIMEOUT_TMA);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // bf16 A and B (format 1), fp32 D; bit 15 / 16: operand MN-major
      const uint32_t idesc = umma_idesc_f16_f32(GT, GT) | (1u << 7) | (1u << 10) | (a.a_mn ? 1u << 15 : 0u) |
                             (a.b_mn ? 1u << 16 : 0u);
      bool failed = false;
      for (int kb = 0; kb < nkb; ++kb) {
        const int s = kb % GSTAGES;
        const bool ok = mbar_wait(&h.full[s], (kb / GSTAGES) & 1, abort_flag, 20000);
        failed |= !ok;
        tc_fence_after();
        const uint32_t sa = ring + s * 2 * TILE_BYTES, sb = sa + TILE_BYTES;
        // K-major: rows of 128 B, 8-row groups 1024 B apart, a 16-deep K step = 32 B;
        // MN-major: 64-wide mn atoms 8 KB apart, 8-row K groups 1024 B apart, a K step = 2 KB
        const uint64_t ad = a.a_mn ? gdesc(sa, TILE_BYTES / 2, 1024) : gdesc(sa, 16, 1024);
        const uint64_t bd = a.b_mn ? gdesc(sb, TILE_BYTES / 2, 1024) : gdesc(sb, 16, 1024);
        if (ok) {
#pragma unroll
          for (int ks = 0; ks < GK / 16; ++ks) {
            const uint32_t da = a.a_mn ? (ks * 2048) >> 4 : (ks * 32) >> 4;
            const uint32_t db = a.b_mn ? (ks * 2048) >> 4 : (ks * 32) >> 4;
            umma_f16(h.tmem_base, ad + da, bd + db, idesc, (kb == 0 && ks == 0) ? 0u : 1u);
          }
        }
        umma_commit(&h.empty[s]);
      }
      umma_commit(&h.acc_full);
      if (failed) atomicOr(a.status, SF_DEVERR_TIMEOUT_MMA);
    }
  } else if (warp >= 4) {
    const int q = warp - 4;
    const bool ok = mbar_wait(&h.acc_full, 0, abort_flag, 20000);
    tc_fence_after();
    const int m = m0 + q * 32 + lane;
    const uint32_t taddr = h.tmem_base + (static_cast<uint32_t>(q * 32) << 16);
    // a row's 16 columns go out as 16-byte stores when the pitch and the chunk allow it
    const bool vec_bf16 = (a.ldo % 8) == 0 && (reinterpret_cast<uintptr_t>(a.out) % 16) == 0;
    const bool vec_f32 = (a.ldo % 4) == 0 && (reinterpret_cast<uintptr_t>(a.out) % 16) == 0;
    const bool vec_mask = a.mask && (a.ldm % 8) == 0 && (reinterpret_cast<uintptr_t>(a.mask) % 16) == 0;
    uint32_t nxt[16];
    tmem_ld16(taddr, nxt);
    for (int cb = 0; cb < GT / 16; ++cb) {
      uint32_t v[16];
      __syncwarp();  // converged for the warp-wide tensor-memory operations
      tmem_wait_ld();
#pragma unroll
      for (int e = 0; e < 16; ++e) v[e] = nxt[e];
      if (cb + 1 < GT / 16) tmem_ld16(taddr + (cb + 1) * 16, nxt);  // next chunk in flight
      if (!ok || nkb == 0 || m >= a.M) continue;
      const int nb = n0 + cb * 16;
      if (nb >= a.N) continue;
      const bool full = nb + 16 <= a.N;
      float x[16];
#pragma unroll
      for (int e = 0; e < 16; ++e) x[e] = __uint_as_float(v[e]);
      if (a.mode == 3) {
        float *o = static_cast<float *>(a.out) + (size_t)m * a.ldo + nb;
#pragma unroll
        for (int e = 0; e < 16; ++e)
          if (nb + e < a.N) atomicAdd(o + e, x[e]);
        continue;
      }
      if ((a.mode == 0 || a.mode == 1) && a.bias) {
#pragma unroll
        for (int e = 0; e < 16; ++e) x[e] += nb + e < a.N ? a.bias[nb + e] : 0.0f;
      }
      if (a.mode == 1) {
        float *o = static_cast<float *>(a.out) + (size_t)m * a.ldo + nb;
        if (full && vec_f32) {
#pragma unroll
          for (int e = 0; e < 16; e += 4) *reinterpret_cast<float4 *>(o + e) = make_float4(x[e], x[e + 1], x[e + 2], x[e + 3]);
        } else {
#pragma unroll
          for (int e = 0; e < 16; ++e)
            if (nb + e < a.N) o[e] = x[e];
        }
        continue;
      }
      if (a.mode == 0) {
#pragma unroll
        for (int e = 0; e < 16; ++e) x[e] = fmaxf(x[e], 0.0f);
      } else {  // mode 2: back through a ReLU
        const __nv_bfloat16 *mk = a.mask + (size_t)m * a.ldm + nb;
        if (full && vec_mask) {
          uint4 mw[2];
          mw[0] = *reinterpret_cast<const uint4 *>(mk);
          mw[1] = *reinterpret_cast<const uint4 *>(mk + 8);
          const __nv_bfloat16 *mb = reinterpret_cast<const __nv_bfloat16 *>(mw);
#pragma unroll
          for (int e = 0; e < 16; ++e) x[e] = __bfloat162float(mb[e]) > 0.0f ? x[e] : 0.0f;
        } else {
#pragma unroll
          for (int e = 0; e < 16; ++e)
            if (nb + e < a.N) x[e] = __bfloat162float(mk[e]) > 0.0f ? x[e] : 0.0f;
        }
      }
      __nv_bfloat16 *o = static_cast<__nv_bfloat16 *>(a.out) + (size_t)m * a.ldo + nb;
      if (full && vec_bf16) {
        uint4 pk[2];
        uint32_t *pw = reinterpret_cast<uint32_t *>(pk);
#pragma unroll
        for (int e = 0; e < 16; e += 2) {
          const __nv_bfloat162 b2 = __floats2bfloat162_rn(x[e], x[e + 1]);
          pw[e / 2] = *reinterpret_cast<const uint32_t *>(&b2);
        }
        *reinterpret_cast<uint4 *>(o) = pk[0];
        *reinterpret_cast<uint4 *>(o + 8) = pk[1];
      } else {
#pragma unroll
        for (int e = 0; e < 16; ++e)
          if (nb + e < a.N) o[e] = __float2bfloat16_rn(x[e]);
      }
    }
    __syncwarp();
    if (!ok && lane == 0) atomicOr(a.status, SF_DEVERR_TIMEOUT_EPILOGUE);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(h.tmem_base, GT);
  }
}

PFN_cuTensorMapEncodeTiled_v12000 gemm_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// bf16 matrix [rows][ld] whose inner extent is `inner` elements; box
// {64, box_rows} with the 128-byte swizzle
cudaError_t encode_bf16(CUtensorMap *map, const void *base, int inner, int rows, int ld, int box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 encode = gemm_encoder();
  if (!encode) return cudaErrorNotSupported;
  const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// Training helpers
// ---------------------------------------------------------------------------

// Targets and weights from a full eigendecomposition of the whitened covariances:
// the top four eigenvectors (descending eigenvalue) of the whitened matrix,
// largest component real positive, [row][vec][r][re, im]; weight of vector k =
// clamp(1 - median / lambda_k, 0, 1) (noise-only directions carry no weight).
// The eigensolver returns the un-whitened normalised vectors u = D^{1/2} v /
// ||D^{1/2} v||, so v is D^{-1/2} u renormalised.
__global__ void sf_proposer_targets_kernel(const int32_t *vis, const float *evals, const float2 *evecs, int C, int R,
                                           int NBL, float *targets, float *tw) {
  const int row = blockIdx.x;  // c * 2 + p
  const int c = row >> 1, p = row & 1;
  const int lane = threadIdx.x;
  const float *lam = evals + (size_t)row * R;
  for (int k = 0; k < 4; ++k) {
    const int kk = R - 1 - k;
    const float2 *u = evecs + ((size_t)row * R + kk) * R;  // component l of eigenvector kk
    float2 v[4];
    float nrm = 0.0f, best = -1.0f;
    int bi = 0;
    for (int t = 0; t < 4; ++t) {
      const int i = lane + 32 * t;
      v[t] = make_float2(0.0f, 0.0f);
      if (i < R) {
        const int32_t *d = vis + ((((size_t)c * NBL + baseline_of(i, i)) * 2 + p) * 2 + p) * 2;
        const float s = rsqrtf(fmaxf(static_cast<float>(d[0]), 1e-10f));
        v[t] = make_float2(u[i].x * s, u[i].y * s);
        nrm += v[t].x * v[t].x + v[t].y * v[t].y;
      }
    }
    for (int o = 16; o > 0; o >>= 1) nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
    const float inv = nrm > 0.0f ? rsqrtf(nrm) : 0.0f;
    for (int t = 0; t < 4; ++t) {
      v[t].x *= inv;
      v[t].y *= inv;
      const float m2 = v[t].x * v[t].x + v[t].y * v[t].y;
      if (lane + 32 * t < R && m2 > best) {
        best = m2;
        bi = lane + 32 * t;
      }
    }
    // largest component (lowest index on ties) real positive
    for (int o = 16; o > 0; o >>= 1) {
      const float ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    float2 piv = make_float2(0.0f, 0.0f);
    for (int t = 0; t < 4; ++t) {
      const float px = __shfl_sync(0xffffffffu, v[t].x, bi & 31);
      const float py = __shfl_sync(0xffffffffu, v[t].y, bi & 31);
      if ((bi >> 5) == t) piv = make_float2(px, py);
    }
    const float pm = sqrtf(piv.x * piv.x + piv.y * piv.y);
    const float2 ph = pm > 0.0f ? make_float2(piv.x / pm, -piv.y / pm) : make_float2(1.0f, 0.0f);
    for (int t = 0; t < 4; ++t) {
      const int i = lane + 32 * t;
      if (i < R) {
        const float2 x = cmul(v[t], ph);
        float *o = targets + (size_t)row * 8 * R + (size_t)k * 2 * R + 2 * i;
        o[0] = x.x;
        o[1] = x.y;
      }
    }
    if (lane == 0) {
      const float med = 0.5f * (lam[(R - 1) / 2] + lam[R / 2]);
      const float lk = lam[kk];
      tw[row * 4 + k] = lk > 0.0f ? fminf(1.0f, fmaxf(0.0f, 1.0f - med / lk)) : 0.0f;
    }
  }
}

// Phase-invariant distance of each proposed vector y_k to its target t_k
// (|t_k| = 1): min over phi of ||y_k - t_k e^{i phi}||^2 = ||y_k||^2 + 1 -
// 2 |<t_k, y_k>|, weighted by w_k; gradient 2 w_k (y_k - t_k e^{i psi}) / rows
// with psi = arg <t_k, y_k> (a vector is only defined up to its phase, so the
// loss does not ask for one).  One warp per (row, vector); loss += sum / rows.
__global__ void sf_proposer_loss_kernel(const float *y, const float *t, const float *tw, int rows, int width, int R,
                                        __nv_bfloat16 *dy, int lddy, float *loss) {
  const int row = blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nvec = width / (2 * R);
  __shared__ float red[32];
  float part = 0.0f;
  for (int k = warp; k < nvec; k += blockDim.x >> 5) {
    const float *yk = y + (size_t)row * width + k * 2 * R;
    const float *tk = t + (size_t)row * width + k * 2 * R;
    float dr = 0.0f, di = 0.0f, yy = 0.0f;  // <t, y> = sum conj(t) y, ||y||^2
    for (int i = lane; i < R; i += 32) {
      const float yr = yk[2 * i], yi = yk[2 * i + 1], tr = tk[2 * i], ti = tk[2 * i + 1];
      dr += tr * yr + ti * yi;
      di += tr * yi - ti * yr;
      yy += yr * yr + yi * yi;
    }
    for (int o = 16; o > 0; o >>= 1) {
      dr += __shfl_xor_sync(0xffffffffu, dr, o);
      di += __shfl_xor_sync(0xffffffffu, di, o);
      yy += __shfl_xor_sync(0xffffffffu, yy, o);
    }
    const float w = tw[row * 4 + k];
    const float mag = sqrtf(dr * dr + di * di);
    const float cr = mag > 0.0f ? dr / mag : 1.0f, ci = mag > 0.0f ? di / mag : 0.0f;  // e^{i psi}
    if (lane == 0) part += w * (yy + 1.0f - 2.0f * mag);
    const float g = 2.0f * w / static_cast<float>(rows);
    __nv_bfloat16 *dk = dy + (size_t)row * lddy + k * 2 * R;
    for (int i = lane; i < R; i += 32) {
      const float tr = tk[2 * i], ti = tk[2 * i + 1];
      // t e^{i psi}
      const float er = tr * cr - ti * ci, ei = tr * ci + ti * cr;
      dk[2 * i] = __float2bfloat16_rn(g * (yk[2 * i] - er));
      dk[2 * i + 1] = __float2bfloat16_rn(g * (yk[2 * i + 1] - ei));
    }
  }
  // padding columns of dY stay zero
  for (int j = width + threadIdx.x; j < lddy; j += blockDim.x) dy[(size_t)row * lddy + j] = __float2bfloat16_rn(0.0f);
  if (lane == 0) red[warp] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s2 = 0.0f;
    for (int w2 = 0; w2 < (int)(blockDim.x >> 5); ++w2) s2 += red[w2];
    atomicAdd(loss, s2 / static_cast<float>(rows));
  }
}

// db[n] = sum_m dY[m][n] (bf16 dY [rows][ld])
__global__ void sf_column_sums_kernel(const __nv_bfloat16 *dy, int rows, int cols, int ld, float *db) {
  const int n = blockIdx.x * blockDim.y + threadIdx.y;
  if (n >= cols) return;
  float s = 0.0f;
  for (int m = threadIdx.x; m < rows; m += 32) s += __bfloat162float(dy[(size_t)m * ld + n]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (threadIdx.x == 0) db[n] = s;
}

// Adam on fp32 master parameters (bias-corrected, step t >= 1); writes the
// bf16 copy the GEMMs read (w16 may be NULL for biases) and clears the gradient.
__global__ void sf_adam_kernel(float *w, float *g, float *m, float *v, __nv_bfloat16 *w16, int n, float lr, float b1,
                               float b2, float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    w[i] = wi;
    if (w16) w16[i] = __float2bfloat16_rn(wi);
    g[i] = 0.0f;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Launchers (shared with sf_proposer.cu)
// ---------------------------------------------------------------------------
cudaError_t sf_launch_gemm_bf16(int M, int N, int K, const void *A, int lda, int a_mn, const void *B, int ldb, int b_mn,
                                int mode, const float *bias, const void *mask, int ldm, void *out, int ldo, int splits,
                                uint32_t *status, cudaStream_t stream) {
  if (M <= 0 || N <= 0 || K <= 0) return cudaErrorInvalidValue;
  if ((lda * 2) % 16 || (ldb * 2) % 16 || reinterpret_cast<uintptr_t>(A) % 16 || reinterpret_cast<uintptr_t>(B) % 16)
    return cudaErrorInvalidValue;
  CUtensorMap ta, tb;
  // K-major operand: [rows = M (N)][K], box 64 k x 128 rows; MN-major: [rows = K][M (N)], box 64 mn x 64 k
  cudaError_t e = a_mn ? encode_bf16(&ta, A, M, K, lda, GK) : encode_bf16(&ta, A, K, M, lda, GT);
  if (e != cudaSuccess) return e;
  e = b_mn ? encode_bf16(&tb, B, N, K, ldb, GK) : encode_bf16(&tb, B, K, N, ldb, GT);
  if (e != cudaSuccess) return e;
  GemmArgs a;
  a.M = M;
  a.N = N;
  a.K = K;
  a.a_mn = a_mn;
  a.b_mn = b_mn;
  splits = splits < 1 ? 1 : splits;
  a.k_per_split = ((K + splits - 1) / splits + GK - 1) / GK * GK;
  a.mode = mode;
  a.bias = bias;
  a.mask = static_cast<const __nv_bfloat16 *>(mask);
  a.ldm = ldm;
  a.out = out;
  a.ldo = ldo;
  a.status = status;
  const size_t smem = GHEADER + 1024 + (size_t)GSTAGES * 2 * TILE_BYTES;
  e = sf_smem_optin(reinterpret_cast<const void *>(sf_gemm_bf16_kernel), smem);
  if (e != cudaSuccess) return e;
  const dim3 grid((N + GT - 1) / GT, (M + GT - 1) / GT, (K + a.k_per_split - 1) / a.k_per_split);
  sf_gemm_bf16_kernel<<<grid, GTHREADS, smem, stream>>>(ta, tb, a);
  return cudaGetLastError();
}

cudaError_t sf_launch_proposer_targets(const int32_t *vis, const float *evals, const float *evecs, int C, int R, float *targets,
                                       float *tw, cudaStream_t stream) {
  if (R > 128) return cudaErrorInvalidValue;
  sf_proposer_targets_kernel<<<2 * C, 32, 0, stream>>>(vis, evals, reinterpret_cast<const float2 *>(evecs), C, R,
                                                        R * (R + 1) / 2, targets, tw);
  return cudaGetLastError();
}

cudaError_t sf_launch_proposer_loss(const float *y, const float *t, const float *tw, int rows, int width, int R,
                                    void *dy, int lddy, float *loss, cudaStream_t stream) {
  sf_proposer_loss_kernel<<<rows, 128, 0, stream>>>(y, t, tw, rows, width, R, static_cast<__nv_bfloat16 *>(dy), lddy,
                                                    loss);  // four warps: one per proposed vector
  return cudaGetLastError();
}

cudaError_t sf_launch_column_sums(const void *dy, int rows, int cols, int ld, float *db, cudaStream_t stream) {
  const dim3 block(32, 8);
  sf_column_sums_kernel<<<(cols + 7) / 8, block, 0, stream>>>(static_cast<const __nv_bfloat16 *>(dy), rows, cols, ld,
                                                              db);
  return cudaGetLastError();
}

cudaError_t sf_launch_adam(float *w, float *g, float *m, float *v, void *w16, int n, float lr, int step,
                           cudaStream_t stream) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f / (1.0f - powf(b1, static_cast<float>(step)));
  const float c2 = 1.0f / (1.0f - powf(b2, static_cast<float>(step)));
  sf_adam_kernel<<<(n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024, 256, 0, stream>>>(
      w, g, m, v, static_cast<__nv_bfloat16 *>(w16), n, lr, b1, b2, 1e-8f, c1, c2);
  return cudaGetLastError();
}
