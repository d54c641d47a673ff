// Beam spectra: the two spectra tails the reference runs on its beams,
// computed from the fp16 beams of the beamformer in one read each.
//
// sf_beam_spectra_kernel - LambdaGPUPipeline's tail
// (include/spatial/pipeline/lambda_gpu_pipeline.hpp:522-531): a forward FFT of
// each (channel, pol, beam) series over the whole integration (cuFFT plan of
// length T = P Tp, :814-817 / :944-947), then detect_and_downsample_fft
// (include/spatial/spatial.cuh:795-848): bin g of the output is the mean of
// |X|^2 over the D bins g D .. g D + D - 1, NaN bins skipped, 0 if all are NaN.
// The reference permutes its fp32 beams into a cuFFT input tensor, transforms
// out of place and reads the spectrum back; here one CTA loads one series once
// (T fp16 pairs), transforms it in shared memory (Stockham autosort, radix-16
// passes, the first pass reading global memory directly) and writes only the
// T / D detected bins.
//
// sf_packet_spectra_kernel - the adaptive pipeline's tail
// (include/spatial/pipeline/lambda_adaptive_beamformed_spectra_pipeline.hpp:808-848):
// a Tp-point FFT of every packet (plan :1046-1050), the fine-channel reorder
// and trim (:816-833: upper half without its first `trim` bins, then lower
// half without its last `trim`), and sum_fft_over_packets (spatial.cuh:1508-1567):
// the magnitude |X| summed over the P packets.  The reference makes six passes
// over fp32 copies (permute, FFT, permute, two half copies, permute) before an
// atomic sum; here one warp streams one series through shared memory
// (cp.async, double-buffered), one lane per packet transforms its Tp samples in
// registers and accumulates |X|, and the 32 lanes' partial sums are added in a
// fixed order, so the result is deterministic.
//
// Both transforms are the unnormalised forward DFT X[k] = sum_n x[n] W_N^{nk},
// W_N = exp(-2 pi i / N), in fp32, with twiddles rounded from double precision
// on the host.
#include <cmath>
#include <cstring>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "sf_common.cuh"
#include "sf_plan.cuh"

namespace {

// W_64^k = c[k] + i s[k] (c = cos(2 pi k / 64), s = -sin(2 pi k / 64)), passed by
// value in the launch parameters: after unrolling every index is a constant, so
// each twiddle is a constant-bank operand.
struct Tw64 {
  float c[64];
  float s[64];
};

Tw64 make_tw64() {
  Tw64 t;
  const double pi = 3.14159265358979323846;
  for (int k = 0; k < 64; ++k) {
    t.c[k] = static_cast<float>(std::cos(2.0 * pi * k / 64.0));
    t.s[k] = static_cast<float>(-std::sin(2.0 * pi * k / 64.0));
  }
  return t;
}

const Tw64 &tw64() {
  static const Tw64 t = make_tw64();
  return t;
}

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n >> 1); }

__host__ __device__ constexpr int bitrev(int i, int bits) {
  int r = 0;
  for (int b = 0; b < bits; ++b) r |= ((i >> b) & 1) << (bits - 1 - b);
  return r;
}

// d W_64^e for 0 <= e < 32 (e is a constant after unrolling).
SF_DEVICE float2 tw64_mul(float2 d, int e, const Tw64 &w) {
  if (e == 0) return d;
  if (e == 16) return make_float2(d.y, -d.x);  // W_64^16 = -i
  return make_float2(d.x * w.c[e] - d.y * w.s[e], d.x * w.s[e] + d.y * w.c[e]);
}

// In-register radix-2 decimation-in-frequency DFT of N = 2^LOG2N <= 64 values;
// the result is in bit-reversed order: v[bitrev(k)] = X[k].
template <int LOG2N>
SF_DEVICE void dft_reg(float2 *v, const Tw64 &w) {
  constexpr int N = 1 << LOG2N;
#pragma unroll
  for (int st = 0; st < LOG2N; ++st) {
    const int half = N >> (st + 1);
#pragma unroll
    for (int base = 0; base < N; base += 2 * half) {
#pragma unroll
      for (int k = 0; k < half; ++k) {
        const float2 a = v[base + k], b = v[base + k + half];
        v[base + k] = make_float2(a.x + b.x, a.y + b.y);
        v[base + k + half] = tw64_mul(make_float2(a.x - b.x, a.y - b.y), k * (32 / half), w);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Whole-integration spectra (LambdaGPUPipeline)
// ---------------------------------------------------------------------------
constexpr int BS_THREADS = 256;
constexpr int BS_MIN_LOG2T = 6;
constexpr int BS_MAX_LOG2T = 14;

struct BeamSpecArgs {
  const __half2 *beams;  // [S][T]
  const float2 *tw;      // per-pass twiddles, see sf_fill_spectra_twiddles
  float *out;            // [S][T / D]
  int S, D;
  Tw64 w;
};

// Shared-memory position of element i: xor of bits 4..7 into bits 0..3, so
// that the strided writes of the early passes (stride R * NS) spread over all
// banks while contiguous runs stay contiguous within 16-element groups.
SF_DEVICE int bs_swz(int i) { return i ^ ((i >> 4) & 15); }

// One Stockham autosort pass of radix R: butterfly j < T / R reads
// x[j + r T / R] (r < R), multiplies by W_{NS R}^{r (j mod NS)}, transforms over
// r and writes x[(j / NS) NS R + j mod NS + r NS].  In place: every value is in
// registers before the barrier, and written after it.  The first pass reads
// the fp16 series from global memory instead.  The pass's twiddles sit at
// tw[NS - 1 + (r - 1) NS + j mod NS], so the lanes of a warp read consecutive
// entries.
template <int T, int R, int NS>
SF_DEVICE void stockham_pass(float2 *x, const __half2 *src, const float2 *tw, const Tw64 &w) {
  constexpr int LOG2R = ilog2c(R);
  constexpr int NB = T / R;
  constexpr int PER = (NB + BS_THREADS - 1) / BS_THREADS;
  float2 v[PER][R];
#pragma unroll
  for (int b = 0; b < PER; ++b) {
    const int j = threadIdx.x + b * BS_THREADS;
    if (NB % BS_THREADS == 0 || j < NB) {
      // with NB a multiple of 256, r NB leaves bits 4..7 alone:
      // bs_swz(j + r NB) = bs_swz(j) + r NB
      const int js = bs_swz(j);
#pragma unroll
      for (int r = 0; r < R; ++r)
        v[b][r] = NS == 1 ? __half22float2(src[j + r * NB])
                          : x[NB % 256 == 0 ? js + r * NB : bs_swz(j + r * NB)];
    }
  }
  if (NS > 1) __syncthreads();
#pragma unroll
  for (int b = 0; b < PER; ++b) {
    const int j = threadIdx.x + b * BS_THREADS;
    if (NB % BS_THREADS == 0 || j < NB) {
      const int jm = j & (NS - 1);
      if (NS > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) v[b][r] = cmul(v[b][r], __ldg(tw + (NS - 1) + (r - 1) * NS + jm));
      }
      dft_reg<LOG2R>(v[b], w);
      const int base = (j - jm) * R + jm;
      // the swizzle of base + k NS for the pass shapes of the radix-16 plan:
      // NS = 1 (base a multiple of 16): bs_swz(base) ^ k; NS = R = 16 (base =
      // 256 m + jm): (base ^ k) + 16 k; NS a multiple of 256: bs_swz(base) + k NS
      const int bs = bs_swz(base);
#pragma unroll
      for (int k = 0; k < R; ++k) {
        int pos;
        if constexpr (NS == 1 && R == 16) pos = bs ^ k;
        else if constexpr (NS == 16 && R == 16) pos = (base ^ k) + 16 * k;
        else if constexpr (NS % 256 == 0) pos = bs + k * NS;
        else pos = bs_swz(base + k * NS);
        x[pos] = v[b][bitrev(k, LOG2R)];
      }
    }
  }
  __syncthreads();
}

template <int T, int NS>
SF_DEVICE void stockham_fft(float2 *x, const __half2 *src, const float2 *tw, const Tw64 &w) {
  if constexpr (NS < T) {
    constexpr int R = (T / NS) >= 16 ? 16 : (T / NS);
    stockham_pass<T, R, NS>(x, src, tw, w);
    stockham_fft<T, NS * R>(x, src, tw, w);
  }
}

template <int LOG2T>
__global__ void __launch_bounds__(BS_THREADS) sf_beam_spectra_kernel(const BeamSpecArgs a) {
  constexpr int T = 1 << LOG2T;
  extern __shared__ __align__(16) float2 xs[];
  const int s = blockIdx.x;
  stockham_fft<T, 1>(xs, a.beams + (size_t)s * T, a.tw, a.w);

  // |X|^2 >= 0 (or +inf), so a group's plain sum is NaN exactly when one of
  // its bins is: the plain sum serves every group without NaN bins (same
  // order, same count D), and only a NaN sum takes the NaN-skipping mean
  const int D = a.D, G = T / D;
  float *out = a.out + (size_t)s * G;
  if (D >= 32) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int g = warp; g < G; g += BS_THREADS / 32) {
      float sum = 0.f;
      for (int i = lane; i < D; i += 32) {
        const float2 X = xs[bs_swz(g * D + i)];
        sum += X.x * X.x + X.y * X.y;
      }
#pragma unroll
      for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
      if (isnan(sum)) {  // warp-uniform after the reduction
        sum = 0.f;
        int cnt = 0;
        for (int i = lane; i < D; i += 32) {
          const float2 X = xs[bs_swz(g * D + i)];
          const float pw = X.x * X.x + X.y * X.y;
          if (!isnan(pw)) {
            sum += pw;
            ++cnt;
          }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
          sum += __shfl_xor_sync(0xffffffffu, sum, o);
          cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        }
        if (lane == 0) out[g] = cnt > 0 ? sum / (float)cnt : 0.f;
      } else if (lane == 0) {
        out[g] = sum / (float)D;
      }
    }
  } else {
    for (int g = threadIdx.x; g < G; g += BS_THREADS) {
      float sum = 0.f;
      for (int i = 0; i < D; ++i) {
        const float2 X = xs[bs_swz(g * D + i)];
        sum += X.x * X.x + X.y * X.y;
      }
      if (isnan(sum)) {
        sum = 0.f;
        int cnt = 0;
        for (int i = 0; i < D; ++i) {
          const float2 X = xs[bs_swz(g * D + i)];
          const float pw = X.x * X.x + X.y * X.y;
          if (!isnan(pw)) {
            sum += pw;
            ++cnt;
          }
        }
        out[g] = cnt > 0 ? sum / (float)cnt : 0.f;
      } else {
        out[g] = sum / (float)D;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Per-packet spectra summed over packets (adaptive pipeline)
// ---------------------------------------------------------------------------
constexpr int PK_WARPS = 8;
constexpr int PK_CHUNK = 32;  // packets staged per chunk: one per lane

struct PacketSpecArgs {
  const uint4 *beams;  // fp16 pairs [S][P][TP] as 16-byte vectors
  float *out;          // [S][TP - 2 trim]
  int S, P, trim;
  Tw64 w;
};

// Staged packet rows are NV = TP / 4 16-byte vectors; vector q of row `pk` sits
// at q ^ pk_swz(pk), so that the 8 lanes of a quarter-warp reading vector q of
// their own rows hit 8 different bank groups.
template <int NV>
SF_DEVICE int pk_swz(int pk) {
  return NV >= 8 ? (pk & 7) : ((pk >> 1) & (NV - 1));
}

SF_DEVICE float2 h2f(uint32_t u) {
  __half2 h;
  memcpy(&h, &u, 4);
  return __half22float2(h);
}

template <int LOG2TP>
__global__ void __launch_bounds__(PK_WARPS * 32, 1) sf_packet_spectra_kernel(const PacketSpecArgs a) {
  constexpr int TP = 1 << LOG2TP;
  constexpr int NV = TP / 4;
  constexpr int CHV = PK_CHUNK * NV;  // vectors per staged chunk
  extern __shared__ __align__(16) uint4 sm_pk[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = blockIdx.x * PK_WARPS + warp;
  if (s >= a.S) return;  // no block-wide barrier below
  uint4 *buf = sm_pk + (size_t)warp * 2 * CHV;
  const uint4 *src = a.beams + (size_t)s * a.P * NV;
  const int nch = (a.P + PK_CHUNK - 1) / PK_CHUNK;

  auto stage = [&](int ch) {
    const int p0 = ch * PK_CHUNK;
    const int nvec = min(PK_CHUNK, a.P - p0) * NV;
    uint4 *dst = buf + (ch & 1) * CHV;
    const uint4 *g = src + (size_t)p0 * NV;
    for (int i = lane; i < nvec; i += 32) {
      const int pk = i / NV, q = i % NV;
      cp_async16(dst + pk * NV + (q ^ pk_swz<NV>(pk)), g + i);
    }
    cp_async_commit();
  };

  float acc[TP];
#pragma unroll
  for (int i = 0; i < TP; ++i) acc[i] = 0.f;
  const int sw = pk_swz<NV>(lane);
  stage(0);
  for (int ch = 0; ch < nch; ++ch) {
    if (ch + 1 < nch) {
      stage(ch + 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncwarp();
    if (ch * PK_CHUNK + lane < a.P) {
      const uint4 *row = buf + (ch & 1) * CHV + lane * NV;
      float2 v[TP];
#pragma unroll
      for (int q = 0; q < NV; ++q) {
        const uint4 u = row[q ^ sw];
        v[4 * q + 0] = h2f(u.x);
        v[4 * q + 1] = h2f(u.y);
        v[4 * q + 2] = h2f(u.z);
        v[4 * q + 3] = h2f(u.w);
      }
      dft_reg<LOG2TP>(v, a.w);
#pragma unroll
      for (int i = 0; i < TP; ++i) acc[i] += sqrtf(v[i].x * v[i].x + v[i].y * v[i].y);
    }
    __syncwarp();  // the buffer just read is refilled by the next stage()
  }

  // Partial sums by bin, one padded row per lane, then fixed-order column sums.
  float *red = reinterpret_cast<float *>(buf);  // [32][TP + 1]
#pragma unroll
  for (int i = 0; i < TP; ++i) red[lane * (TP + 1) + bitrev(i, LOG2TP)] = acc[i];
  __syncwarp();
  const int W = TP - 2 * a.trim;
  const int hi0 = TP / 2 + a.trim, lo_end = TP / 2 - a.trim;
  for (int k = lane; k < TP; k += 32) {
    float sum = 0.f;
    for (int r = 0; r < 32; ++r) sum += red[r * (TP + 1) + k];
    const int g = k >= hi0 ? k - hi0 : (k < lo_end ? k + lo_end : -1);
    if (g >= 0) a.out[(size_t)s * W + g] = sum;
  }
}


// ---------------------------------------------------------------------------
// Per-packet spectra on the tensor cores (Tp = 64, P a multiple of 32)
// ---------------------------------------------------------------------------
// The 64-point DFT of every packet is one GEMM row: with the packet's 64
// complex fp16 samples as a K = 128 row (re, im interleaved, exactly the
// beams' memory layout) and the DFT as a 128 x 128 real matrix
//   B[2t][2f] = cos, B[2t+1][2f] = sin, B[2t][2f+1] = -sin, B[2t+1][2f+1] = cos
// (angle 2 pi f t / 64), D = A B holds Re X[f], Im X[f] at columns 2f, 2f+1.
// A tile is 128 packets (rows), loaded by TMA straight from the beams with the
// 128-byte swizzle (two 16 KB boxes, K halves); B is split into fp16 hi + lo
// parts (B = hi + lo to ~2^-22) and both are accumulated, so the result equals
// the fp32 DFT of the fp16 beams to fp32 accumulation error.
//
// A tile holds 32 consecutive packets of 4 series (series-major: TMEM lane
// 32 q + r is packet r of series q), loaded by one 3-D TMA box per K half.
// Warp roles: warps 0-7 epilogue (TMEM lane quarter q = warp % 4, frequency
// half warp / 4), warp 8 TMA producer, warp 9 MMA issuer and TMEM owner.  Each
// persistent CTA owns a contiguous range of series and walks it 4 series at a
// time, P / 32 tiles per quad, so epilogue warp q only ever sees series q of
// the quad: each thread adds its row's |X| into registers tile after tile
// (packets r, 32 + r, ... of the series), and at the series' last tile the
// warp sums its 32 rows per frequency in shared memory in row order.  The
// summation order is fixed, the output deterministic, and no epilogue warp
// waits for another.
constexpr int TC_EPI_WARPS = 8;
constexpr int TC_WARP_TMA = 8;
constexpr int TC_WARP_MMA = 9;
constexpr int TC_THREADS = 320;
constexpr int TC_STAGES = 4;
constexpr uint32_t TC_ATOM = 128 * 128;          // one K half of a tile: 128 rows x 128 B
constexpr uint32_t TC_TILE_BYTES = 2 * TC_ATOM;   // 128 packets x 256 B
constexpr uint32_t TC_B_BYTES = 2 * TC_TILE_BYTES;  // hi and lo DFT matrices
constexpr int TC_RED_STRIDE = 33;
constexpr uint32_t TC_SUSPEND_NS = 20000;

constexpr int TC_ACC = 4;  // tensor-memory accumulators (128 columns each): the epilogue may lag 3 tiles

struct TcHeader {
  uint64_t a_full[TC_STAGES];
  uint64_t a_empty[TC_STAGES];
  uint64_t acc_full[TC_ACC];
  uint64_t acc_empty[TC_ACC];
  uint64_t b_full;
  uint64_t mma_done;
  uint32_t tmem_base;
  int abort;
};

struct TcSpecArgs {
  const uint8_t *dft;  // the B image (hi, lo), TC_B_BYTES, already swizzled
  float *out;          // [S][64 - 2 trim]
  uint32_t *status;
  int S, P, trim;
};

SF_DEVICE float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    sf_packet_spectra_tc_kernel(const __grid_constant__ CUtensorMap tmap, const TcSpecArgs a) {
  extern __shared__ uint8_t smem_raw[];
  // 1024-byte alignment for the swizzled operand atoms
  uint8_t *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  uint8_t *b_img = smem;                                     // TC_B_BYTES
  uint8_t *a_stage = b_img + TC_B_BYTES;                     // TC_STAGES x TC_TILE_BYTES
  float *red = reinterpret_cast<float *>(a_stage + TC_STAGES * TC_TILE_BYTES);  // [8][32][33]
  TcHeader &h = *reinterpret_cast<TcHeader *>(red + TC_EPI_WARPS * 32 * TC_RED_STRIDE);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // this CTA's series [s0, s1), walked 4 at a time, P / 32 tiles per quad
  const int s0 = (int)((long long)blockIdx.x * a.S / gridDim.x);
  const int s1 = (int)((long long)(blockIdx.x + 1) * a.S / gridDim.x);
  const int tiles_per_quad = a.P / 32;
  const int n_tiles = ((s1 - s0 + 3) / 4) * tiles_per_quad;

  if (threadIdx.x == 0) {
    for (int i = 0; i < TC_STAGES; ++i) {
      mbar_init(&h.a_full[i], 1);
      mbar_init(&h.a_empty[i], 1);
    }
    for (int i = 0; i < TC_ACC; ++i) {
      mbar_init(&h.acc_full[i], 1);
      mbar_init(&h.acc_empty[i], TC_EPI_WARPS);
    }
    mbar_init(&h.b_full, 1);
    mbar_init(&h.mma_done, 1);
    h.abort = 0;
    fence_mbarrier_init();
  }
  if (warp == TC_WARP_MMA) {
    tmem_alloc(&h.tmem_base, 128 * TC_ACC);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  volatile int *abort_flag = &h.abort;

  if (warp == TC_WARP_TMA) {
    // ---------------- producer ----------------
    if (lane == 0) {
      mbar_arrive_expect_tx(&h.b_full, TC_B_BYTES);
      for (int q = 0; q < 4; ++q)
        bulk_copy_g2s(b_img + q * (TC_B_BYTES / 4), a.dft + q * (TC_B_BYTES / 4), TC_B_BYTES / 4, &h.b_full);
      int i = 0;
      bool stop = false;
      for (; i < n_tiles; ++i) {
        const int st = i % TC_STAGES, it = i / TC_STAGES;
        if (!mbar_wait(&h.a_empty[st], (it & 1) ^ 1, abort_flag, TC_SUSPEND_NS)) {
          stop = true;
          break;
        }
        const int quad = i / tiles_per_quad, t = i - quad * tiles_per_quad;
        uint8_t *dst = a_stage + st * TC_TILE_BYTES;
        mbar_arrive_expect_tx(&h.a_full[st], TC_TILE_BYTES);
        tma_load_3d(dst, &tmap, 0, 32 * t, s0 + 4 * quad, &h.a_full[st]);
        tma_load_3d(dst + TC_ATOM, &tmap, 64, 32 * t, s0 + 4 * quad, &h.a_full[st]);
      }
      // every issued copy lands before shared memory is released
      mbar_wait_drain(&h.b_full, 0);
      for (int j = i > TC_STAGES ? i - TC_STAGES : 0; j < i; ++j)
        mbar_wait_drain(&h.a_full[j % TC_STAGES], (j / TC_STAGES) & 1);
      if (stop) atomicOr(a.status, SF_DEVERR_TIMEOUT_TMA);
    }
  } else if (warp == TC_WARP_MMA) {
    // ---------------- UMMA issuer ----------------
    if (lane == 0) {
      const uint32_t idesc = umma_idesc_f16_f32(128, 128);
      const uint64_t d_a0 = umma_desc_sw128(smem_u32(a_stage));
      const uint64_t d_b0 = umma_desc_sw128(smem_u32(b_img));
      bool failed = !mbar_wait(&h.b_full, 0, abort_flag);
      tc_fence_after();
      for (int i = 0; i < n_tiles; ++i) {
        const int st = i % TC_STAGES, it = i / TC_STAGES, buf = i % TC_ACC;
        bool ok = mbar_wait(&h.a_full[st], it & 1, abort_flag);
        ok = mbar_wait(&h.acc_empty[buf], ((i / TC_ACC) & 1) ^ 1, abort_flag) && ok;
        tc_fence_after();
        failed |= !ok;
        const uint32_t go = (ok && !failed) ? 1u : 0u;
        const uint32_t d = h.tmem_base + buf * 128;
        const uint64_t da = d_a0 + ((st * TC_TILE_BYTES) >> 4);
#pragma unroll
        for (int ks = 0; ks < 8; ++ks) {
          const uint32_t kof = ((ks >> 2) * TC_ATOM + (ks & 3) * 32) >> 4;
          umma_f16_if(d, da + kof, d_b0 + kof, idesc, ks > 0 ? 1u : 0u, go);
          umma_f16_if(d, da + kof, d_b0 + ((TC_TILE_BYTES >> 4) + kof), idesc, 1u, go);
        }
        umma_commit(&h.a_empty[st]);
        umma_commit(&h.acc_full[buf]);
      }
      umma_commit(&h.mma_done);
      mbar_wait_drain(&h.mma_done, 0);
      if (failed) atomicOr(a.status, SF_DEVERR_TIMEOUT_MMA);
    }
  } else {
    // ---------------- epilogue ----------------
    const int q = warp & 3, half = warp >> 2;
    const uint32_t tmem = h.tmem_base + (static_cast<uint32_t>(q * 32) << 16) + half * 64;
    float *my_red = red + warp * 32 * TC_RED_STRIDE;
    const int W = 64 - 2 * a.trim;
    const int hi0 = 32 + a.trim, lo_end = 32 - a.trim;
    const int f = half * 32 + lane;  // frequency this lane reduces and writes
    const int g_out = f >= hi0 ? f - hi0 : (f < lo_end ? f + lo_end : -1);
    float acc[32];  // this row's |X| summed over the series' tiles
#pragma unroll
    for (int k = 0; k < 32; ++k) acc[k] = 0.f;
    bool failed = false;
    for (int i = 0; i < n_tiles; ++i) {
      const int buf = i % TC_ACC;
      const int quad = i / tiles_per_quad, t = i - quad * tiles_per_quad;
      const int s = s0 + 4 * quad + q;
      const bool ok = mbar_wait(&h.acc_full[buf], (i / TC_ACC) & 1, abort_flag);
      tc_fence_after();
      failed |= !ok;
      uint32_t v[4][16];  // Re, Im of this row's 32 frequencies
      if (ok) {
#pragma unroll
        for (int j = 0; j < 4; ++j) tmem_ld16(tmem + buf * 128 + 16 * j, v[j]);
        tmem_wait_ld();
      }
      // the tile is in registers: hand the accumulator back before the math
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&h.acc_empty[buf]);
      if (ok) {
#pragma unroll
        for (int k = 0; k < 32; ++k) {
          const float re = __uint_as_float(v[k >> 3][(2 * k) & 15]);
          const float im = __uint_as_float(v[k >> 3][(2 * k + 1) & 15]);
          acc[k] += sqrt_approx(re * re + im * im);
        }
      }
      if (t == tiles_per_quad - 1) {
        // series done: sum the 32 rows (packets r, 32 + r, ...) per frequency in row order
        if (ok && s < s1) {
#pragma unroll
          for (int k = 0; k < 32; ++k) my_red[lane * TC_RED_STRIDE + k] = acc[k];
          __syncwarp();
          float part[4] = {0.f, 0.f, 0.f, 0.f};  // rows r = 4 m + j into part[j]
#pragma unroll
          for (int r = 0; r < 32; ++r) part[r & 3] += my_red[r * TC_RED_STRIDE + lane];
          __syncwarp();
          if (g_out >= 0) a.out[(size_t)s * W + g_out] = (part[0] + part[1]) + (part[2] + part[3]);
        }
#pragma unroll
        for (int k = 0; k < 32; ++k) acc[k] = 0.f;
      }
    }
    if (failed && lane == 0) atomicOr(a.status, SF_DEVERR_TIMEOUT_EPILOGUE);
  }

  tc_fence_before();
  __syncthreads();
  if (warp == TC_WARP_MMA) {
    tc_fence_after();
    tmem_dealloc(h.tmem_base, 128 * TC_ACC);
  }
}

size_t tc_smem_bytes() {
  return 1024 + TC_B_BYTES + TC_STAGES * TC_TILE_BYTES + sizeof(float) * TC_EPI_WARPS * 32 * TC_RED_STRIDE +
         sizeof(TcHeader);
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

template <typename K>
cudaError_t ensure_smem(K kernel, size_t smem) {
  return sf_smem_optin(reinterpret_cast<const void *>(kernel), smem);
}

template <int LOG2T>
cudaError_t launch_bs(const BeamSpecArgs &a, int dev, cudaStream_t stream) {
  const size_t smem = sizeof(float2) << LOG2T;
  cudaError_t e = ensure_smem(sf_beam_spectra_kernel<LOG2T>, smem);
  if (e != cudaSuccess) return e;
  sf_beam_spectra_kernel<LOG2T><<<a.S, BS_THREADS, smem, stream>>>(a);
  return cudaGetLastError();
}

template <int LOG2TP>
cudaError_t launch_pk(const PacketSpecArgs &a, int dev, cudaStream_t stream) {
  const size_t smem = (size_t)PK_WARPS * 2 * PK_CHUNK * (1 << LOG2TP) * 4;
  cudaError_t e = ensure_smem(sf_packet_spectra_kernel<LOG2TP>, smem);
  if (e != cudaSuccess) return e;
  sf_packet_spectra_kernel<LOG2TP><<<(a.S + PK_WARPS - 1) / PK_WARPS, PK_WARPS * 32, smem, stream>>>(a);
  return cudaGetLastError();
}

int log2_exact(int n) {
  if (n < 1 || (n & (n - 1))) return -1;
  return ilog2c(n);
}

}  // namespace

int sf_beam_spectra_supported(int T) {
  const int l = log2_exact(T);
  return l >= BS_MIN_LOG2T && l <= BS_MAX_LOG2T;
}

int sf_packet_spectra_supported(int Tp) {
  const int l = log2_exact(Tp);
  return l >= 4 && l <= 6;
}

// Twiddles of every Stockham pass of a T-point transform (radix 16 while at
// least 16 remain, then the remainder): the pass combining sub-transforms of
// length NS uses W_{NS R}^{r jm} (1 <= r < R, jm < NS) at NS - 1 + (r - 1) NS + jm.
// The pass blocks telescope: sum (R - 1) NS = T - 1 entries in all.
cudaError_t sf_fill_spectra_twiddles(float2 *d_tw, int T) {
  float2 *h = static_cast<float2 *>(calloc(T, sizeof(float2)));
  if (!h) return cudaErrorMemoryAllocation;
  const double pi = 3.14159265358979323846;
  for (int ns = 1; ns < T;) {
    const int r_max = T / ns >= 16 ? 16 : T / ns;
    for (int r = 1; r < r_max; ++r)
      for (int jm = 0; jm < ns; ++jm) {
        const double a = 2.0 * pi * (double)r * jm / ((double)ns * r_max);
        h[ns - 1 + (r - 1) * ns + jm] = make_float2(static_cast<float>(std::cos(a)), static_cast<float>(-std::sin(a)));
      }
    ns *= r_max;
  }
  cudaError_t e = cudaMemcpy(d_tw, h, sizeof(float2) * T, cudaMemcpyHostToDevice);
  free(h);
  return e;
}

cudaError_t sf_launch_beam_spectra(const sf_plan *p, const __half2 *beams, int n_beams_out,
                                   int downsample, float *out, cudaStream_t stream) {
  BeamSpecArgs a;
  a.beams = beams;
  a.tw = p->d_spec_tw;
  a.out = out;
  a.S = p->C * 2 * n_beams_out;
  a.D = downsample;
  a.w = tw64();
  switch (log2_exact(p->T)) {
    case 6: return launch_bs<6>(a, p->device, stream);
    case 7: return launch_bs<7>(a, p->device, stream);
    case 8: return launch_bs<8>(a, p->device, stream);
    case 9: return launch_bs<9>(a, p->device, stream);
    case 10: return launch_bs<10>(a, p->device, stream);
    case 11: return launch_bs<11>(a, p->device, stream);
    case 12: return launch_bs<12>(a, p->device, stream);
    case 13: return launch_bs<13>(a, p->device, stream);
    case 14: return launch_bs<14>(a, p->device, stream);
    default: return cudaErrorInvalidValue;
  }
}

int sf_packet_spectra_tc_supported(const sf_plan *p) { return p->Tp == 64 && p->P % 32 == 0; }

// The DFT operand image for the tensor-core path: [hi, lo][K half][128 rows n]
// [128 B], each row's 16-byte chunks stored at chunk ^ (n % 8) (the 128-byte
// swizzle), values B[k][n] of the real 128 x 128 form of the 64-point DFT.
cudaError_t sf_fill_packet_dft(uint8_t *d_img) {
  uint8_t *h = static_cast<uint8_t *>(calloc(TC_B_BYTES, 1));
  if (!h) return cudaErrorMemoryAllocation;
  const double pi = 3.14159265358979323846;
  for (int n = 0; n < 128; ++n)
    for (int k = 0; k < 128; ++k) {
      const int f = n >> 1, c = n & 1, t = k >> 1, d = k & 1;
      const double ang = 2.0 * pi * (double)((f * t) % 64) / 64.0;
      const double co = std::cos(ang), si = std::sin(ang);
      const double v = c == 0 ? (d == 0 ? co : si) : (d == 0 ? -si : co);
      const __half hi = __double2half(v);
      const __half lo = __double2half(v - (double)__half2float(hi));
      const int atom = k >> 6, kk = k & 63;
      const size_t off = (size_t)atom * TC_ATOM + n * 128 + ((((kk >> 3) ^ (n & 7))) << 4) + (kk & 7) * 2;
      memcpy(h + off, &hi, 2);
      memcpy(h + TC_TILE_BYTES + off, &lo, 2);
    }
  cudaError_t e = cudaMemcpy(d_img, h, TC_B_BYTES, cudaMemcpyHostToDevice);
  free(h);
  return e;
}

size_t sf_packet_dft_bytes() { return TC_B_BYTES; }

cudaError_t sf_launch_packet_spectra(const sf_plan *p, const __half2 *beams, int n_beams_out,
                                     int trim, float *out, cudaStream_t stream) {
  if (sf_packet_spectra_tc_supported(p) && p->d_packet_dft) {
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode) return cudaErrorNotSupported;
    const int S = p->C * 2 * n_beams_out;
    CUtensorMap tmap;
    // [series][packet][128 fp16]; a box is 4 series x 32 packets x one K half
    const cuuint64_t dims[3] = {128, (cuuint64_t)p->P, (cuuint64_t)S};
    const cuuint64_t strides[2] = {256, (cuuint64_t)p->P * 256};
    const cuuint32_t box[3] = {64, 32, 4};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = encode(&tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, const_cast<__half2 *>(beams), dims, strides,
                        box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
    TcSpecArgs a;
    a.dft = p->d_packet_dft;
    a.out = out;
    a.status = p->d_status;
    a.S = S;
    a.P = p->P;
    a.trim = trim;
    const size_t smem = tc_smem_bytes();
    cudaError_t e = ensure_smem(sf_packet_spectra_tc_kernel, smem);
    if (e != cudaSuccess) return e;
    const int grid = S < p->num_sms ? S : p->num_sms;
    sf_packet_spectra_tc_kernel<<<grid, TC_THREADS, smem, stream>>>(tmap, a);
    return cudaGetLastError();
  }
  PacketSpecArgs a;
  a.beams = reinterpret_cast<const uint4 *>(beams);
  a.out = out;
  a.S = p->C * 2 * n_beams_out;
  a.P = p->P;
  a.trim = trim;
  a.w = tw64();
  switch (log2_exact(p->Tp)) {
    case 4: return launch_pk<4>(a, p->device, stream);
    case 5: return launch_pk<5>(a, p->device, stream);
    case 6: return launch_pk<6>(a, p->device, stream);
    default: return cudaErrorInvalidValue;
  }
}
