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
  const float2 *tw;      // W_T^k, k < T
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
// the fp16 series from global memory instead.
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
#pragma unroll
      for (int r = 0; r < R; ++r)
        v[b][r] = NS == 1 ? __half22float2(src[j + r * NB]) : x[bs_swz(j + r * NB)];
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
        for (int r = 1; r < R; ++r) v[b][r] = cmul(v[b][r], __ldg(tw + r * jm * (T / (NS * R))));
      }
      dft_reg<LOG2R>(v[b], w);
      const int base = (j - jm) * R + jm;
#pragma unroll
      for (int k = 0; k < R; ++k) x[bs_swz(base + k * NS)] = v[b][bitrev(k, LOG2R)];
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

  const int D = a.D, G = T / D;
  float *out = a.out + (size_t)s * G;
  if (D >= 32) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int g = warp; g < G; g += BS_THREADS / 32) {
      float sum = 0.f;
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
    }
  } else {
    for (int g = threadIdx.x; g < G; g += BS_THREADS) {
      float sum = 0.f;
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

constexpr int MAX_DEVICES = 64;
bool g_bs_attr[MAX_DEVICES][BS_MAX_LOG2T + 1];
bool g_pk_attr[MAX_DEVICES][7];

template <typename K>
cudaError_t ensure_smem(K kernel, bool &done, size_t smem) {
  if (done || smem <= 48 * 1024) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) done = true;
  return e;
}

template <int LOG2T>
cudaError_t launch_bs(const BeamSpecArgs &a, int dev, cudaStream_t stream) {
  const size_t smem = sizeof(float2) << LOG2T;
  cudaError_t e = ensure_smem(sf_beam_spectra_kernel<LOG2T>, g_bs_attr[dev][LOG2T], smem);
  if (e != cudaSuccess) return e;
  sf_beam_spectra_kernel<LOG2T><<<a.S, BS_THREADS, smem, stream>>>(a);
  return cudaGetLastError();
}

template <int LOG2TP>
cudaError_t launch_pk(const PacketSpecArgs &a, int dev, cudaStream_t stream) {
  const size_t smem = (size_t)PK_WARPS * 2 * PK_CHUNK * (1 << LOG2TP) * 4;
  cudaError_t e = ensure_smem(sf_packet_spectra_kernel<LOG2TP>, g_pk_attr[dev][LOG2TP], smem);
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

cudaError_t sf_fill_spectra_twiddles(float2 *d_tw, int T) {
  float2 *h = static_cast<float2 *>(malloc(sizeof(float2) * T));
  if (!h) return cudaErrorMemoryAllocation;
  const double pi = 3.14159265358979323846;
  for (int k = 0; k < T; ++k)
    h[k] = make_float2(static_cast<float>(std::cos(2.0 * pi * k / T)),
                       static_cast<float>(-std::sin(2.0 * pi * k / T)));
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
  if (p->device < 0 || p->device >= MAX_DEVICES) return cudaErrorInvalidDevice;
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

cudaError_t sf_launch_packet_spectra(const sf_plan *p, const __half2 *beams, int n_beams_out,
                                     int trim, float *out, cudaStream_t stream) {
  PacketSpecArgs a;
  a.beams = reinterpret_cast<const uint4 *>(beams);
  a.out = out;
  a.S = p->C * 2 * n_beams_out;
  a.P = p->P;
  a.trim = trim;
  a.w = tw64();
  if (p->device < 0 || p->device >= MAX_DEVICES) return cudaErrorInvalidDevice;
  switch (log2_exact(p->Tp)) {
    case 4: return launch_pk<4>(a, p->device, stream);
    case 5: return launch_pk<5>(a, p->device, stream);
    case 6: return launch_pk<6>(a, p->device, stream);
    default: return cudaErrorInvalidValue;
  }
}
