// Tensor-core correlator and beamformer over one integration of int8 complex
// voltages in the packet layout.
//
// One persistent CTA per SM streams each channel's packets once through
// shared memory and builds fp16 operand tiles A[u][t] (row u = 2k + comp,
// k = pol * R + receiver; 64 samples t per 128-byte row, 128-byte swizzle).
// From the same tiles it can
//   * correlate: G = A A^T with tcgen05 UMMA (A K-major), fp32 accumulation in
//     tensor memory, drained every 512 samples into int32 running sums -> exact
//     int32 visibilities in the trimmed packed-triangle layout.  Replaces the
//     reference's fp16 ingest + layout permutations + Tensor Core Correlator +
//     trim (include/spatial/spatial.cuh:55-304, lambda_gpu_pipeline.hpp:640-671,
//     src/spatial.cu:176-200).
//       Re V(k,m) = G[2k][2m] + G[2k+1][2m+1],  Im V(k,m) = G[2k+1][2m] - G[2k][2m+1]
//     Rows 0..127 of G come from one M=128 x N=NR MMA; rows 128..NR-1 x columns
//     128..NR-1 from a second M=128 x N=NR-128 MMA; the rest is V(k,m) = conj(V(m,k)).
//   * beamform: Y^T[t][n] = sum_u A^T[t][u] W[n][u] per 128 samples, A read
//     MN-major (two 64-sample tiles side by side), W the block-diagonal real
//     form of the effective weights (n = pol, beam, re/im), fp32 accumulation,
//     fp16 output [C][Pol][NB][T][2].  Replaces the reference's
//     col-major sample layout + weight permutation + ccglib GEMM + half output
//     (spatial.cuh:145-213, 376-418; lambda_gpu_pipeline.hpp:708-743).
//   * or both in one pass (the plain pipelines).
// Operands: fp16(x * scale) is exact for |x s| <= 2048 and equals the
// reference's ingest for unit gain; correlation chunks are exact while
// |partial sums| <= 2^24 (512 samples of |x s| <= 128).
//
// CTA roles (16 warps):
//   warp 0           producer: one bulk (TMA) copy per packet [F][Tp][Rpp][Pol][2]
//                    plus the packet's scales by 4-byte cp.async, completing on
//                    the slot's mbarrier
//   warp 1           TMEM allocation + the single-thread UMMA issuer
//   warps 4-7        epilogue (one TMEM lane quarter each)
//   warps 2-3, 8-15  converters: ring (int8) -> swizzled fp16 tiles (per-packet
//                    scale, per-FPGA window offset); per channel the weight tile
// Every wait is bounded (about a second) and reports through the status word.
#include <algorithm>
#include <cstdio>

#include "sf_common.cuh"
#include "sf_plan.cuh"

namespace {

constexpr int KBLK = 64;        // samples per K block = one 128-byte fp16 row
constexpr int CHUNK_KBLK = 8;   // K blocks per exact fp32 chunk (512 samples)
constexpr int NUM_OP_STAGES = 4;
constexpr int NUM_WARPS = 16;
constexpr int NTHREADS = NUM_WARPS * 32;
constexpr int WARP_TMA = 0;
constexpr int WARP_MMA = 1;
constexpr int WARP_EPI0 = 4;
constexpr int WARP_CONV0 = 8;  // converters: warps 2-3 and 8-15
constexpr int NUM_CONV_THREADS = 10 * 32;
constexpr int MAX_SLOTS = 32;
constexpr int MAX_F = 64;
constexpr uint32_t HEADER_BYTES = 2048;
constexpr int MAX_R = 48;
constexpr int MAX_BEAM_OUT = 16;  // beams (all slots) per pol in the tensor beamformer

struct CorrArgs {
  const int8_t *samples;
  const int16_t *scales;
  const int32_t *offsets;
  int32_t *vis;
  const float2 *weff;  // [C][2][NBW][R]
  __half2 *beams;      // [C][2][NB][T]
  uint32_t *status;
  int C, F, Tp, R, Rpp, P, T, NBL;
  int NR;           // operand rows holding data: round_up(4R, 16)
  int stage_rows;   // rows per operand stage: max(NR, 128)
  int nkb;          // K blocks per channel (even when beamforming)
  int slot_bytes;   // one packet of one channel: R * Tp * 4 bytes
  int slot_stride;  // slot_bytes + the packet's scales, rounded to 16
  int num_slots;    // packet ring depth (power of two)
  int NB, NBW;      // beams written per pol; rows of weff per (c, p)
  int BN;           // beam MMA N = round_up(4 NB, 16)
  int katoms;       // 64-column K atoms of the weight tile: ceil(NR / 64)
  uint32_t wtile_bytes;
  uint32_t tmem_cols, i32_off, beam_off;
  int nacc;  // fp32 chunk accumulators in tensor memory (2 = double-buffered)
  uint32_t acc_stride;  // tensor-memory columns between the fp32 accumulators
};

struct __align__(8) Header {
  uint64_t pk_full[MAX_SLOTS];
  uint64_t pk_empty[MAX_SLOTS];
  uint64_t op_full[NUM_OP_STAGES];
  uint64_t op_empty[NUM_OP_STAGES];
  uint64_t acc_full[2];
  uint64_t acc_empty[2];
  uint64_t beam_full[2];
  uint64_t beam_empty[2];
  uint64_t w_full[2];
  uint64_t w_empty[2];
  uint64_t mma_done;
  uint32_t tmem_base;
  int abort;
  int offsets[MAX_F];
};
static_assert(sizeof(Header) <= HEADER_BYTES, "header too large");

__device__ __forceinline__ uint32_t u32_of(__half2 h) { return *reinterpret_cast<uint32_t *>(&h); }
__device__ __forceinline__ __half2 h2_of(uint32_t u) { return *reinterpret_cast<__half2 *>(&u); }

// Four int8 (pol0 re, pol0 im, pol1 re, pol1 im) times the two int16 scales
// -> two half2 equal to __float2half_rn(float(x * s)), the value the
// reference's ingest produces for a unit gain (spatial.cuh:464-483).
__device__ __forceinline__ void convert_word(uint32_t word, uint32_t scw, __half2 &p0, __half2 &p1) {
  const uint32_t biased = word ^ 0x80808080u;  // x + 128 as unsigned bytes
  // 0x6400 | b is the fp16 value 1024 + b, exact for b in [0, 1023]
  const __half2 h01 = h2_of(__byte_perm(biased, 0x64646464u, 0x4140));
  const __half2 h23 = h2_of(__byte_perm(biased, 0x64646464u, 0x4342));
  const __half2 bias = h2_of(0x64806480u);  // 1152
  __half2 x01 = __hsub2(h01, bias);         // exact integers in [-128, 127]
  __half2 x23 = __hsub2(h23, bias);
  if (scw != 0x00010001u) {
    const int s0 = static_cast<int16_t>(scw & 0xFFFFu);
    const int s1 = static_cast<int16_t>(scw >> 16);
    if (s0 >= -2048 && s0 <= 2048 && s1 >= -2048 && s1 <= 2048) {
      // both factors exact in fp16: one correctly rounded product, as the
      // reference's int multiply + float->half conversion
      x01 = __hmul2(x01, __half2half2(__int2half_rn(s0)));
      x23 = __hmul2(x23, __half2half2(__int2half_rn(s1)));
    } else {
      const int a0 = static_cast<int8_t>(word & 0xFF), a1 = static_cast<int8_t>((word >> 8) & 0xFF);
      const int a2 = static_cast<int8_t>((word >> 16) & 0xFF), a3 = static_cast<int8_t>(word >> 24);
      x01 = __floats2half2_rn(static_cast<float>(a0 * s0), static_cast<float>(a1 * s0));
      x23 = __floats2half2_rn(static_cast<float>(a2 * s1), static_cast<float>(a3 * s1));
    }
  }
  p0 = x01;
  p1 = x23;
}

__device__ __forceinline__ void emit_vis(const CorrArgs &a, int c, int p, int i, int q, int j,
                                         int comp, int val) {
  const size_t idx = ((((size_t)c * a.NBL + baseline_of(i, j)) * 2 + p) * 2 + q) * 2 + comp;
  a.vis[idx] = val;
}

// Shared-memory descriptor with explicit strides (128-byte swizzle).
__device__ __forceinline__ uint64_t desc_sw128(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((addr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
  d |= static_cast<uint64_t>(1u) << 46;
  d |= static_cast<uint64_t>(2u) << 61;
  return d;
}

template <bool DO_CORR, bool DO_BEAM>
__global__ void __launch_bounds__(NTHREADS, 1) sf_corrbeam_kernel(const CorrArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  Header &h = *reinterpret_cast<Header *>(smem);
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane = tid & 31;

  const uint32_t sbase = smem_u32(smem);
  const uint32_t op_addr = (sbase + HEADER_BYTES + 1023u) & ~1023u;
  uint8_t *op_ptr = smem + (op_addr - sbase);
  const uint32_t stage_bytes = static_cast<uint32_t>(a.stage_rows) * 128u;
  const uint32_t w_addr = op_addr + NUM_OP_STAGES * stage_bytes;  // weight tiles (1024-aligned)
  uint8_t *w_ptr = op_ptr + NUM_OP_STAGES * stage_bytes;
  uint8_t *ring_ptr = w_ptr + (DO_BEAM ? 2 * a.wtile_bytes : 0u);
  const int NS = a.num_slots;
  const uint32_t ns_mask = static_cast<uint32_t>(NS - 1);
  const uint32_t ns_shift = __popc(ns_mask);

  if (tid == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(&h.pk_full[s], 1 + 32);
      mbar_init(&h.pk_empty[s], 1);
    }
    for (int s = 0; s < NUM_OP_STAGES; ++s) {
      mbar_init(&h.op_full[s], 1);
      mbar_init(&h.op_empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&h.acc_full[b], 1);
      mbar_init(&h.acc_empty[b], 4);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&h.beam_full[b], 1);
      mbar_init(&h.beam_empty[b], 4);
      mbar_init(&h.w_full[b], 1);
      mbar_init(&h.w_empty[b], 1);
    }
    mbar_init(&h.mma_done, 1);
    h.abort = 0;
    fence_mbarrier_init();
  }
  for (int f = tid; f < a.F; f += NTHREADS) h.offsets[f] = a.offsets[f];
  // Padding rows/columns of the operand and weight tiles must read as zero.
  {
    uint4 *z = reinterpret_cast<uint4 *>(op_ptr);
    const int n16 = (NUM_OP_STAGES * stage_bytes + (DO_BEAM ? 2 * a.wtile_bytes : 0u)) / 16;
    for (int i = tid; i < n16; i += NTHREADS) z[i] = make_uint4(0, 0, 0, 0);
    fence_proxy_async_smem();
  }
  if (warp == WARP_MMA) {
    tmem_alloc(&h.tmem_base, a.tmem_cols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();

  int off_min = 1 << 30, off_max = -(1 << 30);
  for (int f = 0; f < a.F; ++f) {
    off_min = min(off_min, h.offsets[f]);
    off_max = max(off_max, h.offsets[f]);
  }
  const int Tp = a.Tp, T = a.T, R = a.R;
  const int qa0 = off_min / Tp;
  const int qbN = min(a.P + 1, (T - 1 + off_max) / Tp);
  const int npk = qbN - qa0 + 1;
  const int nchunks = (a.nkb + CHUNK_KBLK - 1) / CHUNK_KBLK;
  volatile int *abort_flag = &h.abort;

  if (warp == WARP_TMA) {
    // ---------------- producer (whole warp) ----------------
    uint32_t g = 0;
    bool stop = false;
    for (int c = blockIdx.x; c < a.C && !stop; c += gridDim.x) {
      const int8_t *chan = a.samples + (size_t)c * (a.P + 2) * a.slot_bytes;
      const int16_t *chan_sc = a.scales + (size_t)c * (a.P + 2) * R * 2;
      for (int q = qa0; q <= qbN; ++q) {
        const uint32_t slot = g & ns_mask;
        const bool ok = mbar_wait(&h.pk_empty[slot], ((g >> ns_shift) & 1u) ^ 1u, abort_flag, 64);
        if (__any_sync(0xffffffffu, !ok)) {
          stop = true;
          break;
        }
        uint8_t *dst = ring_ptr + (size_t)slot * a.slot_stride;
        if (lane == 0) {
          mbar_arrive_expect_tx(&h.pk_full[slot], a.slot_bytes);
          bulk_copy_g2s(dst, chan + (size_t)q * a.slot_bytes, a.slot_bytes, &h.pk_full[slot]);
        }
        const uint32_t *src_sc = reinterpret_cast<const uint32_t *>(chan_sc + (size_t)q * R * 2);
        uint32_t *dst_sc = reinterpret_cast<uint32_t *>(dst + a.slot_bytes);
        for (int r = lane; r < R; r += 32) cp_async4(dst_sc + r, src_sc + r);
        cp_async_mbar_arrive(&h.pk_full[slot]);
        ++g;
      }
    }
    // Every issued copy lands before shared memory is released.
    if (lane == 0) {
      const uint32_t first = g > (uint32_t)NS ? g - NS : 0u;
      for (uint32_t gq = first; gq < g; ++gq) mbar_wait_drain(&h.pk_full[gq & ns_mask], (gq >> ns_shift) & 1u);
      if (stop) atomicOr(a.status, SF_DEVERR_TIMEOUT_TMA);
    }
  } else if (warp == WARP_MMA) {
    // ---------------- UMMA issuer ----------------
    if (lane == 0) {
      const uint32_t tmem = h.tmem_base;
      const int NR = a.NR;
      const bool corner = NR > 128;
      const uint32_t idesc_main = umma_idesc_f16_f32(128, NR);
      // rows 128..NR-1 come from an M=64 MMA over rows NR-64..NR-1 (its
      // accumulator rows l sit in lanes (l % 16) + 32 (l / 16))
      const uint32_t idesc_corner = umma_idesc_f16_f32(64, corner ? NR - 128 : 16);
      // beam: A (samples) MN-major, B (weights) K-major, M = 128 samples, N = BN
      const uint32_t idesc_beam = umma_idesc_f16_f32(128, a.BN) | (1u << 15);
      uint32_t op_iter = 0, acc_iter = 0, beam_iter = 0, cw = 0;
      bool failed = false;
      for (int c = blockIdx.x; c < a.C; c += gridDim.x, ++cw) {
        const uint32_t wb = cw & 1u;
        if (DO_BEAM) failed |= !mbar_wait(&h.w_full[wb], (cw >> 1) & 1u, abort_flag);
        for (int kb = 0; kb < a.nkb; ++kb) {
          const uint32_t st = op_iter % NUM_OP_STAGES;
          bool ok = mbar_wait(&h.op_full[st], (op_iter / NUM_OP_STAGES) & 1u, abort_flag);
          const bool chunk_start = (kb % CHUNK_KBLK) == 0;
          const uint32_t abuf = acc_iter % a.nacc;
          if (DO_CORR && chunk_start)
            ok = mbar_wait(&h.acc_empty[abuf], ((acc_iter / a.nacc) & 1u) ^ 1u, abort_flag) && ok;
          const bool beam_now = DO_BEAM && (kb & 1);
          if (beam_now)
            ok = mbar_wait(&h.beam_empty[beam_iter & 1u], ((beam_iter >> 1) & 1u) ^ 1u, abort_flag) && ok;
          tc_fence_after();
          if (ok) {
            const uint32_t base = op_addr + st * stage_bytes;
            if (DO_CORR) {
              const uint32_t dacc = tmem + abuf * a.acc_stride;
#pragma unroll
              for (int ks = 0; ks < KBLK / 16; ++ks) {
                const uint32_t acc = (!chunk_start || ks > 0) ? 1u : 0u;
                umma_f16(dacc, umma_desc_sw128(base + ks * 32), umma_desc_sw128(base + ks * 32),
                         idesc_main, acc);
                if (corner)
                  umma_f16(dacc + NR, umma_desc_sw128(base + (NR - 64) * 128 + ks * 32),
                           umma_desc_sw128(base + 128 * 128 + ks * 32), idesc_corner, acc);
              }
            }
            if (beam_now) {
              // the pair (st - 1, st): samples 0..63 and 64..127 of this tile
              const uint32_t abase = base - stage_bytes;
              const uint32_t wbase = w_addr + wb * a.wtile_bytes;
              const uint32_t d = tmem + a.beam_off + (beam_iter & 1u) * a.BN;
              for (int ks = 0; ks < NR / 16; ++ks) {
                const uint64_t ad = desc_sw128(abase + ks * 16 * 128, stage_bytes, 1024);
                const uint32_t kcol = ks * 16;
                const uint64_t bd =
                    desc_sw128(wbase + (kcol / 64) * (a.BN * 128) + (kcol % 64) * 2, 16, 1024);
                umma_f16(d, ad, bd, idesc_beam, ks > 0 ? 1u : 0u);
              }
            }
          } else {
            failed = true;
          }
          if (!DO_BEAM) {
            umma_commit(&h.op_empty[st]);
          } else if (kb & 1) {
            umma_commit(&h.op_empty[(st + NUM_OP_STAGES - 1) % NUM_OP_STAGES]);
            umma_commit(&h.op_empty[st]);
            umma_commit(&h.beam_full[beam_iter & 1u]);
            ++beam_iter;
          }
          if (DO_CORR && ((kb % CHUNK_KBLK) == CHUNK_KBLK - 1 || kb == a.nkb - 1)) {
            umma_commit(&h.acc_full[abuf]);
            ++acc_iter;
          }
          ++op_iter;
        }
        if (DO_BEAM) umma_commit(&h.w_empty[wb]);
      }
      umma_commit(&h.mma_done);
      mbar_wait_drain(&h.mma_done, 0);
      if (failed) atomicOr(a.status, SF_DEVERR_TIMEOUT_MMA);
    }
  } else if (warp >= WARP_EPI0 && warp < WARP_EPI0 + 4) {
    // ---------------- epilogue ----------------
    const int ew = warp - WARP_EPI0;  // == warp % 4: this warp's TMEM lane quarter
    const uint32_t tmem = h.tmem_base + (static_cast<uint32_t>(ew * 32) << 16);
    const int NR = a.NR;
    const int ncols = NR + (NR > 128 ? NR - 128 : 0);
    const int R4 = 4 * R;
    uint32_t acc_iter = 0, beam_iter = 0;
    bool failed = false;
    for (int c = blockIdx.x; c < a.C; c += gridDim.x) {
      for (int kb = 0; kb < a.nkb; ++kb) {
        if (DO_BEAM && (kb & 1)) {
          const uint32_t buf = beam_iter & 1u;
          const bool ok = mbar_wait(&h.beam_full[buf], (beam_iter >> 1) & 1u, abort_flag, 32);
          failed |= !ok;
          tc_fence_after();
          const int t = (kb >> 1) * 128 + ew * 32 + lane;
          for (int cb = 0; cb < a.BN / 16; ++cb) {
            uint32_t v[16];
            tmem_ld16(tmem + a.beam_off + buf * a.BN + cb * 16, v);
            tmem_wait_ld();
            if (ok && t < T) {
#pragma unroll
              for (int e2 = 0; e2 < 8; ++e2) {
                const int col = cb * 8 + e2;  // complex column (pol, beam)
                const int p = col / a.NB;
                const int m = col - p * a.NB;
                if (p < 2)
                  a.beams[(((size_t)c * 2 + p) * a.NB + m) * T + t] =
                      __floats2half2_rn(__uint_as_float(v[2 * e2]), __uint_as_float(v[2 * e2 + 1]));
              }
            }
          }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&h.beam_empty[buf]);
          ++beam_iter;
        }
        if (!DO_CORR || !((kb % CHUNK_KBLK) == CHUNK_KBLK - 1 || kb == a.nkb - 1)) continue;
        const int ch = kb / CHUNK_KBLK;
        const uint32_t abuf = acc_iter % a.nacc;
        const bool ok = mbar_wait(&h.acc_full[abuf], (acc_iter / a.nacc) & 1u, abort_flag, 32);
        failed |= !ok;
        tc_fence_after();
        const bool first = ch == 0;
        const bool last = ch == nchunks - 1;
        const uint32_t tacc = tmem + abuf * a.acc_stride;
        for (int cb = 0; cb < ncols / 16; ++cb) {
          uint32_t fv[16], sv[16];
          tmem_ld16(tacc + cb * 16, fv);
          if (!first) tmem_ld16(tmem + a.i32_off + cb * 16, sv);
          tmem_wait_ld();
          int acc[16];
#pragma unroll
          for (int e = 0; e < 16; ++e)
            acc[e] = (first ? 0 : static_cast<int>(sv[e])) + __float2int_rn(__uint_as_float(fv[e]));
          if (!last) {
            uint32_t out[16];
#pragma unroll
            for (int e = 0; e < 16; ++e) out[e] = static_cast<uint32_t>(acc[e]);
            tmem_st16(tmem + a.i32_off + cb * 16, out);
            continue;
          }
          // Final chunk of this channel: combine (re, im) row pairs and write.
          const bool main_region = cb * 16 < NR;
          const int u = main_region ? ew * 32 + lane : (lane < 16 ? (NR - 64) + ew * 16 + lane : 1 << 20);
          const int k = u >> 1;
          const int comp = u & 1;
          const int p = k / R;
          const int i = k - p * R;
          const bool row_ok = ok && u < R4 && (main_region || u >= 128);
          const int m0 = main_region ? cb * 8 : 64 + ((cb * 16 - NR) >> 1);
#pragma unroll
          for (int e2 = 0; e2 < 8; ++e2) {
            const int g0 = acc[2 * e2];
            const int g1 = acc[2 * e2 + 1];
            const int other = __shfl_xor_sync(0xffffffffu, g1, 1);
            const int val = comp ? g0 - other : g0 + other;
            const int m = m0 + e2;
            if (!row_ok || 2 * m >= R4) continue;
            const int q = m / R;
            const int j = m - q * R;
            if (i <= j) emit_vis(a, c, p, i, q, j, comp, val);
            // Rows m >= 64 are not main-tile rows: their entries with a main-tile
            // column come from here, conjugated.
            if (main_region && m >= 64 && j <= i) emit_vis(a, c, q, j, p, i, comp, comp ? -val : val);
          }
        }
        if (!last) tmem_wait_st();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&h.acc_empty[abuf]);
        ++acc_iter;
      }
    }
    if (failed && lane == 0) atomicOr(a.status, SF_DEVERR_TIMEOUT_EPILOGUE);
  } else if (warp >= WARP_CONV0 || warp == 2 || warp == 3) {
    // ---------------- converters ----------------
    const int ct = warp >= WARP_CONV0 ? (warp - WARP_CONV0 + 2) * 32 + lane : (warp - 2) * 32 + lane;
    uint32_t g_base = 0, op_iter = 0, cw = 0;
    bool failed = false;
    const int Rpp4 = a.Rpp * 4;
    for (int c = blockIdx.x; c < a.C; c += gridDim.x, ++cw) {
      if (DO_BEAM) {
        // weight tile for this channel: B[n][u], n = (pol, beam, re/im), K-major,
        // 128-byte swizzle, one [BN rows][64 cols] block per K atom
        const uint32_t wb = cw & 1u;
        const bool ok = mbar_wait(&h.w_empty[wb], ((cw >> 1) & 1u) ^ 1u, abort_flag);
        failed |= !ok;
        if (ok) {
          uint8_t *wt = w_ptr + wb * a.wtile_bytes;
          const int nchunk = a.katoms * 8;  // 16-byte chunks per row
          for (int task = ct; task < a.BN * nchunk; task += NUM_CONV_THREADS) {
            const int n = task / nchunk;
            const int ch = task - n * nchunk;
            const int atom = ch >> 3, cc = ch & 7;
            const int pn = n / (2 * a.NB);
            const int mn = (n >> 1) - pn * a.NB;
            const int cn = n & 1;
            uint32_t pk[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              float vals[2];
#pragma unroll
              for (int dd = 0; dd < 2; ++dd) {
                const int u = atom * 64 + cc * 8 + q * 2 + dd;
                float v = 0.0f;
                const int ku = u >> 1, cu = u & 1;
                if (pn < 2 && u < 4 * R && ku / R == pn) {
                  const int r = ku - pn * R;
                  const float2 w = a.weff[(((size_t)c * 2 + pn) * a.NBW + mn) * R + r];
                  v = cn == 0 ? (cu == 0 ? w.x : -w.y) : (cu == 0 ? w.y : w.x);
                }
                vals[dd] = v;
              }
              pk[q] = u32_of(__floats2half2_rn(vals[0], vals[1]));
            }
            *reinterpret_cast<uint4 *>(wt + atom * (a.BN * 128) + n * 128 + ((cc ^ (n & 7)) << 4)) =
                make_uint4(pk[0], pk[1], pk[2], pk[3]);
          }
        }
        fence_proxy_async_smem();
        named_bar_sync(1, NUM_CONV_THREADS);
        if (ct == 0) mbar_arrive(&h.w_full[wb]);
      }
      int q_rel = qa0;   // next packet to release
      int q_wait = qa0;  // next packet not yet waited for
      // per-task packet/time cursor of the task's first sample, advanced by
      // one K block (64 samples) at a time: no division in the loop
      int cur_pkt[2], cur_tt[2];
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int task = ct + j * NUM_CONV_THREADS;
        const int r = (task >> 3) < R ? (task >> 3) : 0;
        const int qq = (task & 7) * 8 + h.offsets[r / a.Rpp];
        cur_pkt[j] = qq / Tp;
        cur_tt[j] = qq - cur_pkt[j] * Tp;
      }
      for (int kb = 0; kb < a.nkb; kb += 2) {
        const int s0 = kb * KBLK;
        const int qb = s0 < T ? min(a.P + 1, (min(s0 + 2 * KBLK - 1, T - 1) + off_max) / Tp) : qbN;
        bool ok = true;
        for (; q_wait <= qb && ok; ++q_wait) {
          const uint32_t gq = g_base + (q_wait - qa0);
          ok = mbar_wait(&h.pk_full[gq & ns_mask], (gq >> ns_shift) & 1u, abort_flag);
        }
        const uint32_t st0 = op_iter % NUM_OP_STAGES;
        const uint32_t st1 = (op_iter + 1) % NUM_OP_STAGES;
        ok = ok && mbar_wait(&h.op_empty[st0], ((op_iter / NUM_OP_STAGES) & 1u) ^ 1u, abort_flag);
        ok = ok && mbar_wait(&h.op_empty[st1], (((op_iter + 1) / NUM_OP_STAGES) & 1u) ^ 1u, abort_flag);
        failed |= !ok;
        const bool fast = (s0 + 2 * KBLK <= T) && Tp >= 8;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const int task = ct + j * NUM_CONV_THREADS;
          if (ok && task < R * 8) {
            const int oct = task & 7;
            const int r = task >> 3;
            const int f = r / a.Rpp;
            const int n = r - f * a.Rpp;
            const uint32_t fn_off = static_cast<uint32_t>((f * Tp) * Rpp4 + n * 4);
            uint32_t word[2][8], scw[2][8];
#pragma unroll
            for (int b = 0; b < 2; ++b) {
              // cursor of this block's first sample
              int pkt = cur_pkt[j], tt = cur_tt[j];
              if (b) {
                tt += KBLK;
                while (tt >= Tp) { tt -= Tp; ++pkt; }
              }
              if (fast) {
                const uint8_t *slot_a = ring_ptr + (size_t)((g_base + (pkt - qa0)) & ns_mask) * a.slot_stride;
                const uint8_t *slot_b = ring_ptr + (size_t)((g_base + (pkt + 1 - qa0)) & ns_mask) * a.slot_stride;
                const uint32_t sc_a = *reinterpret_cast<const uint32_t *>(slot_a + a.slot_bytes + r * 4);
                const uint32_t sc_b = tt + 7 >= Tp
                                          ? *reinterpret_cast<const uint32_t *>(slot_b + a.slot_bytes + r * 4)
                                          : sc_a;
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                  const int t = tt + e;
                  const bool cross = t >= Tp;
                  const uint8_t *sp = cross ? slot_b : slot_a;
                  word[b][e] = *reinterpret_cast<const uint32_t *>(sp + fn_off + (cross ? t - Tp : t) * Rpp4);
                  scw[b][e] = cross ? sc_b : sc_a;
                }
              } else {
                const int sfirst = s0 + b * KBLK + oct * 8;
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                  if (sfirst + e < T) {
                    const uint8_t *slot_ptr = ring_ptr + (size_t)((g_base + (pkt - qa0)) & ns_mask) * a.slot_stride;
                    word[b][e] = *reinterpret_cast<const uint32_t *>(slot_ptr + fn_off + tt * Rpp4);
                    scw[b][e] = *reinterpret_cast<const uint32_t *>(slot_ptr + a.slot_bytes + r * 4);
                  } else {
                    word[b][e] = 0;
                    scw[b][e] = 0;
                  }
                  if (++tt == Tp) {
                    tt = 0;
                    ++pkt;
                  }
                }
              }
            }
#pragma unroll
            for (int b = 0; b < 2; ++b) {
              uint32_t col[4][4];  // [row: p0re, p0im, p1re, p1im][pair of samples]
#pragma unroll
              for (int e = 0; e < 8; e += 2) {
                __half2 v0[2], v1[2];
                convert_word(word[b][e], scw[b][e], v0[0], v1[0]);
                convert_word(word[b][e + 1], scw[b][e + 1], v0[1], v1[1]);
                col[0][e >> 1] = __byte_perm(u32_of(v0[0]), u32_of(v0[1]), 0x5410);
                col[1][e >> 1] = __byte_perm(u32_of(v0[0]), u32_of(v0[1]), 0x7632);
                col[2][e >> 1] = __byte_perm(u32_of(v1[0]), u32_of(v1[1]), 0x5410);
                col[3][e >> 1] = __byte_perm(u32_of(v1[0]), u32_of(v1[1]), 0x7632);
              }
              uint8_t *stage = op_ptr + (b ? st1 : st0) * stage_bytes;
#pragma unroll
              for (int rr = 0; rr < 4; ++rr) {
                const int pol = rr >> 1;
                const int comp = rr & 1;
                const int u = 2 * (pol * R + r) + comp;
                uint4 *dst = reinterpret_cast<uint4 *>(stage + u * 128 + ((oct ^ (u & 7)) << 4));
                *dst = make_uint4(col[rr][0], col[rr][1], col[rr][2], col[rr][3]);
              }
            }
          }
          // advance the cursor by two K blocks
          cur_tt[j] += 2 * KBLK;
          while (cur_tt[j] >= Tp) { cur_tt[j] -= Tp; ++cur_pkt[j]; }
        }
        fence_proxy_async_smem();
        named_bar_sync(1, NUM_CONV_THREADS);
        // bookkeeping on the last converter thread
        if (ct == NUM_CONV_THREADS - 1) {
          mbar_arrive(&h.op_full[st0]);
          mbar_arrive(&h.op_full[st1]);
          int next = qbN + 1;
          if (kb + 2 < a.nkb && (kb + 2) * KBLK < T) next = ((kb + 2) * KBLK + off_min) / Tp;
          for (; q_rel < next; ++q_rel) {
            const uint32_t gq = g_base + (q_rel - qa0);
            mbar_arrive(&h.pk_empty[gq & ns_mask]);
          }
        }
        op_iter += 2;
      }
      g_base += npk;
    }
    if (failed && ct == 0) atomicOr(a.status, SF_DEVERR_TIMEOUT_CONVERT);
  }

  tc_fence_before();
  __syncthreads();
  if (warp == WARP_MMA) {
    tc_fence_after();
    tmem_dealloc(h.tmem_base, a.tmem_cols);
  }
}

int g_max_smem = 0;
bool g_attr_set[4] = {false, false, false, false};

template <bool DO_CORR, bool DO_BEAM>
cudaError_t launch_mode(const CorrArgs &a, size_t smem, int grid, cudaStream_t stream) {
  const int idx = (DO_CORR ? 1 : 0) + (DO_BEAM ? 2 : 0);
  if (!g_attr_set[idx]) {
    cudaError_t e = cudaFuncSetAttribute(sf_corrbeam_kernel<DO_CORR, DO_BEAM>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, g_max_smem);
    if (e != cudaSuccess) return e;
    g_attr_set[idx] = true;
  }
  sf_corrbeam_kernel<DO_CORR, DO_BEAM><<<grid, NTHREADS, smem, stream>>>(a);
  return cudaGetLastError();
}

uint32_t pow2_at_least(uint32_t x) {
  uint32_t p = 32;
  while (p < x) p <<= 1;
  return p;
}

}  // namespace

int sf_correlate_supported(const sf_plan *p, char *why, size_t why_len) {
  auto fail = [&](const char *msg) {
    if (why && why_len) snprintf(why, why_len, "%s", msg);
    return 0;
  };
  if (p->R > MAX_R) return fail("correlator supports at most 48 receivers per channel");
  if (p->F > MAX_F) return fail("correlator supports at most 64 FPGAs");
  if ((p->R * p->Tp * 4) % 16 != 0) return fail("R * Tp must be a multiple of 4 (16-byte packets)");
  return 1;
}

int sf_beam_tc_supported(const sf_plan *p, int n_beams_out) {
  return p->R <= MAX_R && p->F <= MAX_F && (p->R * p->Tp * 4) % 16 == 0 && n_beams_out <= MAX_BEAM_OUT;
}

// mode bit 0: correlate, bit 1: beamform (n_beams_out beams per pol from the
// plan's effective weights).
cudaError_t sf_launch_corrbeam(const sf_plan *p, const int8_t *samples, const int16_t *scales,
                               const int32_t *offsets, int32_t *vis, int n_beams_out, __half2 *beams,
                               int mode, cudaStream_t stream) {
  const bool do_corr = mode & 1, do_beam = (mode & 2) != 0;
  CorrArgs a;
  a.samples = samples;
  a.scales = scales;
  a.offsets = offsets;
  a.vis = vis;
  a.weff = p->d_weff;
  a.beams = beams;
  a.status = p->d_status;
  a.C = p->C;
  a.F = p->F;
  a.Tp = p->Tp;
  a.R = p->R;
  a.Rpp = p->Rpp;
  a.P = p->P;
  a.T = p->T;
  a.NBL = p->NBL;
  a.NR = ((4 * p->R + 15) / 16) * 16;
  a.stage_rows = std::max(a.NR, 128);
  a.nkb = ((p->T + KBLK - 1) / KBLK + 1) & ~1;  // converters fill K blocks in pairs
  a.slot_bytes = p->R * p->Tp * 4;
  a.slot_stride = a.slot_bytes + ((p->R * 4 + 15) / 16) * 16;
  a.NB = n_beams_out;
  a.NBW = 2 * p->B;
  a.BN = ((4 * n_beams_out + 15) / 16) * 16;
  a.katoms = (a.NR + 63) / 64;
  a.wtile_bytes = do_beam ? static_cast<uint32_t>(a.katoms * a.BN * 128) : 0u;
  const int ncols = a.NR + (a.NR > 128 ? a.NR - 128 : 0);
  a.nacc = 1;
  a.acc_stride = ncols;
  if (do_corr && do_beam) {
    a.beam_off = ncols;
    a.i32_off = ncols + 2 * a.BN;
    a.tmem_cols = pow2_at_least(a.i32_off + ncols);
  } else if (do_corr) {
    a.beam_off = 0;
    if (3 * ncols <= 512) {
      a.nacc = 2;  // drain one chunk while the next accumulates
      a.i32_off = 2 * ncols;
    } else {
      a.i32_off = 256;
    }
    a.tmem_cols = 512;
  } else {
    a.beam_off = 0;
    a.i32_off = 0;
    a.tmem_cols = pow2_at_least(2 * a.BN);
  }
  if (a.tmem_cols > 512) return cudaErrorInvalidConfiguration;

  if (!g_max_smem) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  }
  const size_t fixed = HEADER_BYTES + 1024 + (size_t)NUM_OP_STAGES * a.stage_rows * 128 + 2 * a.wtile_bytes;
  const int need_slots = 63 / p->Tp + 5;
  long avail = (long)g_max_smem - (long)fixed;
  int ns = avail > 0 ? (int)std::min<long>(MAX_SLOTS, avail / a.slot_stride) : 0;
  while (ns & (ns - 1)) ns &= ns - 1;  // round down to a power of two
  if (ns < need_slots) return cudaErrorInvalidConfiguration;
  a.num_slots = ns;
  const size_t smem = fixed + (size_t)ns * a.slot_stride;
  const int grid = std::max(1, std::min(p->C, p->num_sms));
  if (do_corr && do_beam) return launch_mode<true, true>(a, smem, grid, stream);
  if (do_corr) return launch_mode<true, false>(a, smem, grid, stream);
  return launch_mode<false, true>(a, smem, grid, stream);
}

cudaError_t sf_launch_correlate(const sf_plan *p, const int8_t *samples, const int16_t *scales,
                                const int32_t *offsets, int32_t *vis, cudaStream_t stream) {
  return sf_launch_corrbeam(p, samples, scales, offsets, vis, 0, nullptr, 1, stream);
}
