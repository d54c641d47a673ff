// Tensor-core correlator: one integration of int8 complex voltages in the
// packet layout -> exact int32 visibilities in the trimmed packed-triangle
// layout.  Replaces the reference's fp16 conversion + layout permutations +
// Tensor Core Correlator + trim (include/spatial/spatial.cuh:55-304,
// include/spatial/pipeline/lambda_gpu_pipeline.hpp:640-671, src/spatial.cu:176-200).
//
// Per channel the kernel forms the real Gram matrix G = A A^T of the stacked
// real/imaginary rows of all receivers and polarisations (row u = 2k + comp,
// k = pol * R + receiver) with tcgen05 UMMA, fp16 operands and fp32
// accumulation in tensor memory.  The int8 x int16-scale products are exact in
// fp16 (|x s| <= 2048) and every 512-sample chunk of fp32 partial sums is exact
// (|sum| <= 512 * 2 * 128^2 = 2^24), so each chunk is drained into int32
// running sums held in tensor memory; the visibilities come out bit-exact.
//   Re V(k,m) = G[2k][2m] + G[2k+1][2m+1],  Im V(k,m) = G[2k+1][2m] - G[2k][2m+1]
// Rows 0..127 of G come from one M=128 x N=NR MMA; when NR > 128 the rows
// 128..NR-1 x columns 128..NR-1 come from a second M=128 x N=NR-128 MMA and
// the rest of those rows follow from V(k,m) = conj(V(m,k)).
//
// CTA roles (one persistent CTA per SM, 16 warps):
//   warp 0      producer: one bulk (TMA) copy per packet [F][Tp][Rpp][Pol][2]
//               of a channel into a shared-memory ring, plus the packet's
//               int16 scales by 4-byte cp.async, both completing on the
//               slot's mbarrier
//   warp 1      TMEM allocation + the single-thread UMMA issuer
//   warps 4-7   epilogue: drain fp32 chunks into int32, emit visibilities
//   warps 2-3, 8-15  converters: ring (int8) -> swizzled fp16 operand tiles,
//               applying the per-packet scale and the per-FPGA window offset
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
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t TMEM_I32 = 256;   // column offset of the int32 running sums
constexpr uint32_t HEADER_BYTES = 2048;
constexpr int MAX_R = 48;            // NR + (NR - 128) <= 256 tensor-memory columns

struct CorrArgs {
  const int8_t *samples;
  const int16_t *scales;
  const int32_t *offsets;
  int32_t *vis;
  uint32_t *status;
  int C, F, Tp, R, Rpp, P, T, NBL;
  int NR;          // operand rows holding data: round_up(4R, 16)
  int stage_rows;  // rows per operand stage: max(NR, 128)
  int nkb;         // K blocks per channel
  int slot_bytes;  // one packet of one channel: R * Tp * 4 bytes
  int slot_stride; // slot_bytes + the packet's scales (R * 4 bytes), rounded to 16
  int num_slots;   // packet ring depth (power of two)
};

struct __align__(8) Header {
  uint64_t pk_full[MAX_SLOTS];
  uint64_t pk_empty[MAX_SLOTS];
  uint64_t op_full[NUM_OP_STAGES];
  uint64_t op_empty[NUM_OP_STAGES];
  uint64_t acc_full;
  uint64_t acc_empty;
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
  const __half2 bias = __floats2half2_rn(1152.0f, 1152.0f);
  __half2 x01 = __hsub2(h01, bias);  // exact integers in [-128, 127]
  __half2 x23 = __hsub2(h23, bias);
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
  p0 = x01;
  p1 = x23;
}

__device__ __forceinline__ void emit_vis(const CorrArgs &a, int c, int p, int i, int q, int j,
                                         int comp, int val) {
  const size_t idx =
      ((((size_t)c * a.NBL + baseline_of(i, j)) * 2 + p) * 2 + q) * 2 + comp;
  a.vis[idx] = val;
}

__global__ void __launch_bounds__(NTHREADS, 1) sf_corr_kernel(const CorrArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  Header &h = *reinterpret_cast<Header *>(smem);
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane = tid & 31;

  const uint32_t sbase = smem_u32(smem);
  const uint32_t op_addr = (sbase + HEADER_BYTES + 1023u) & ~1023u;
  uint8_t *op_ptr = smem + (op_addr - sbase);
  const uint32_t stage_bytes = static_cast<uint32_t>(a.stage_rows) * 128u;
  uint8_t *ring_ptr = op_ptr + NUM_OP_STAGES * stage_bytes;
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
    mbar_init(&h.acc_full, 1);
    mbar_init(&h.acc_empty, 4);
    mbar_init(&h.mma_done, 1);
    h.abort = 0;
    fence_mbarrier_init();
  }
  for (int f = tid; f < a.F; f += NTHREADS) h.offsets[f] = a.offsets[f];
  // Padding rows of the operand tiles must read as zero; data rows are
  // rewritten for every K block.
  {
    uint4 *z = reinterpret_cast<uint4 *>(op_ptr);
    const int n16 = NUM_OP_STAGES * stage_bytes / 16;
    for (int i = tid; i < n16; i += NTHREADS) z[i] = make_uint4(0, 0, 0, 0);
    fence_proxy_async_smem();
  }
  if (warp == WARP_MMA) {
    tmem_alloc(&h.tmem_base, TMEM_COLS);
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
        const bool ok = mbar_wait(&h.pk_empty[slot], ((g >> ns_shift) & 1u) ^ 1u, abort_flag);
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
      const uint32_t idesc_corner = umma_idesc_f16_f32(128, corner ? NR - 128 : 16);
      uint32_t op_iter = 0, acc_iter = 0;
      bool failed = false;
      for (int c = blockIdx.x; c < a.C; c += gridDim.x) {
        for (int kb = 0; kb < a.nkb; ++kb) {
          const uint32_t st = op_iter % NUM_OP_STAGES;
          bool ok = mbar_wait(&h.op_full[st], (op_iter / NUM_OP_STAGES) & 1u, abort_flag);
          const bool chunk_start = (kb % CHUNK_KBLK) == 0;
          if (chunk_start) ok = mbar_wait(&h.acc_empty, (acc_iter & 1u) ^ 1u, abort_flag) && ok;
          tc_fence_after();
          if (ok) {
            const uint32_t base = op_addr + st * stage_bytes;
#pragma unroll
            for (int ks = 0; ks < KBLK / 16; ++ks) {
              const uint32_t acc = (!chunk_start || ks > 0) ? 1u : 0u;
              umma_f16(tmem, umma_desc_sw128(base + ks * 32), umma_desc_sw128(base + ks * 32),
                       idesc_main, acc);
              if (corner)
                umma_f16(tmem + NR, umma_desc_sw128(base + (NR - 128) * 128 + ks * 32),
                         umma_desc_sw128(base + 128 * 128 + ks * 32), idesc_corner, acc);
            }
          } else {
            failed = true;
          }
          umma_commit(&h.op_empty[st]);
          if ((kb % CHUNK_KBLK) == CHUNK_KBLK - 1 || kb == a.nkb - 1) {
            umma_commit(&h.acc_full);
            ++acc_iter;
          }
          ++op_iter;
        }
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
    uint32_t acc_iter = 0;
    bool failed = false;
    for (int c = blockIdx.x; c < a.C; c += gridDim.x) {
      for (int ch = 0; ch < nchunks; ++ch) {
        const bool ok = mbar_wait(&h.acc_full, acc_iter & 1u, abort_flag);
        failed |= !ok;
        tc_fence_after();
        const bool first = ch == 0;
        const bool last = ch == nchunks - 1;
        for (int cb = 0; cb < ncols / 16; ++cb) {
          uint32_t fv[16], sv[16];
          tmem_ld16(tmem + cb * 16, fv);
          if (!first) tmem_ld16(tmem + TMEM_I32 + cb * 16, sv);
          tmem_wait_ld();
          int acc[16];
#pragma unroll
          for (int e = 0; e < 16; ++e)
            acc[e] = (first ? 0 : static_cast<int>(sv[e])) + __float2int_rn(__uint_as_float(fv[e]));
          if (!last) {
            uint32_t out[16];
#pragma unroll
            for (int e = 0; e < 16; ++e) out[e] = static_cast<uint32_t>(acc[e]);
            tmem_st16(tmem + TMEM_I32 + cb * 16, out);
            continue;
          }
          // Final chunk of this channel: combine (re, im) row pairs and write.
          const bool main_region = cb * 16 < NR;
          const int u = main_region ? ew * 32 + lane : (NR - 128) + ew * 32 + lane;
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
        if (lane == 0) mbar_arrive(&h.acc_empty);
        ++acc_iter;
      }
    }
    if (failed && lane == 0) atomicOr(a.status, SF_DEVERR_TIMEOUT_EPILOGUE);
  } else if (warp >= WARP_CONV0 || warp == 2 || warp == 3) {
    // ---------------- converters ----------------
    const int ct = warp >= WARP_CONV0 ? (warp - WARP_CONV0 + 2) * 32 + lane : (warp - 2) * 32 + lane;
    uint32_t g_base = 0, op_iter = 0;
    bool failed = false;
    const int Rpp4 = a.Rpp * 4;
    for (int c = blockIdx.x; c < a.C; c += gridDim.x) {
      int q_rel = qa0;
      for (int kb = 0; kb < a.nkb; ++kb) {
        const int s0 = kb * KBLK;
        const int s1 = min(s0 + KBLK - 1, T - 1);
        const int qa = (s0 + off_min) / Tp;
        const int qb = min(a.P + 1, (s1 + off_max) / Tp);
        bool ok = true;
        for (int q = qa; q <= qb && ok; ++q) {
          const uint32_t gq = g_base + (q - qa0);
          ok = mbar_wait(&h.pk_full[gq & ns_mask], (gq >> ns_shift) & 1u, abort_flag);
        }
        const uint32_t st = op_iter % NUM_OP_STAGES;
        ok = ok && mbar_wait(&h.op_empty[st], ((op_iter / NUM_OP_STAGES) & 1u) ^ 1u, abort_flag);
        failed |= !ok;
        if (ok) {
          uint8_t *stage = op_ptr + st * stage_bytes;
          for (int task = ct; task < R * 8; task += NUM_CONV_THREADS) {
            const int oct = task & 7;
            const int r = task >> 3;
            const int f = r / a.Rpp;
            const int n = r - f * a.Rpp;
            const int sfirst = s0 + oct * 8;
            // packet / time of the first sample, then step forward
            int qq = sfirst + h.offsets[f];
            int pkt = qq / Tp;
            int tt = qq - pkt * Tp;
            const uint8_t *slot_ptr = ring_ptr + (size_t)((g_base + (pkt - qa0)) & ns_mask) * a.slot_stride;
            uint32_t scw = *reinterpret_cast<const uint32_t *>(slot_ptr + a.slot_bytes + r * 4);
            const uint8_t *src = slot_ptr + (f * Tp + tt) * Rpp4 + n * 4;
            uint32_t col[4][4];  // [row: p0re, p0im, p1re, p1im][pair of samples]
#pragma unroll
            for (int e = 0; e < 8; e += 2) {
              __half2 v0[2], v1[2];
#pragma unroll
              for (int dd = 0; dd < 2; ++dd) {
                uint32_t word = 0, sc = 0;
                if (sfirst + e + dd < T) {
                  word = *reinterpret_cast<const uint32_t *>(src);
                  sc = scw;
                }
                convert_word(word, sc, v0[dd], v1[dd]);
                // advance one sample (crossing into the next packet's slot if needed)
                if (++tt == Tp) {
                  tt = 0;
                  ++pkt;
                  slot_ptr = ring_ptr + (size_t)((g_base + (pkt - qa0)) & ns_mask) * a.slot_stride;
                  if (sfirst + e + dd + 1 < T)
                    scw = *reinterpret_cast<const uint32_t *>(slot_ptr + a.slot_bytes + r * 4);
                  src = slot_ptr + (f * Tp) * Rpp4 + n * 4;
                } else {
                  src += Rpp4;
                }
              }
              col[0][e >> 1] = __byte_perm(u32_of(v0[0]), u32_of(v0[1]), 0x5410);
              col[1][e >> 1] = __byte_perm(u32_of(v0[0]), u32_of(v0[1]), 0x7632);
              col[2][e >> 1] = __byte_perm(u32_of(v1[0]), u32_of(v1[1]), 0x5410);
              col[3][e >> 1] = __byte_perm(u32_of(v1[0]), u32_of(v1[1]), 0x7632);
            }
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
        fence_proxy_async_smem();
        named_bar_sync(1, NUM_CONV_THREADS);
        if (ct == 0) {
          mbar_arrive(&h.op_full[st]);
          const int next = (kb + 1 < a.nkb) ? ((kb + 1) * KBLK + off_min) / Tp : qbN + 1;
          for (; q_rel < next; ++q_rel) {
            const uint32_t gq = g_base + (q_rel - qa0);
            mbar_arrive(&h.pk_empty[gq & ns_mask]);
          }
        }
        ++op_iter;
      }
      g_base += npk;
    }
    if (failed && ct == 0) atomicOr(a.status, SF_DEVERR_TIMEOUT_CONVERT);
  }

  tc_fence_before();
  __syncthreads();
  if (warp == WARP_MMA) {
    tc_fence_after();
    tmem_dealloc(h.tmem_base, TMEM_COLS);
  }
}

int g_max_smem = 0;
int g_attr_set = 0;

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

cudaError_t sf_launch_correlate(const sf_plan *p, const int8_t *samples, const int16_t *scales,
                                const int32_t *offsets, int32_t *vis, cudaStream_t stream) {
  CorrArgs a;
  a.samples = samples;
  a.scales = scales;
  a.offsets = offsets;
  a.vis = vis;
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
  a.nkb = (p->T + KBLK - 1) / KBLK;
  a.slot_bytes = p->R * p->Tp * 4;
  a.slot_stride = a.slot_bytes + ((p->R * 4 + 15) / 16) * 16;

  if (!g_max_smem) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  }
  const size_t fixed = HEADER_BYTES + 1024 + (size_t)NUM_OP_STAGES * a.stage_rows * 128;
  const int need_slots = 63 / p->Tp + 5;
  long avail = (long)g_max_smem - (long)fixed;
  int ns = avail > 0 ? (int)std::min<long>(MAX_SLOTS, avail / a.slot_stride) : 0;
  while (ns & (ns - 1)) ns &= ns - 1;  // round down to a power of two
  if (ns < need_slots) return cudaErrorInvalidConfiguration;
  a.num_slots = ns;
  const size_t smem = fixed + (size_t)ns * a.slot_stride;
  if (!g_attr_set) {
    cudaError_t e = cudaFuncSetAttribute(sf_corr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         g_max_smem);
    if (e != cudaSuccess) return e;
    g_attr_set = 1;
  }
  const int grid = std::max(1, std::min(p->C, p->num_sms));
  sf_corr_kernel<<<grid, NTHREADS, smem, stream>>>(a);
  return cudaGetLastError();
}
