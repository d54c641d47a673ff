// Tensor-core correlator and beamformer over one integration of int8 complex
// voltages in the packet layout.
//
// One persistent CTA per SM streams its channels' packets once through
// shared memory (whole channels, then a balanced range of the remaining
// channels' stages; see WorkItems) and builds, per 128 samples, one fp16
// operand tile
//   X[t][u],  u = 4 r + 2 pol + comp   (receiver r, polarization, re/im)
// i.e. the packet's own byte order: for every sample the 4R values of the
// channel are contiguous.  The tile is stored as 64-value atoms
// [atom][t][128 bytes] with the 128-byte swizzle, so the tensor cores read it
//   * MN-major for the Gram G = X^T X (M/N = u, K = t), and
//   * K-major for the beamformer Y[t][n] = sum_u X[t][u] W[n][u] (M = t, K = u).
// Converting is then a straight element-wise int8 -> fp16 (x * scale) copy:
// one lane = one sample, two receivers, one 16-byte store.
//
//   * correlate: G accumulates in fp32 in tensor memory and is drained every
//     1024 samples into int32 running sums -> exact int32 visibilities in the
//     trimmed packed-triangle layout.  Replaces the reference's fp16 ingest +
//     layout permutations + Tensor Core Correlator + trim
//     (include/spatial/spatial.cuh:55-304, lambda_gpu_pipeline.hpp:640-671,
//     src/spatial.cu:176-200).
//       Re V(k,m) = G[2k][2m] + G[2k+1][2m+1],  Im V(k,m) = G[2k+1][2m] - G[2k][2m+1]
//     with k = 2 r + pol.  Rows 0..127 of G come from one M=128 x N=NR MMA,
//     rows and columns 128..NR-1 from an M=64 MMA over the third atom; the
//     rest is V(k,m) = conj(V(m,k)).
//   * beamform: Y[t][n] per 128 samples, W the block-diagonal real form of the
//     effective weights (n = pol, beam, re/im), fp32 accumulation, fp16 output
//     [C][Pol][NB][T][2].  Replaces the reference's col-major sample layout +
//     weight permutation + ccglib GEMM + half output (spatial.cuh:145-213,
//     376-418; lambda_gpu_pipeline.hpp:708-743).
//   * or both in one pass (the plain pipelines).
// Operands: fp16(x * scale) is exact for |x s| <= 2048 and equals the
// reference's ingest for unit gain; correlation chunks are exact while
// |partial sums| <= 2^24 (1024 samples of |x s| <= 128: every product of two
// int8 values is at most 2^14 in magnitude).
//
// CTA roles (16 warps):
//   warp 0           producer: one bulk (TMA) copy per packet [F][Tp][Rpp][Pol][2]
//                    plus the packet's scales by 4-byte cp.async, completing on
//                    the slot's mbarrier
//   warp 1           TMEM allocation + the single-thread UMMA issuer
//   warps 4-7        epilogue (one TMEM lane quarter each)
//   warps 2-3, 8-15  converters: ring (int8) -> swizzled fp16 tiles (per-packet
//                    scale, per-FPGA window offset); per channel the weight tile.
//                    One of them (the leader) acquires each stage's packets and
//                    operand stage ahead; another hands each written stage to
//                    the MMA issuer and returns its packets to the producer.
// Operand stages: three when they fit beside a packet ring deep enough to
// prefetch a stage (the correlator; the beamformer alone when its last K atom
// holds at most 16 values, stored compact as 32-byte rows with the 32-byte
// swizzle in the operand and weight tiles), else two.
// Every wait is bounded (about a second) and reports through the status word.
#include <algorithm>
#include <cstdio>

#include "sf_common.cuh"
#include "sf_plan.cuh"

namespace {

constexpr int KBLK = 64;         // samples per K block (chunk accounting)
constexpr int TILE_T = 128;      // samples per operand stage
constexpr uint32_t ATOM_BYTES = TILE_T * 128;  // one 64-value atom of a stage
constexpr int CHUNK_KBLK = 16;   // K blocks per exact fp32 chunk (1024 samples)
constexpr int MAX_OP_STAGES = 3;  // operand stages (two or three, as shared memory allows)
constexpr int NUM_WARPS = 16;
constexpr int NTHREADS = NUM_WARPS * 32;
constexpr int WARP_TMA = 0;
constexpr int WARP_MMA = 1;
constexpr int WARP_EPI0 = 4;
constexpr int WARP_CONV0 = 8;  // converters: warps 2-3 and 8-15
constexpr int NUM_CONV_WARPS = 10;  // nine converting warps + one leader
constexpr int NUM_CONV_THREADS = NUM_CONV_WARPS * 32;
constexpr int NUM_WORKERS = NUM_CONV_WARPS - 1;  // warps that convert
constexpr int HANDOFF_CWP = 3;  // converting warp that also hands finished stages on
constexpr uint32_t BAR_START = 1;  // named barrier that opens a stage to the converter group
constexpr int MAX_SLOTS = 32;
constexpr int MAX_F = 64;
constexpr uint32_t HEADER_BYTES = 3072;
constexpr int MAX_ITEMS = 64;  // work items of one CTA (whole channels + tail pieces)
constexpr int MAX_R = 48;
constexpr int MAX_BEAM_OUT = 16;  // beams (all slots) per pol in the tensor beamformer
// receiver pairs (16-byte chunks of a sample) one converter warp owns at most
constexpr int MAX_JP = (MAX_R / 2 + NUM_WORKERS - 1) / NUM_WORKERS;
constexpr uint32_t SUSPEND_NS = 20000;  // mbarrier suspend hint for waits off the MMA path

struct CorrArgs {
  const int8_t *samples;
  const int16_t *scales;
  const int32_t *offsets;
  const int32_t *perm;  // [2R] stream permutation ((src_r << 1) | src_pol, -1 = zero), or NULL
  int32_t *vis;
  const float2 *weff;  // [C][2][NBW][R]
  __half2 *beams;      // [C][2][NB][T]
  uint32_t *status;
  int C, F, Tp, R, Rpp, P, T, NBL;
  int NR;           // Gram rows/columns holding data: round_up(4R, 16)
  int natoms;       // 64-value atoms per operand stage: max(2, ceil(NR / 64))
  int nkb;          // K blocks per channel (even: stages hold two)
  int slot_bytes;   // one packet of one channel: R * Tp * 4 bytes
  int slot_stride;  // slot_bytes + the packet's scales, rounded to 16
  int num_slots;    // packet ring depth (power of two)
  int nstages;      // operand stages: 3 when they fit beside a ring deep enough to prefetch, else 2
  int prefetch;     // ring deep enough to hold a stage's packets and the next stage's
  uint32_t tp_magic;  // ceil(2^32 / Tp): q / Tp == umulhi(q, tp_magic) while q * Tp < 2^32
  int NB, NBW;      // beams written per pol; rows of weff per (c, p)
  int BN;           // beam MMA N = round_up(4 NB, 16)
  int katoms;       // 64-column K atoms of the weight tile: ceil(NR / 64)
  uint32_t wtile_bytes;
  uint32_t stage_bytes;  // one operand stage (natoms full atoms, or two + the compact last atom)
  int compact;  // beamformer alone with 128 < NR <= 144: the last K atom holds its 16 values as
                // 32-byte rows (32-byte swizzle) in the operand tile and the weight tile
  uint32_t tmem_cols, i32_off, beam_off;
  int nacc;  // fp32 chunk accumulators in tensor memory (2 = double-buffered)
  uint32_t acc_stride;  // tensor-memory columns between the fp32 accumulators
};

struct __align__(8) Header {
  uint64_t pk_full[MAX_SLOTS];
  uint64_t pk_empty[MAX_SLOTS];
  uint64_t op_full[MAX_OP_STAGES];
  uint64_t op_empty[MAX_OP_STAGES];
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
  int rx_off[MAX_R];   // byte offset of receiver r's word at packet time 0 within a slot
  int rx_woff[MAX_R];  // window offset (samples) of receiver r's FPGA
  uint32_t unit_bits[MAX_OP_STAGES];   // per operand stage: bit s = ring slot s holds a packet whose scales are all 1
  uint32_t stage_unit[MAX_OP_STAGES];  // per operand stage: every packet the stage reads has scales all 1
  int perm[2 * MAX_R];    // output stream 2 r + p <- source (src_r << 1) | src_pol, -1 = zero
  int n_items;
  int4 items[MAX_ITEMS];  // channel, first stage, end stage, whole (stored) or piece (atomics)
};
static_assert(sizeof(Header) <= HEADER_BYTES, "header too large");

// The work of one CTA: channels [0, full_end) are processed whole, C / G of
// them per CTA (channel b, b + G, ...); the stages of the remaining channels
// are concatenated and dealt out as one contiguous range per CTA, cut at
// channel boundaries into pieces.  Every CTA then carries the same number of
// stages to within one, instead of whole channels to within one (384 channels
// on 152 SMs: 2.53 channels each, not 3).  Pieces of a channel on different
// CTAs add their exact int32 partial visibilities with integer atomics into a
// region the launcher zeroes; whole channels store them.  Every role walks
// the same list in the same order.
struct WorkItems {
  int nst, G, b, full, full_end;
  int t, t1;  // cursor and end of this CTA's range of tail stages (32-bit: C * nst < 2^31)
  int i;      // whole channels handed out so far
  __device__ __forceinline__ WorkItems(int C, int nst_) : nst(nst_), G(gridDim.x), b(blockIdx.x), i(0) {
    full = C / G;
    full_end = full * G;
    const int ts = (C - full_end) * nst;  // < G * nst
    t = static_cast<int>((static_cast<unsigned>(ts) * static_cast<unsigned>(b)) / static_cast<unsigned>(G));
    t1 = static_cast<int>((static_cast<unsigned>(ts) * static_cast<unsigned>(b + 1)) / static_cast<unsigned>(G));
  }
  // Next item: channel c, stages [pb, pe); whole = stored, else atomically added.
  __device__ __forceinline__ bool next(int &c, int &pb, int &pe, bool &whole) {
    if (i < full) {
      c = b + i * G;
      ++i;
      pb = 0;
      pe = nst;
      whole = true;
      return true;
    }
    if (t >= t1) return false;
    const int tc = t / nst;
    c = full_end + tc;
    pb = t - tc * nst;
    pe = min(nst, pb + (t1 - t));
    t += pe - pb;
    whole = false;
    return true;
  }
};

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

// Shared-memory descriptor with explicit strides (128-byte swizzle).  K-major:
// lbo unused, sbo = 8-row group stride.  MN-major: lbo = stride between
// 64-value MN atoms, sbo = stride between 8-row K groups.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((addr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
  d |= static_cast<uint64_t>(1u) << 46;
  d |= static_cast<uint64_t>(2u) << 61;
  return d;
}

// K-major, 32-byte swizzle: rows of 16 fp16 values (one K16 step), 8-row groups
// 256 bytes apart.  Used for the compact last K atom of the beamformer.
__device__ __forceinline__ uint64_t desc_sw32(uint32_t addr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((addr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>(1u) << 16;          // lbo 16 bytes (unused: one atom along K)
  d |= static_cast<uint64_t>(256u >> 4) << 32;   // sbo
  d |= static_cast<uint64_t>(1u) << 46;
  d |= static_cast<uint64_t>(6u) << 61;
  return d;
}

// tcgen05.mma issue is serialised with the issuing thread's own instruction
// stream, so the issue loops below are straight-line: no branch between MMAs.
template <bool DO_CORR, bool DO_BEAM, bool CORNER>
__global__ void __launch_bounds__(NTHREADS, 1) sf_corrbeam_kernel(const CorrArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  Header &h = *reinterpret_cast<Header *>(smem);
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane = tid & 31;

  const uint32_t sbase = smem_u32(smem);
  const uint32_t op_addr = (sbase + HEADER_BYTES + 1023u) & ~1023u;
  uint8_t *op_ptr = smem + (op_addr - sbase);
  const uint32_t stage_bytes = a.stage_bytes;
  const uint32_t SO = static_cast<uint32_t>(a.nstages);
  const uint32_t w_addr = op_addr + SO * stage_bytes;  // weight tiles (1024-aligned)
  uint8_t *w_ptr = op_ptr + SO * stage_bytes;
  // operand stage of the it-th stage processed and the parity of its use
  auto stage_of = [&](uint32_t it, uint32_t &st, uint32_t &ph) {
    const uint32_t q = SO == 2u ? it >> 1 : __umulhi(it, 0x55555556u);  // it / SO
    st = it - q * SO;
    ph = q & 1u;
  };
  uint8_t *ring_ptr = w_ptr + (DO_BEAM ? 2 * a.wtile_bytes : 0u);
  const int NS = a.num_slots;
  const uint32_t ns_mask = static_cast<uint32_t>(NS - 1);
  const uint32_t ns_shift = __popc(ns_mask);

  if (tid == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(&h.pk_full[s], 1 + 32);
      mbar_init(&h.pk_empty[s], 1);
    }
    for (int s = 0; s < a.nstages; ++s) {
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
      mbar_init(&h.w_full[b], NUM_CONV_WARPS);
      mbar_init(&h.w_empty[b], 1);
    }
    mbar_init(&h.mma_done, 1);
    h.abort = 0;
    fence_mbarrier_init();
  }
  if (tid == 0) {
    WorkItems wi(a.C, a.nkb >> 1);
    int c, pb, pe, n = 0;
    bool whole;
    while (n < MAX_ITEMS && wi.next(c, pb, pe, whole)) h.items[n++] = make_int4(c, pb, pe, whole ? 1 : 0);
    h.n_items = n;  // the host keeps C / G + 2 <= MAX_ITEMS
  }
  for (int f = tid; f < a.F; f += NTHREADS) h.offsets[f] = a.offsets[f];
  for (int k = tid; k < 2 * a.R; k += NTHREADS) h.perm[k] = a.perm ? a.perm[k] : ((k >> 1) << 1) | (k & 1);
  for (int r = tid; r < a.R; r += NTHREADS) {
    const int f = r / a.Rpp;
    h.rx_off[r] = (f * a.Tp * a.Rpp + (r - f * a.Rpp)) * 4;
    h.rx_woff[r] = a.offsets[f];
  }
  // Rows of the operand tiles past 4R and padding of the weight tiles must
  // read as zero; the converters never write them.
  {
    uint4 *z = reinterpret_cast<uint4 *>(op_ptr);
    const int n16 = (SO * stage_bytes + (DO_BEAM ? 2 * a.wtile_bytes : 0u)) / 16;
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
  const int npairs = a.nkb >> 1;  // stages per channel
  // packets stages [pb, pe) read: [q_lo(pb), q_hi(pe)]
  auto q_lo = [&](int pb) { return (pb * TILE_T + off_min) / Tp; };
  auto q_hi = [&](int pe) { return min(a.P + 1, (min(pe * TILE_T, T) - 1 + off_max) / Tp); };
  volatile int *abort_flag = &h.abort;

  if (warp == WARP_TMA) {
    // ---------------- producer (whole warp) ----------------
    uint32_t g = 0;
    bool stop = false;
    for (int it = 0; it < h.n_items && !stop; ++it) {
      const int4 w = h.items[it];
      const int c = w.x, pb = w.y, pe = w.z;
      const int8_t *chan = a.samples + (size_t)c * (a.P + 2) * a.slot_bytes;
      const int16_t *chan_sc = a.scales + (size_t)c * (a.P + 2) * R * 2;
      const int qend = q_hi(pe);
      for (int q = q_lo(pb); q <= qend; ++q) {
        const uint32_t slot = g & ns_mask;
        const bool ok = mbar_wait(&h.pk_empty[slot], ((g >> ns_shift) & 1u) ^ 1u, abort_flag, 20000);
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
      // Gram: A and B both the operand tile read MN-major
      const uint32_t mn_major = (1u << 15) | (1u << 16);
      const uint32_t idesc_main = umma_idesc_f16_f32(128, NR) | mn_major;
      // rows/columns 128..NR-1: an M=64 MMA over the third atom (its
      // accumulator rows l sit in lanes (l % 16) + 32 (l / 16))
      const uint32_t idesc_corner = umma_idesc_f16_f32(64, CORNER ? NR - 128 : 16) | mn_major;
      const int nks = NR / 16;  // beam K steps (predicated, at most MAX_R / 4)
      // beam: A = the same tile read K-major (M = 128 samples), B = weights K-major
      const uint32_t idesc_beam = umma_idesc_f16_f32(128, a.BN);
      // descriptors at offset 0; an offset adds (bytes >> 4) to the start field
      const uint64_t d_mn0 = desc_sw128(op_addr, ATOM_BYTES, 1024);
      const uint64_t d_k0 = desc_sw128(op_addr, 16, 1024);
      const uint64_t d_w0 = desc_sw128(w_addr, 16, 1024);
      uint32_t op_iter = 0, acc_iter = 0, beam_iter = 0, cw = 0;
      bool failed = false;
      for (int it = 0; it < h.n_items; ++it, ++cw) {
        const int pb = h.items[it].y, pe = h.items[it].z;
        const uint32_t wb = cw & 1u;
        if (DO_BEAM) failed |= !mbar_wait(&h.w_full[wb], (cw >> 1) & 1u, abort_flag, SUSPEND_NS);
        const uint32_t woff = wb * a.wtile_bytes;
        for (int pr = pb; pr < pe; ++pr) {
          uint32_t st, ph;
          stage_of(op_iter, st, ph);
          bool ok = mbar_wait(&h.op_full[st], ph, abort_flag, SUSPEND_NS);
          tc_fence_after();
          const uint32_t soff = st * stage_bytes;
          if (DO_CORR) {
            // a chunk (CHUNK_KBLK K blocks from the item's first stage) starts
            // and ends on stage boundaries
            const int kb0 = 2 * (pr - pb);
            const bool chunk_start = (kb0 % CHUNK_KBLK) == 0;
            const bool chunk_end = ((kb0 + 1) % CHUNK_KBLK) == CHUNK_KBLK - 1 || pr == pe - 1;
            const uint32_t abuf = acc_iter % a.nacc;
            if (chunk_start) {
              ok = mbar_wait(&h.acc_empty[abuf], ((acc_iter / a.nacc) & 1u) ^ 1u, abort_flag, SUSPEND_NS) && ok;
              tc_fence_after();
            }
            failed |= !ok;
            const uint32_t go = ok ? 1u : 0u;
            const uint32_t dacc = tmem + abuf * a.acc_stride;
            const uint64_t dst = d_mn0 + (soff >> 4);
            // 8 K steps of 16 samples: K group pairs 2048 bytes apart
            umma_f16_if(dacc, dst, dst, idesc_main, chunk_start ? 0u : 1u, go);
            if (CORNER) umma_f16_if(dacc + NR, dst + (2 * ATOM_BYTES >> 4), dst + (2 * ATOM_BYTES >> 4), idesc_corner, chunk_start ? 0u : 1u, go);
#pragma unroll
            for (int ks = 1; ks < 2 * KBLK / 16; ++ks) {
              const uint64_t dm = dst + (ks * 2048 >> 4);
              umma_f16_if(dacc, dm, dm, idesc_main, 1u, go);
              if (CORNER) umma_f16_if(dacc + NR, dm + (2 * ATOM_BYTES >> 4), dm + (2 * ATOM_BYTES >> 4), idesc_corner, 1u, go);
            }
            if (chunk_end) {
              umma_commit(&h.acc_full[abuf]);
              ++acc_iter;
            }
          }
          if (DO_BEAM) {
            ok = mbar_wait(&h.beam_empty[beam_iter & 1u], ((beam_iter >> 1) & 1u) ^ 1u, abort_flag, SUSPEND_NS) && ok;
            tc_fence_after();
            failed |= !ok;
            {
              const uint32_t d = tmem + a.beam_off + (beam_iter & 1u) * a.BN;
              const uint64_t ad0 = d_k0 + (soff >> 4);
              const uint64_t bd0 = d_w0 + (woff >> 4);
              const uint32_t batom = (a.BN * 128) >> 4;
              // the compact last K atom (K step 8): its own 32-byte-swizzle descriptors
              const uint64_t ad2 = desc_sw32(op_addr + 2 * ATOM_BYTES + soff);
              const uint64_t bd2 = desc_sw32(w_addr + woff + 2 * a.BN * 128);
#pragma unroll
              for (int ks = 0; ks < MAX_R / 4; ++ks) {
                const uint32_t kof = ((ks & 3) * 32) >> 4;
                const bool c2 = ks == 8 && a.compact;
                umma_f16_if(d, c2 ? ad2 : ad0 + ((ks >> 2) * (ATOM_BYTES >> 4) + kof),
                            c2 ? bd2 : bd0 + ((ks >> 2) * batom + kof), idesc_beam, ks > 0 ? 1u : 0u,
                            (ok && ks < nks) ? 1u : 0u);
              }
            }
            umma_commit(&h.beam_full[beam_iter & 1u]);
            ++beam_iter;
          }
          umma_commit(&h.op_empty[st]);
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
    const int ncplx = 2 * a.NB;  // beam output columns (pol, beam)
    uint32_t acc_iter = 0, beam_iter = 0;
    bool failed = false;
    for (int it = 0; it < h.n_items; ++it) {
      const int4 w = h.items[it];
      const int c = w.x, pb = w.y, pe = w.z;
      for (int kb = 2 * pb; kb < 2 * pe; ++kb) {
        if (DO_BEAM && (kb & 1)) {
          const uint32_t buf = beam_iter & 1u;
          const bool ok = mbar_wait(&h.beam_full[buf], (beam_iter >> 1) & 1u, abort_flag, 20000);
          failed |= !ok;
          tc_fence_after();
          const int t = (kb >> 1) * TILE_T + ew * 32 + lane;
          const bool st_ok = ok && t < T;
          // the whole tile into registers, then the buffer goes back to the MMA
          // before any global store (an arrive would wait for the stores)
          const uint32_t tb = tmem + a.beam_off + buf * a.BN;
          const int nblk = a.BN / 16;  // at most MAX_BEAM_OUT / 4
          uint32_t v[MAX_BEAM_OUT / 4][16];
#pragma unroll
          for (int cb = 0; cb < MAX_BEAM_OUT / 4; ++cb)
            if (cb < nblk) tmem_ld16(tb + cb * 16, v[cb]);
          tmem_wait_ld();
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&h.beam_empty[buf]);
          if (st_ok) {
            // output column col = pol * NB + beam: Y[c][col][t]
            __half2 *dst = a.beams + ((size_t)c * ncplx) * T + t;
#pragma unroll
            for (int cb = 0; cb < MAX_BEAM_OUT / 4; ++cb) {
#pragma unroll
              for (int e2 = 0; e2 < 8; ++e2) {
                const int col = cb * 8 + e2;
                if (col < ncplx)
                  dst[(size_t)col * T] = __floats2half2_rn(__uint_as_float(v[cb][2 * e2]), __uint_as_float(v[cb][2 * e2 + 1]));
              }
            }
          }
          ++beam_iter;
        }
        if (!DO_CORR || !(((kb - 2 * pb) % CHUNK_KBLK) == CHUNK_KBLK - 1 || kb == 2 * pe - 1)) continue;

        const uint32_t abuf = acc_iter % a.nacc;
        const bool ok = mbar_wait(&h.acc_full[abuf], (acc_iter / a.nacc) & 1u, abort_flag, 20000);
        failed |= !ok;
        tc_fence_after();
        const bool first = kb - 2 * pb < CHUNK_KBLK;  // the item's first chunk
        const bool last = kb == 2 * pe - 1;           // the item's last chunk
        const uint32_t tacc = tmem + abuf * a.acc_stride;
        // the channel's visibilities: (i, j, p, q, comp) at 8 (j (j + 1) / 2 + i) + 4 p + 2 q + comp
        int32_t *const vis_c = a.vis + (size_t)c * a.NBL * 8;
        const bool whole = last && *reinterpret_cast<volatile int *>(&h.items[it].w) != 0;
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
          // Row/column u = 2k + comp, k = 2 r + pol.
          const bool main_region = cb * 16 < NR;
          const int u = main_region ? ew * 32 + lane : (lane < 16 ? 128 + ew * 16 + lane : 1 << 20);
          const int k = u >> 1;
          const int comp = u & 1;
          const int p = k & 1;
          const int i = k >> 1;
          const bool row_ok = ok && u < R4;
          const int m0 = main_region ? cb * 8 : 64 + ((cb * 16 - NR) >> 1);
          const int lane_off = 8 * i + 4 * p + comp;
          // Column pair m = 2 j + q is warp-uniform, so each store's address is
          // the lane's row offset plus a constant (a per-element index chain
          // made this write-out, not the tensor work, the kernel's tail).
          // Every i <= j lies in a main-tile row (i < 32) or in the corner
          // (i, j >= 32).
#pragma unroll
          for (int e2 = 0; e2 < 8; ++e2) {
            const int other = __shfl_xor_sync(0xffffffffu, acc[2 * e2 + 1], 1);
            const int val = comp ? acc[2 * e2] - other : acc[2 * e2] + other;
            const int m = m0 + e2;
            const int j = m >> 1;
            if (row_ok && 2 * m < R4 && i <= j) {
              int32_t *dst = vis_c + (4 * j * (j + 1) + 2 * (m & 1) + lane_off);
              if (whole) *dst = val;
              else atomicAdd(dst, val);  // exact: integer addition in any order
            }
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
    // Nine warps convert; the leader warp acquires each stage's resources (the
    // stage's packets, with a flag per packet whose scales are all 1, and a
    // free operand stage) one stage ahead and opens the stage to the
    // converters with a named barrier.  Passing the barrier that opens stage
    // pr also tells every warp that stage pr - 1 is written: one converting
    // warp (HANDOFF_CWP) then signals the MMA issuer for pr - 1 and returns
    // the packets no later stage needs before it converts its share of pr,
    // so the leader only acquires and the other converters touch no
    // mbarrier.  After an item's last stage one more barrier closes it; so
    // does one after every stage when the ring cannot hold two stages'
    // packets (the next stage is then acquired once this one's packets are
    // back).
    const int cwp = warp >= WARP_CONV0 ? warp - WARP_CONV0 + 2 : warp - 2;  // 0..9
    const int ct = cwp * 32 + lane;
    const bool leader = cwp == NUM_WORKERS;
    const bool handoff = cwp == HANDOFF_CWP;
    uint32_t g_base = 0, op_iter = 0, cw = 0;
    bool failed = false;
    const int nrp = (R + 1) >> 1;  // receiver pairs = 16-byte chunks per sample
    const uint32_t Rpp4 = static_cast<uint32_t>(a.Rpp * 4);
    const uint32_t sstride = static_cast<uint32_t>(a.slot_stride);
    const uint32_t ring_s = smem_u32(ring_ptr);
    const uint32_t op_s = smem_u32(op_ptr);
    // This warp owns receiver pairs jp = cwp + 9 k (rows u = 8 jp .. 8 jp + 7)
    // for all 128 samples of a stage: lane = sample within each 32-sample group.
    int woff0[MAX_JP];                   // window offset of the pair's first receiver
    uint32_t roff0[MAX_JP], dr1[MAX_JP]; // word offset in a slot; second receiver's word - first's
    uint32_t stoff[MAX_JP];              // this lane's 16-byte chunk in group 0 of a stage
    uint32_t gstr[MAX_JP];               // bytes between the 32-sample groups of that atom
    bool same[MAX_JP], has1[MAX_JP];
    int woff1[MAX_JP];
#pragma unroll
    for (int k = 0; k < MAX_JP; ++k) {
      const int jp = min(cwp + NUM_WORKERS * k, nrp - 1);
      const int r0 = 2 * jp, r1 = min(2 * jp + 1, R - 1);
      woff0[k] = h.rx_woff[r0];
      woff1[k] = h.rx_woff[r1];
      roff0[k] = h.rx_off[r0];
      dr1[k] = static_cast<uint32_t>(h.rx_off[r1] - h.rx_off[r0]);
      same[k] = woff1[k] == woff0[k];
      has1[k] = 2 * jp + 1 < R;
      // rows of 128 bytes (128-byte swizzle), or of 32 bytes in the compact last
      // atom (32-byte swizzle: the chunk flips with bit 2 of the sample)
      const bool cpt = a.compact && (jp >> 3) == 2;
      stoff[k] = cpt ? 2 * ATOM_BYTES + lane * 32 + (((jp & 1) ^ ((lane >> 2) & 1)) << 4)
                     : (jp >> 3) * ATOM_BYTES + lane * 128 + (((jp & 7) ^ (lane & 7)) << 4);
      gstr[k] = cpt ? 32 * 32 : 32 * 128;
    }
    uint32_t unit_bits = 0;  // leader: bit s = ring slot s holds a packet whose scales are all 1
    int q_rel = 0;           // hand-off warp: first packet not yet returned to the producer
    int q_wait = 0;          // leader: first packet not yet waited for
    bool acq_ok = true;
    // leader: wait for the packets of stage pr of the current channel and for
    // the operand stage of iteration `it` to be free; publish the packets'
    // scale flags and whether the whole stage is on unit scales
    auto acquire = [&](int pr, uint32_t gq0, uint32_t it) {
      const int s0 = pr * TILE_T;
      const int qb = s0 < T ? min(a.P + 1, static_cast<int>(__umulhi(static_cast<uint32_t>(min(s0 + TILE_T - 1, T - 1) + off_max), a.tp_magic)))
                            : q_hi(npairs);
      bool ok = true;
      const int q0 = q_wait;
      for (; q_wait <= qb && ok; ++q_wait) {
        const uint32_t gq = gq0 + q_wait;
        ok = mbar_wait(&h.pk_full[gq & ns_mask], (gq >> ns_shift) & 1u, abort_flag, SUSPEND_NS);
      }
      // scale flags of the new packets, two at a time: lanes 16 h + j read
      // scale words 4 j .. 4 j + 3 (R <= 48) of packet q + h
      for (int q = q0; q < q_wait; q += 2) {
        const int h2 = lane >> 4, j = lane & 15;
        const uint32_t sl = (gq0 + q + h2) & ns_mask;
        bool unit = true;
        if (q + h2 < q_wait && 4 * j < R) {
          const uint4 v = lds128(ring_s + sl * sstride + a.slot_bytes + 16 * j);
          unit = (v.x == 0x00010001u) && (4 * j + 1 >= R || v.y == 0x00010001u) &&
                 (4 * j + 2 >= R || v.z == 0x00010001u) && (4 * j + 3 >= R || v.w == 0x00010001u);
        }
        const uint32_t bad = __ballot_sync(0xffffffffu, !unit);
        const uint32_t sl0 = (gq0 + q) & ns_mask, sl1 = (gq0 + q + 1) & ns_mask;
        unit_bits = (bad & 0xffffu) ? (unit_bits & ~(1u << sl0)) : (unit_bits | (1u << sl0));
        if (q + 1 < q_wait) unit_bits = (bad >> 16) ? (unit_bits & ~(1u << sl1)) : (unit_bits | (1u << sl1));
      }
      // the whole stage on unit scales?
      uint32_t su = 1u;
      for (int q = static_cast<int>(__umulhi(static_cast<uint32_t>(s0 + off_min), a.tp_magic)); q <= qb; ++q)
        su &= unit_bits >> ((gq0 + q) & ns_mask);
      uint32_t ist, iph;
      stage_of(it, ist, iph);
      ok = ok && mbar_wait(&h.op_empty[ist], iph ^ 1u, abort_flag, SUSPEND_NS);
      if (lane == 0) {
        h.unit_bits[ist] = unit_bits;
        h.stage_unit[ist] = su & 1u;
      }
      if (!ok) {
        failed = true;
        if (lane == 0) *abort_flag = 1;
      }
      return ok;
    };
    for (int it = 0; it < h.n_items; ++it, ++cw) {
      const int c = h.items[it].x, pb = h.items[it].y, pe = h.items[it].z;
      const int qlo = q_lo(pb), qhi = q_hi(pe);
      if (DO_BEAM) {
        // weight tile for this channel: B[n][u], n = (pol, beam, re/im),
        // u = (receiver, pol, re/im), K-major, 128-byte swizzle, one
        // [BN rows][64 cols] block per K atom
        const uint32_t wb = cw & 1u;
        const bool ok = mbar_wait(&h.w_empty[wb], ((cw >> 1) & 1u) ^ 1u, abort_flag, SUSPEND_NS);
        failed |= !ok;
        if (ok) {
          uint8_t *wt = w_ptr + wb * a.wtile_bytes;
          // Only entries with the output's pol (pu == pn) and a real receiver
          // are nonzero; the rest of both tiles was zeroed at start and is
          // never written.  Weight w = weff[c][pn][mn][r] fills rows
          // n = 2 (pn NB + mn) + cn at columns u = 4 r + 2 pn + cu with
          // (w.x, -w.y) for cn = 0 and (w.y, w.x) for cn = 1.  Each thread
          // loads all its weights before storing any, so a channel's tile costs
          // one memory latency instead of one per 16-byte chunk (the serial
          // form was ~9 k cycles per channel between the stage loops).
          constexpr int MAXW = (2 * MAX_BEAM_OUT * MAX_R + NUM_CONV_THREADS - 1) / NUM_CONV_THREADS;
          const int nw = 2 * a.NB * R;
          float2 wv[MAXW];
#pragma unroll
          for (int k = 0; k < MAXW; ++k) {
            const int idx = ct + k * NUM_CONV_THREADS;
            if (idx < nw) {
              const int q = idx / R, r = idx - q * R;  // q = pn NB + mn
              const int pn = q / a.NB, mn = q - pn * a.NB;
              wv[k] = a.weff[(((size_t)c * 2 + pn) * a.NBW + mn) * R + r];
            }
          }
#pragma unroll
          for (int k = 0; k < MAXW; ++k) {
            const int idx = ct + k * NUM_CONV_THREADS;
            if (idx < nw) {
              const int q = idx / R, r = idx - q * R;
              const int pn = q / a.NB;
              const int n0 = 2 * q;
              const int u = 4 * r + 2 * pn;
              const int kk = u & 63, cc = kk >> 3;
              uint8_t *blk = wt + (u >> 6) * (a.BN * 128) + ((kk & 7) << 1);
              // 128-byte rows, or 32-byte rows in the compact last atom
              const bool cpt = a.compact && (u >> 6) == 2;
              const int n1 = n0 + 1;
              const uint32_t o0 = cpt ? n0 * 32 + (((cc & 1) ^ ((n0 >> 2) & 1)) << 4) : n0 * 128 + ((cc ^ (n0 & 7)) << 4);
              const uint32_t o1 = cpt ? n1 * 32 + (((cc & 1) ^ ((n1 >> 2) & 1)) << 4) : n1 * 128 + ((cc ^ (n1 & 7)) << 4);
              *reinterpret_cast<uint32_t *>(blk + o0) = u32_of(__floats2half2_rn(wv[k].x, -wv[k].y));
              *reinterpret_cast<uint32_t *>(blk + o1) = u32_of(__floats2half2_rn(wv[k].y, wv[k].x));
            }
          }
        }
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&h.w_full[wb]);
      }
      const uint32_t gq0 = g_base - static_cast<uint32_t>(qlo);  // ring index of packet q: gq0 + q
      q_rel = qlo;
      if (leader) {
        q_wait = qlo;
        acq_ok = acquire(pb, gq0, op_iter);
      }
      // first packet a stage starting at sample s reads
      auto first_packet = [&](int s) { return static_cast<int>(__umulhi(static_cast<uint32_t>(s + off_min), a.tp_magic)); };
      // hand-off warp: stage `st` is written; return packets below `next`
      auto hand_off = [&](uint32_t st, int next) {
        if (lane == 0) {
          mbar_arrive(&h.op_full[st]);
          for (; q_rel < next; ++q_rel) mbar_arrive(&h.pk_empty[(gq0 + q_rel) & ns_mask]);
        }
        __syncwarp();
      };
      for (int pr = pb; pr < pe; ++pr) {
        const int s0 = pr * TILE_T;
        uint32_t st, ph;
        stage_of(op_iter, st, ph);
        named_bar_sync(BAR_START, NUM_CONV_THREADS);  // stage pr is open
        if (leader) {
          // the next stage's resources while the converters work
          if (pr + 1 < pe && a.prefetch) acq_ok = acquire(pr + 1, gq0, op_iter + 1);
        } else {
          // stage pr - 1 is written: to the MMA issuer, with its packets
          // below stage pr's first
          if (handoff && pr > pb && a.prefetch) hand_off(st == 0u ? SO - 1u : st - 1u, first_packet(s0));
          const bool ok = *abort_flag == 0;
          const uint32_t ubits = *reinterpret_cast<volatile uint32_t *>(&h.unit_bits[st]);
          // every packet of the stage on unit scales and every sample inside the
          // integration: no per-sample scale or range tests
          const bool stage_fast = *reinterpret_cast<volatile uint32_t *>(&h.stage_unit[st]) != 0u && s0 + TILE_T <= T;
          const uint32_t stage_s = op_s + st * stage_bytes;
          if (ok && a.perm) {
            // permuted streams (reorder_streams semantics): every output stream
            // of a chunk loads its own source receiver / pol with that source's
            // FPGA window offset and packet scale
#pragma unroll
            for (int k = 0; k < MAX_JP; ++k) {
              const int jp = cwp + NUM_WORKERS * k;
              if (jp >= nrp) break;
#pragma unroll 1
              for (int g = 0; g < 4; ++g) {
                const int t = s0 + g * 32 + lane;
                uint32_t o[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                  const int r = 2 * jp + (e >> 1);
                  const int src = r < R && t < T ? h.perm[2 * r + (e & 1)] : -1;
                  float xr = 0.0f, xi = 0.0f;
                  if (src >= 0) {
                    const int sr = src >> 1, sp = src & 1;
                    const uint32_t qq = static_cast<uint32_t>(t + h.rx_woff[sr]);
                    const uint32_t pkt = __umulhi(qq, a.tp_magic);
                    const uint32_t tt = qq - pkt * static_cast<uint32_t>(Tp);
                    const uint32_t slot = ring_s + ((gq0 + pkt) & ns_mask) * sstride;
                    const uint32_t raw = lds16(slot + h.rx_off[sr] + tt * Rpp4 + 2 * sp);
                    const int sc = static_cast<int16_t>(lds16(slot + a.slot_bytes + sr * 4 + 2 * sp));
                    xr = static_cast<float>(static_cast<int8_t>(raw & 0xFFu) * sc);
                    xi = static_cast<float>(static_cast<int8_t>(raw >> 8) * sc);
                  }
                  o[e] = u32_of(__floats2half2_rn(xr, xi));  // fp16(x * scale)
                }
                sts128(stage_s + stoff[k] + g * gstr[k], o[0], o[1], o[2], o[3]);
              }
            }
          } else if (ok && stage_fast && off_min == off_max) {
            // one window offset for every FPGA: a lane's packet slot and time
            // within the packet are the same for every receiver, so each
            // 32-sample group's address is formed once
            uint32_t base[4];
#pragma unroll
            for (int g = 0; g < 4; ++g) {
              const uint32_t qq = static_cast<uint32_t>(s0 + g * 32 + lane + off_min);
              const uint32_t pkt = __umulhi(qq, a.tp_magic);
              const uint32_t tt = qq - pkt * static_cast<uint32_t>(Tp);
              base[g] = ring_s + ((gq0 + pkt) & ns_mask) * sstride + tt * Rpp4;
            }
#pragma unroll
            for (int k = 0; k < MAX_JP; ++k) {
              const int jp = cwp + NUM_WORKERS * k;
              if (jp >= nrp) break;
              uint32_t wd[4][2];
#pragma unroll
              for (int g = 0; g < 4; ++g) {
                const uint32_t a0 = base[g] + roff0[k];
                wd[g][0] = lds32(a0);
                wd[g][1] = has1[k] ? lds32(a0 + dr1[k]) : 0u;
              }
#pragma unroll
              for (int g = 0; g < 4; ++g) {
                // x -> fp16(x) by the 1024 + b bias trick
                uint32_t o[4];
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                  const uint32_t biased = wd[g][e] ^ 0x80808080u;
                  const __half2 bias = h2_of(0x64806480u);  // 1152
                  o[2 * e] = u32_of(__hsub2(h2_of(__byte_perm(biased, 0x64646464u, 0x4140)), bias));
                  o[2 * e + 1] = u32_of(__hsub2(h2_of(__byte_perm(biased, 0x64646464u, 0x4342)), bias));
                }
                sts128(stage_s + stoff[k] + g * gstr[k], o[0], o[1], o[2], o[3]);
              }
            }
          } else if (ok && stage_fast) {
#pragma unroll
            for (int k = 0; k < MAX_JP; ++k) {
              const int jp = cwp + NUM_WORKERS * k;
              if (jp >= nrp) break;
              uint32_t wd[4][2];
#pragma unroll
              for (int g = 0; g < 4; ++g) {
                const int t = s0 + g * 32 + lane;
                uint32_t qq = static_cast<uint32_t>(t + woff0[k]);
                uint32_t pkt = __umulhi(qq, a.tp_magic);
                uint32_t tt = qq - pkt * static_cast<uint32_t>(Tp);
                const uint32_t a0 = ring_s + ((gq0 + pkt) & ns_mask) * sstride + roff0[k] + tt * Rpp4;
                uint32_t a1 = a0 + dr1[k];
                if (!same[k]) {
                  qq = static_cast<uint32_t>(t + woff1[k]);
                  pkt = __umulhi(qq, a.tp_magic);
                  tt = qq - pkt * static_cast<uint32_t>(Tp);
                  a1 = ring_s + ((gq0 + pkt) & ns_mask) * sstride + roff0[k] + dr1[k] + tt * Rpp4;
                }
                wd[g][0] = lds32(a0);
                wd[g][1] = has1[k] ? lds32(a1) : 0u;
              }
#pragma unroll
              for (int g = 0; g < 4; ++g) {
                // x -> fp16(x) by the 1024 + b bias trick
                uint32_t o[4];
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                  const uint32_t biased = wd[g][e] ^ 0x80808080u;
                  const __half2 bias = h2_of(0x64806480u);  // 1152
                  o[2 * e] = u32_of(__hsub2(h2_of(__byte_perm(biased, 0x64646464u, 0x4140)), bias));
                  o[2 * e + 1] = u32_of(__hsub2(h2_of(__byte_perm(biased, 0x64646464u, 0x4342)), bias));
                }
                sts128(stage_s + stoff[k] + g * gstr[k], o[0], o[1], o[2], o[3]);
              }
            }
          } else if (ok) {
#pragma unroll
            for (int k = 0; k < MAX_JP; ++k) {
              const int jp = cwp + NUM_WORKERS * k;
              if (jp >= nrp) break;
              // loads of the four 32-sample groups first, then convert + store
              uint32_t wd[4][2], sl[4][2];
              bool unit = true;
#pragma unroll
              for (int g = 0; g < 4; ++g) {
                const int t = s0 + g * 32 + lane;
                const bool valid = t < T;
                uint32_t qq = static_cast<uint32_t>(t + woff0[k]);
                uint32_t pkt = __umulhi(qq, a.tp_magic);
                uint32_t tt = qq - pkt * static_cast<uint32_t>(Tp);
                sl[g][0] = (gq0 + pkt) & ns_mask;
                const uint32_t a0 = ring_s + sl[g][0] * sstride + roff0[k] + tt * Rpp4;
                uint32_t a1 = a0 + dr1[k];
                sl[g][1] = sl[g][0];
                if (!same[k]) {
                  qq = static_cast<uint32_t>(t + woff1[k]);
                  pkt = __umulhi(qq, a.tp_magic);
                  tt = qq - pkt * static_cast<uint32_t>(Tp);
                  sl[g][1] = (gq0 + pkt) & ns_mask;
                  a1 = ring_s + sl[g][1] * sstride + roff0[k] + dr1[k] + tt * Rpp4;
                }
                wd[g][0] = valid ? lds32(a0) : 0u;
                wd[g][1] = valid && has1[k] ? lds32(a1) : 0u;
                unit &= !valid || ((ubits >> sl[g][0]) & (ubits >> sl[g][1]) & 1u);
              }
              if (__all_sync(0xffffffffu, unit)) {
                // every scale is 1: x -> fp16(x) by the 1024 + b bias trick
#pragma unroll
                for (int g = 0; g < 4; ++g) {
                  uint32_t o[4];
#pragma unroll
                  for (int e = 0; e < 2; ++e) {
                    const uint32_t biased = wd[g][e] ^ 0x80808080u;
                    const __half2 bias = h2_of(0x64806480u);  // 1152
                    o[2 * e] = u32_of(__hsub2(h2_of(__byte_perm(biased, 0x64646464u, 0x4140)), bias));
                    o[2 * e + 1] = u32_of(__hsub2(h2_of(__byte_perm(biased, 0x64646464u, 0x4342)), bias));
                  }
                  sts128(stage_s + stoff[k] + g * gstr[k], o[0], o[1], o[2], o[3]);
                }
              } else {
                const int r0 = 2 * jp;
#pragma unroll
                for (int g = 0; g < 4; ++g) {
                  const bool valid = s0 + g * 32 + lane < T;
                  const uint32_t sc0 = valid ? lds32(ring_s + sl[g][0] * sstride + a.slot_bytes + r0 * 4) : 0x00010001u;
                  const uint32_t sc1 =
                      valid && has1[k] ? lds32(ring_s + sl[g][1] * sstride + a.slot_bytes + r0 * 4 + 4) : 0x00010001u;
                  __half2 a0, a1, b0, b1;
                  convert_word(wd[g][0], sc0, a0, a1);
                  convert_word(wd[g][1], sc1, b0, b1);
                  sts128(stage_s + stoff[k] + g * gstr[k], u32_of(a0), u32_of(a1), u32_of(b0), u32_of(b1));
                }
              }
            }
          }
          fence_proxy_async_smem();
        }
        ++op_iter;
        if (!a.prefetch && pr + 1 < pe) {
          named_bar_sync(BAR_START, NUM_CONV_THREADS);  // stage pr is written
          if (handoff) hand_off(st, first_packet(s0 + TILE_T));
          if (leader) acq_ok = acquire(pr + 1, gq0, op_iter);
        }
      }
      // the item's last stage is written: to the MMA issuer, with every packet
      named_bar_sync(BAR_START, NUM_CONV_THREADS);
      if (handoff) {
        uint32_t lst, lph;
        stage_of(op_iter - 1u, lst, lph);
        hand_off(lst, qhi + 1);
      }
      g_base += qhi - qlo + 1;
    }
    (void)acq_ok;
    if (failed && lane == 0) atomicOr(a.status, SF_DEVERR_TIMEOUT_CONVERT);
  }

  tc_fence_before();
  __syncthreads();
  if (warp == WARP_MMA) {
    tc_fence_after();
    tmem_dealloc(h.tmem_base, a.tmem_cols);
  }
}

template <bool DO_CORR, bool DO_BEAM, bool CORNER>
cudaError_t launch_mode(const CorrArgs &a, size_t smem, int grid, cudaStream_t stream) {
  cudaError_t e = sf_smem_optin(reinterpret_cast<const void *>(sf_corrbeam_kernel<DO_CORR, DO_BEAM, CORNER>), smem);
  if (e != cudaSuccess) return e;
  sf_corrbeam_kernel<DO_CORR, DO_BEAM, CORNER><<<grid, NTHREADS, smem, stream>>>(a);
  return cudaGetLastError();
}

template <bool DO_CORR, bool DO_BEAM>
cudaError_t launch_corner(const CorrArgs &a, size_t smem, int grid, cudaStream_t stream) {
  return a.NR > 128 ? launch_mode<DO_CORR, DO_BEAM, true>(a, smem, grid, stream)
                    : launch_mode<DO_CORR, DO_BEAM, false>(a, smem, grid, stream);
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
  // packet index by multiply-high: every window-shifted sample (< (P + 2) Tp) times Tp below 2^32
  if ((double)(p->P + 2) * p->Tp * p->Tp >= 4294967296.0) return fail("integration too long for the packet index");
  return 1;
}

int sf_beam_tc_supported(const sf_plan *p, int n_beams_out) {
  return sf_correlate_supported(p, nullptr, 0) && n_beams_out <= MAX_BEAM_OUT;
}

// One pass producing both visibilities and beams: the fp32 chunk accumulator,
// the int32 running sums and two beam tiles share the 512 tensor-memory
// columns.
int sf_corrbeam_fused_supported(const sf_plan *p, int n_beams_out) {
  if (!sf_beam_tc_supported(p, n_beams_out)) return 0;
  const int NR = ((4 * p->R + 15) / 16) * 16;
  const int ncols = NR + (NR > 128 ? NR - 128 : 0);
  const int BN = ((4 * n_beams_out + 15) / 16) * 16;
  return 2 * ncols + 2 * BN <= 512;
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
  a.perm = p->d_perm;
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
  a.natoms = std::max(2, (a.NR + 63) / 64);  // the M=128 Gram MMA always reads two atoms
  a.nkb = ((p->T + KBLK - 1) / KBLK + 1) & ~1;  // stages hold K blocks in pairs
  a.slot_bytes = p->R * p->Tp * 4;
  a.slot_stride = a.slot_bytes + ((p->R * 4 + 15) / 16) * 16;
  a.tp_magic = static_cast<uint32_t>((0x100000000ull + p->Tp - 1) / p->Tp);
  a.NB = n_beams_out;
  a.NBW = 2 * p->B;
  a.BN = ((4 * n_beams_out + 15) / 16) * 16;
  a.katoms = (a.NR + 63) / 64;
  // The beamformer alone reads the tile K-major only, so a last K atom with at
  // most 16 values can be stored as 32-byte rows: 36 instead of 48 KB per
  // operand stage at R = 36, which leaves room for a third operand stage.
  a.compact = (!do_corr && do_beam && a.NR > 128 && a.NR <= 144) ? 1 : 0;
  a.stage_bytes = a.compact ? 2 * ATOM_BYTES + TILE_T * 32 : static_cast<uint32_t>(a.natoms) * ATOM_BYTES;
  a.wtile_bytes = do_beam ? (a.compact ? ((2 * a.BN * 128 + a.BN * 32 + 1023u) & ~1023u)
                                       : static_cast<uint32_t>(a.katoms * a.BN * 128))
                          : 0u;
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

  const int max_smem = sf_device_max_smem();
  // packets one stage touches: (TILE_T - 1 + window spread <= 2 Tp) / Tp + 2, plus one in flight
  const int need_slots = (TILE_T - 1) / p->Tp + 5;
  const int prefetch_slots = (2 * TILE_T - 1) / p->Tp + 5;
  // ring depth beside `stages` operand stages (a power of two)
  auto ring_depth = [&](int stages) {
    const long fixed = HEADER_BYTES + 1024 + (long)stages * a.stage_bytes + 2 * (long)a.wtile_bytes;
    const long avail = (long)max_smem - fixed;
    int ns = avail > 0 ? (int)std::min<long>(MAX_SLOTS, avail / a.slot_stride) : 0;
    while (ns & (ns - 1)) ns &= ns - 1;  // round down to a power of two
    return ns;
  };
  // a third operand stage lets the converters run a stage ahead of the MMAs
  a.nstages = ring_depth(3) >= prefetch_slots ? 3 : 2;
  const int ns = ring_depth(a.nstages);
  if (ns < need_slots) return cudaErrorInvalidConfiguration;
  a.num_slots = ns;
  a.prefetch = ns >= prefetch_slots ? 1 : 0;
  const size_t smem = HEADER_BYTES + 1024 + (size_t)a.nstages * a.stage_bytes + 2 * (size_t)a.wtile_bytes +
                      (size_t)ns * a.slot_stride;
  const int grid = std::max(1, std::min(p->C, p->num_sms));
  // WorkItems computes (tail stages) x (CTA index) in 32 bits; a CTA holds at
  // most C / grid whole channels and two pieces
  if ((double)(p->C % grid) * (a.nkb / 2) * grid >= 4294967296.0) return cudaErrorInvalidConfiguration;
  if (p->C / grid + 2 > MAX_ITEMS) return cudaErrorInvalidConfiguration;
  if (do_corr) {
    // channels past the whole-channel share are summed from pieces by integer atomics
    const int full_end = (p->C / grid) * grid;
    if (full_end < p->C) {
      const size_t per = (size_t)p->NBL * 8;
      cudaError_t e = cudaMemsetAsync(vis + (size_t)full_end * per, 0, sizeof(int32_t) * (p->C - full_end) * per, stream);
      if (e != cudaSuccess) return e;
    }
  }
  if (do_corr && do_beam) return launch_corner<true, true>(a, smem, grid, stream);
  if (do_corr) return launch_corner<true, false>(a, smem, grid, stream);
  return launch_corner<false, true>(a, smem, grid, stream);
}

cudaError_t sf_launch_correlate(const sf_plan *p, const int8_t *samples, const int16_t *scales,
                                const int32_t *offsets, int32_t *vis, cudaStream_t stream) {
  return sf_launch_corrbeam(p, samples, scales, offsets, vis, 0, nullptr, 1, stream);
}
