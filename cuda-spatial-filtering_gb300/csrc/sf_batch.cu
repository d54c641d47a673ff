// Batched form over sub-arrays of uneven size: one persistent tcgen05 launch
// correlates (or beamforms) every unit of a mixed batch -- units of 16, 36,
// 64, 128 or 256 receivers side by side -- from one work list.
//
// A unit is one channel-integration of one sub-array: int8 complex samples
// [T][R][Pol][2] (the packet layout with one FPGA and no window padding).
// Units are stored grouped by receiver count ("size class"), each class one
// contiguous array, so one 2-D TMA tensor map per class addresses all of its
// units: rows = samples of consecutive units, 4R bytes per row.
//
// Per 128-sample stage a unit's samples form the operand X[t][u],
// u = 4 r + 2 pol + comp (the byte order of a sample row), cut into 64-value
// atoms.  TMA loads an atom's int8 bytes ([128 t][64 B], zero-filled past 4R)
// into an int8 ring; converter warps turn them into fp16 atoms
// [128 t][128 B] with the 128-byte swizzle in an fp16 ring ("slabs" of up to
// four atoms); one thread issues tcgen05.mma on the slabs:
//   * correlate: the Gram G = X^T X block by block.  A work item is one row
//     block of 128 u (M = 128, or M = 64 when at most 64 rows remain) against
//     a column chunk of at most 160 u at or right of the block's diagonal
//     (N <= 160: two fp32 chunk accumulators and the int32 running sums fit
//     the 512 tensor-memory columns).  fp32 sums of 1024 samples (|x| <= 128)
//     are exact and are drained into int32, so visibilities are bit-exact.
//     Entries i <= j of the packed triangle come from exactly one item.
//   * beamform: Y[t][n] = sum_u X[t][u] W[n][u] over K = 4R in slabs of the
//     stage's atoms, W the block-diagonal real form of the unit's effective
//     weights (n = pol, beam, re/im), fp32 accumulation, fp16 output
//     [Pol][NB][T][2] per unit.
// Replaces, for sub-arrays, the reference's fp16 ingest + TCC correlation +
// trim and the ccglib beamformer (spatial.cuh:55-304, lambda_gpu_pipeline.hpp:
// 640-671, 708-743, src/spatial.cu:176-200), which run one shape per build.
//
// Work list: the host deals the items to the CTAs (longest first, to the
// least-loaded CTA, by a cost model the autotuner can reweight); every CTA
// walks its own list.  Warp roles (16 warps): 0 tensor-memory owner + MMA
// issuer, 1 TMA producer, 4-7 epilogue (one tensor-memory lane quarter each),
// 2-3 and 8-15 converters.  Every mbarrier wait is bounded and reports
// through the status word.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <queue>
#include <vector>

#include "sf_batch.cuh"
#include "sf_common.cuh"

namespace {

constexpr int BT = 128;                   // samples per stage
constexpr uint32_t ATOM = BT * 128;       // fp16 atom: 128 samples x 64 values, 128-byte swizzle
constexpr uint32_t IATOM = BT * 64;       // int8 atom: 128 samples x 64 bytes
constexpr int MAX_SA = 4;                 // atoms per slab
constexpr int CHUNK = 8;                  // stages per exact fp32 chunk (1024 samples)
constexpr int NWARPS = 16;
constexpr int NTHREADS = NWARPS * 32;
constexpr int WARP_MMA = 0, WARP_TMA = 1, WARP_EPI0 = 4;
constexpr int NCONV = 10;                 // converter warps: 2, 3, 8..15
constexpr int NCT = NCONV * 32;
constexpr int MAX_RING = 4;
constexpr uint32_t HEADER = 1024;
constexpr uint32_t SUSPEND = 20000;
constexpr int ACC_STRIDE = 160;           // tensor-memory columns between the two fp32 chunk accumulators
constexpr int I32_OFF = 320;              // int32 running sums

struct __align__(8) Header {
  uint64_t i8_full[MAX_RING], i8_empty[MAX_RING];
  uint64_t f16_full[MAX_RING], f16_empty[MAX_RING];
  uint64_t acc_full[2], acc_empty[2];
  uint64_t w_full, w_empty;
  uint64_t mma_done;
  uint32_t tmem_base;
  int abort;
};
static_assert(sizeof(Header) <= HEADER, "header");

__device__ __forceinline__ uint64_t desc_sw128(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((addr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
  d |= static_cast<uint64_t>(1u) << 46;
  d |= static_cast<uint64_t>(2u) << 61;
  return d;
}

__device__ __forceinline__ uint32_t u32_of(__half2 h) { return *reinterpret_cast<uint32_t *>(&h); }
__device__ __forceinline__ __half2 h2_of(uint32_t u) { return *reinterpret_cast<__half2 *>(&u); }

// four int8 (one 32-bit word) -> two half2, exactly: 0x6400 | b is the fp16
// value 1024 + b; subtracting 1152 leaves b - 128 = x.
__device__ __forceinline__ void int8x4_to_half(uint32_t word, uint32_t &o0, uint32_t &o1) {
  const uint32_t biased = word ^ 0x80808080u;
  const __half2 bias = h2_of(0x64806480u);
  o0 = u32_of(__hsub2(h2_of(__byte_perm(biased, 0x64646464u, 0x4140)), bias));
  o1 = u32_of(__hsub2(h2_of(__byte_perm(biased, 0x64646464u, 0x4342)), bias));
}

// Beam operand precisions (SF_BEAM_*): fp16 or bf16 samples and weights
// (kind::f16, exact samples); e4m3 samples and weights (kind::f8f6f4, samples
// rounded to e4m3); e4m3 weights with exact samples split as
// x = 16 (x >> 4) + (x & 15), both parts exact in e4m3, two MMAs per K step.
enum : int { OP_F16 = 0, OP_BF16 = 1, OP_E4M3 = 2, OP_E4M3_SPLIT = 3 };

__device__ __forceinline__ uint32_t bf16x2_of(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&v);
}

// two floats -> two e4m3 bytes (round to nearest, saturate to the finite range)
__device__ __forceinline__ uint32_t e4m3x2_of(float lo, float hi) {
  const __nv_fp8x2_storage_t v = __nv_cvt_float2_to_fp8x2(make_float2(lo, hi), __NV_SATFINITE, __NV_E4M3);
  return static_cast<uint32_t>(v);
}

// four int8 of a word -> four e4m3 bytes of f(x) for f = rounding (mode 0),
// 16 (x >> 4) (mode 1) or x & 15 (mode 2); the last two are exact in e4m3
__device__ __forceinline__ uint32_t int8x4_to_e4m3(uint32_t word, int mode) {
  float v[4];
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const int x = static_cast<int8_t>((word >> (8 * b)) & 0xFFu);
    v[b] = mode == 0 ? static_cast<float>(x) : (mode == 1 ? static_cast<float>(16 * (x >> 4)) : static_cast<float>(x & 15));
  }
  return e4m3x2_of(v[0], v[1]) | (e4m3x2_of(v[2], v[3]) << 16);
}

SF_DEVICE void umma_f8(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

struct BatchArgs {
  CUtensorMap tmap[SF_BATCH_MAX_CLASSES];  // int8 [rows][4R bytes] per size class
  const SfBatchUnit *units;
  const SfBatchItem *items;
  const int *cta_first;  // [grid + 1]: CTA b walks order[cta_first[b] .. cta_first[b+1])
  const int *order;
  int T, nst;            // samples per unit, stages per unit
  int32_t *vis;
  const float2 *weff;    // [unit][Pol][NB][R] at unit.weff_off
  __half2 *beams;        // [unit][Pol][NB][T] at unit.beam_off
  int NB, BN;            // beams per pol written (all slots), beam MMA N = round16(4 NBG)
  int NBG;               // beams per pol of one beam item (a group of the NB)
  const float *scales;   // fp8 operands: per-beam weight scale [unit][Pol][NB] (weights / scale in e4m3)
  int sa, ni, nf;        // atoms per slab, int8 / fp16 ring depths
  uint32_t wtile_bytes;  // beam weight tile (katoms_max x BN x 128 B)
  uint32_t tmem_cols;
  uint32_t *status;
};

template <bool BEAM, int OP>
__global__ void __launch_bounds__(NTHREADS, 1) sf_batch_kernel(const __grid_constant__ BatchArgs a) {
  constexpr bool F8 = OP == OP_E4M3 || OP == OP_E4M3_SPLIT;
  extern __shared__ __align__(16) uint8_t smem[];
  Header &h = *reinterpret_cast<Header *>(smem);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t sbase = smem_u32(smem);
  const uint32_t i8_addr = (sbase + HEADER + 1023u) & ~1023u;
  const uint32_t i8_slab = static_cast<uint32_t>(a.sa) * IATOM;
  const uint32_t f16_addr = i8_addr + static_cast<uint32_t>(a.ni) * i8_slab;  // 1024-aligned (IATOM multiple)
  const uint32_t f16_slab = static_cast<uint32_t>(a.sa) * ATOM;
  const uint32_t w_addr = f16_addr + static_cast<uint32_t>(a.nf) * f16_slab;
  uint8_t *w_ptr = smem + (w_addr - sbase);
  const int first = a.cta_first[blockIdx.x], last = a.cta_first[blockIdx.x + 1];

  if (tid == 0) {
    for (int s = 0; s < a.ni; ++s) {
      mbar_init(&h.i8_full[s], 1);
      mbar_init(&h.i8_empty[s], NCONV);
    }
    for (int s = 0; s < a.nf; ++s) {
      mbar_init(&h.f16_full[s], NCONV);
      mbar_init(&h.f16_empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&h.acc_full[b], 1);
      mbar_init(&h.acc_empty[b], 4);
    }
    mbar_init(&h.w_full, NCONV);
    mbar_init(&h.w_empty, 1);
    mbar_init(&h.mma_done, 1);
    h.abort = 0;
    fence_mbarrier_init();
  }
  if (warp == WARP_MMA) {
    tmem_alloc(&h.tmem_base, a.tmem_cols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  volatile int *abort_flag = &h.abort;

  // slabs of an item: corr one per stage; beam ceil(katoms / sa) per stage
  auto slabs_per_stage = [&](const SfBatchItem &it) { return BEAM ? (it.natoms + a.sa - 1) / a.sa : 1; };
  auto slab_atoms = [&](const SfBatchItem &it, int g) {
    return BEAM ? min(a.sa, it.natoms - g * a.sa) : it.natoms;
  };
  auto slab_atom = [&](const SfBatchItem &it, int g, int k) {  // global atom index of slab slot k
    return BEAM ? g * a.sa + k : static_cast<int>((it.atoms >> (8 * k)) & 0xFFu);
  };

  if (warp == WARP_TMA) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      uint32_t g = 0;
      bool ok = true;
      for (int oi = first; oi < last && ok; ++oi) {
        const SfBatchItem it = a.items[a.order[oi]];
        const SfBatchUnit un = a.units[it.unit];
        const void *tm = &a.tmap[un.cls];
        const int nsl = slabs_per_stage(it);
        for (int st = 0; st < a.nst && ok; ++st)
          for (int gs = 0; gs < nsl && ok; ++gs, ++g) {
            const uint32_t s = g % a.ni, ph = (g / a.ni) & 1u;
            ok = mbar_wait(&h.i8_empty[s], ph ^ 1u, abort_flag, SUSPEND);
            if (!ok) break;
            const int na = slab_atoms(it, gs);
            mbar_arrive_expect_tx(&h.i8_full[s], na * IATOM);
            for (int k = 0; k < na; ++k)
              tma_load_2d(smem + (i8_addr - sbase) + s * i8_slab + k * IATOM, tm, 64 * slab_atom(it, gs, k),
                          static_cast<int>(un.row0) + st * BT, &h.i8_full[s]);
          }
      }
      const uint32_t begin = g > static_cast<uint32_t>(a.ni) ? g - a.ni : 0u;
      for (uint32_t q = begin; q < g; ++q) mbar_wait_drain(&h.i8_full[q % a.ni], (q / a.ni) & 1u);
      if (!ok) atomicOr(a.status, SF_DEVERR_TIMEOUT_TMA);
    }
  } else if (warp == WARP_MMA) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const uint32_t tmem = h.tmem_base;
      uint32_t g = 0, acc_iter = 0, beam_iter = 0;
      bool failed = false;
      for (int oi = first; oi < last; ++oi) {
        const SfBatchItem it = a.items[a.order[oi]];
        const int nsl = slabs_per_stage(it);
        if (BEAM) {
          failed |= !mbar_wait(&h.w_full, (oi - first) & 1, abort_flag, SUSPEND);
          tc_fence_after();
        }
        // beam: K-major A and B; bf16 operands set the format fields (bits 7-9, 10-12), e4m3 is format 0
        // of kind::f8f6f4; correlator: both operands MN-major (bits 15, 16)
        const uint32_t idesc = BEAM ? (umma_idesc_f16_f32(128, a.BN) | (OP == OP_BF16 ? (1u << 7) | (1u << 10) : 0u))
                                    : (umma_idesc_f16_f32(it.m, it.n) | (1u << 15) | (1u << 16));
        for (int st = 0; st < a.nst; ++st) {
          uint32_t abuf = 0, dacc = 0;
          const bool chunk_start = !BEAM && (st % CHUNK) == 0;
          const bool chunk_end = !BEAM && ((st % CHUNK) == CHUNK - 1 || st == a.nst - 1);
          if (BEAM) {
            abuf = beam_iter & 1u;
            failed |= !mbar_wait(&h.acc_empty[abuf], ((beam_iter >> 1) & 1u) ^ 1u, abort_flag, SUSPEND);
            tc_fence_after();
            dacc = tmem + abuf * a.BN;
          } else {
            abuf = acc_iter & 1u;
            if (chunk_start) {
              failed |= !mbar_wait(&h.acc_empty[abuf], ((acc_iter >> 1) & 1u) ^ 1u, abort_flag, SUSPEND);
              tc_fence_after();
            }
            dacc = tmem + abuf * ACC_STRIDE;
          }
          for (int gs = 0; gs < nsl; ++gs, ++g) {
            const uint32_t s = g % a.nf, ph = (g / a.nf) & 1u;
            const bool ok = mbar_wait(&h.f16_full[s], ph, abort_flag, SUSPEND);
            failed |= !ok;
            tc_fence_after();
            const uint32_t slab = f16_addr + s * f16_slab;
            if (ok && !*abort_flag) {
              if (BEAM && !F8) {
                const int na = slab_atoms(it, gs);
                for (int k = 0; k < na; ++k) {
                  const uint64_t ad = desc_sw128(slab + k * ATOM, 16, 1024);
                  const uint64_t bd = desc_sw128(w_addr + (gs * a.sa + k) * (a.BN * 128), 16, 1024);
#pragma unroll
                  for (int ks = 0; ks < 4; ++ks)
                    umma_f16(dacc, ad + ((ks * 32) >> 4), bd + ((ks * 32) >> 4), idesc,
                             (gs == 0 && k == 0 && ks == 0) ? 0u : 1u);
                }
              } else if (BEAM) {
                // e4m3 atoms of 128 u (two int8 boxes each): [hi (or rounded) atoms][lo atoms]
                const int nf8 = (slab_atoms(it, gs) + 1) >> 1;
                const int half = a.sa >> 1;
                for (int k = 0; k < nf8; ++k) {
                  const uint64_t bd = desc_sw128(w_addr + (gs * half + k) * (a.BN * 128), 16, 1024);
                  const uint64_t ad = desc_sw128(slab + k * ATOM, 16, 1024);
#pragma unroll
                  for (int ks = 0; ks < 4; ++ks)
                    umma_f8(dacc, ad + ((ks * 32) >> 4), bd + ((ks * 32) >> 4), idesc,
                            (gs == 0 && k == 0 && ks == 0) ? 0u : 1u);
                  if (OP == OP_E4M3_SPLIT) {
                    const uint64_t al = desc_sw128(slab + (half + k) * ATOM, 16, 1024);
#pragma unroll
                    for (int ks = 0; ks < 4; ++ks) umma_f8(dacc, al + ((ks * 32) >> 4), bd + ((ks * 32) >> 4), idesc, 1u);
                  }
                }
              } else {
                const uint64_t ad = desc_sw128(slab, ATOM, 1024);
                const uint64_t bd = desc_sw128(slab + it.b_slot * ATOM, ATOM, 1024);
#pragma unroll
                for (int ks = 0; ks < BT / 16; ++ks)
                  umma_f16(dacc, ad + ((ks * 2048) >> 4), bd + ((ks * 2048) >> 4), idesc,
                           (chunk_start && ks == 0) ? 0u : 1u);
              }
            }
            umma_commit(&h.f16_empty[s]);
          }
          if (BEAM) {
            umma_commit(&h.acc_full[abuf]);
            ++beam_iter;
          } else if (chunk_end) {
            umma_commit(&h.acc_full[abuf]);
            ++acc_iter;
          }
        }
        if (BEAM) umma_commit(&h.w_empty);
      }
      umma_commit(&h.mma_done);
      mbar_wait_drain(&h.mma_done, 0);
      if (failed) atomicOr(a.status, SF_DEVERR_TIMEOUT_MMA);
    }
  } else if (warp >= WARP_EPI0 && warp < WARP_EPI0 + 4) {
    // ---------------- epilogue ----------------
    const int q4 = warp - WARP_EPI0;  // tensor-memory lane quarter
    const uint32_t tq = h.tmem_base + (static_cast<uint32_t>(q4 * 32) << 16);
    uint32_t acc_iter = 0, beam_iter = 0;
    bool failed = false;
    for (int oi = first; oi < last; ++oi) {
      const SfBatchItem it = a.items[a.order[oi]];
      const SfBatchUnit un = a.units[it.unit];
      const int R = un.R;
      for (int st = 0; st < a.nst; ++st) {
        if (BEAM) {
          const uint32_t buf = beam_iter & 1u;
          const bool ok = mbar_wait(&h.acc_full[buf], (beam_iter >> 1) & 1u, abort_flag, SUSPEND);
          failed |= !ok;
          tc_fence_after();
          const int t = st * BT + q4 * 32 + lane;
          __half2 *dst = a.beams + un.beam_off + t;
          // this item's beams: c0 .. c0 + n - 1 of every pol; tile column pair (pol, local beam)
          for (int cb = 0; cb < a.BN / 16; ++cb) {
            uint32_t v[16];
            tmem_ld16(tq + buf * a.BN + cb * 16, v);
            tmem_wait_ld();
            if (ok) {
#pragma unroll
              for (int e2 = 0; e2 < 8; ++e2) {
                const int lo = cb * 8 + e2;
                const int pn = lo / a.NBG, mn = lo - pn * a.NBG;
                if (pn < 2 && mn < it.n) {
                  const int col = pn * a.NB + it.c0 + mn;
                  const float sc = F8 ? a.scales[((size_t)it.unit * 2 + pn) * a.NB + it.c0 + mn] : 1.0f;
                  dst[(size_t)col * a.T] =
                      __floats2half2_rn(sc * __uint_as_float(v[2 * e2]), sc * __uint_as_float(v[2 * e2 + 1]));
                }
              }
            }
          }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&h.acc_empty[buf]);
          ++beam_iter;
          continue;
        }
        if (!((st % CHUNK) == CHUNK - 1 || st == a.nst - 1)) continue;
        const uint32_t buf = acc_iter & 1u;
        const bool ok = mbar_wait(&h.acc_full[buf], (acc_iter >> 1) & 1u, abort_flag, SUSPEND);
        failed |= !ok;
        tc_fence_after();
        const bool first_chunk = st < CHUNK, last_chunk = st == a.nst - 1;
        // this lane's accumulator row: M = 128 rows in lanes 0..127; M = 64 rows l in lanes (l % 16) + 32 (l / 16)
        const int row = it.m == 128 ? q4 * 32 + lane : (lane < 16 ? q4 * 16 + lane : 1 << 20);
        const int u = it.row0 + row;
        const int k = u >> 1, comp = u & 1, p = k & 1, i = k >> 1;
        const bool row_ok = ok && u < 4 * R;
        // (i, j, p, q, comp) sits at 8 (j (j + 1) / 2 + i) + 4 p + 2 q + comp of
        // the unit's visibilities; column pair m = 2 j + q is warp-uniform
        int32_t *const vis_u = a.vis + un.vis_off;
        const int lane_off = 8 * i + 4 * p + comp;
        for (int cb = 0; cb < it.n / 16; ++cb) {
          uint32_t fv[16], sv[16];
          tmem_ld16(tq + buf * ACC_STRIDE + cb * 16, fv);
          if (!first_chunk) tmem_ld16(tq + I32_OFF + cb * 16, sv);
          tmem_wait_ld();
          int acc[16];
#pragma unroll
          for (int e = 0; e < 16; ++e)
            acc[e] = (first_chunk ? 0 : static_cast<int>(sv[e])) + __float2int_rn(__uint_as_float(fv[e]));
          if (!last_chunk) {
            uint32_t out[16];
#pragma unroll
            for (int e = 0; e < 16; ++e) out[e] = static_cast<uint32_t>(acc[e]);
            tmem_st16(tq + I32_OFF + cb * 16, out);
            continue;
          }
          // final chunk: combine (re, im) row pairs and store the packed upper triangle
#pragma unroll
          for (int e2 = 0; e2 < 8; ++e2) {
            const int other = __shfl_xor_sync(0xffffffffu, acc[2 * e2 + 1], 1);
            const int val = comp ? acc[2 * e2] - other : acc[2 * e2] + other;
            const int m = (it.c0 >> 1) + cb * 8 + e2;
            const int j = m >> 1;
            if (row_ok && 2 * m < 4 * R && i <= j) vis_u[4 * j * (j + 1) + 2 * (m & 1) + lane_off] = val;
          }
        }
        if (!last_chunk) tmem_wait_st();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&h.acc_empty[buf]);
        ++acc_iter;
      }
    }
    if (failed && lane == 0) atomicOr(a.status, SF_DEVERR_TIMEOUT_EPILOGUE);
  } else {
    // ---------------- converters ----------------
    const int cw = warp >= 8 ? warp - 6 : warp - 2;  // 0..9
    const int ct = cw * 32 + lane;
    uint32_t g = 0;
    bool failed = false;
    const uint32_t i8s = i8_addr, f16s = f16_addr;
    for (int oi = first; oi < last; ++oi) {
      const SfBatchItem it = a.items[a.order[oi]];
      const SfBatchUnit un = a.units[it.unit];
      const int nsl = slabs_per_stage(it);
      if (BEAM) {
        // weight tile of this unit: B[n][u] K-major, one [BN rows][128 B] block per atom,
        // n = (pol, beam, re/im), u = (receiver, pol, re/im), block-diagonal real form
        const bool ok = mbar_wait(&h.w_empty, ((oi - first) & 1) ^ 1, abort_flag, SUSPEND);
        failed |= !ok;
        if (ok) {
          const int R = un.R;
          // 16-byte chunks per row: 8 per 64-u atom (16-bit), 8 per 128-u atom (e4m3)
          const int vper = F8 ? 16 : 8;  // u values per chunk
          const int natw = F8 ? (it.natoms + 1) >> 1 : it.natoms;
          const int nchunk = natw * 8;
          for (int task = ct; task < a.BN * nchunk; task += NCT) {
            const int n = task / nchunk, ch = task - n * nchunk;
            const int atom = ch >> 3, cc = ch & 7;
            const int pn = n / (2 * a.NBG), mn = (n >> 1) - pn * a.NBG, cn = n & 1;
            const bool beam_ok = pn < 2 && mn < it.n;
            const float inv = F8 && beam_ok ? 1.0f / a.scales[((size_t)it.unit * 2 + pn) * a.NB + it.c0 + mn] : 1.0f;
            float vals[16];
#pragma unroll
            for (int dd = 0; dd < 16; ++dd) {
              vals[dd] = 0.0f;
              if (dd >= vper) continue;
              const int uu = atom * (8 * vper) + cc * vper + dd;
              const int r = uu >> 2, pu = (uu >> 1) & 1, cu = uu & 1;
              if (beam_ok && uu < 4 * R && pu == pn) {
                const float2 w = a.weff[un.weff_off + ((size_t)pn * a.NB + it.c0 + mn) * R + r];
                vals[dd] = (cn == 0 ? (cu == 0 ? w.x : -w.y) : (cu == 0 ? w.y : w.x)) * inv;
              }
            }
            uint32_t pk[4];
#pragma unroll
            for (int qq = 0; qq < 4; ++qq) {
              if (OP == OP_F16) pk[qq] = u32_of(__floats2half2_rn(vals[2 * qq], vals[2 * qq + 1]));
              else if (OP == OP_BF16) pk[qq] = bf16x2_of(vals[2 * qq], vals[2 * qq + 1]);
              else pk[qq] = e4m3x2_of(vals[4 * qq], vals[4 * qq + 1]) | (e4m3x2_of(vals[4 * qq + 2], vals[4 * qq + 3]) << 16);
            }
            *reinterpret_cast<uint4 *>(w_ptr + atom * (a.BN * 128) + n * 128 + ((cc ^ (n & 7)) << 4)) =
                make_uint4(pk[0], pk[1], pk[2], pk[3]);
          }
        }
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&h.w_full);
      }
      for (int st = 0; st < a.nst; ++st)
        for (int gs = 0; gs < nsl; ++gs, ++g) {
          const uint32_t si = g % a.ni, sf = g % a.nf;
          bool ok = mbar_wait(&h.i8_full[si], (g / a.ni) & 1u, abort_flag, SUSPEND);
          ok = ok && mbar_wait(&h.f16_empty[sf], ((g / a.nf) & 1u) ^ 1u, abort_flag, SUSPEND);
          failed |= !ok;
          if (ok && !F8) {
            const int na = slab_atoms(it, gs);
            // task = (atom slot, sample t, 16-byte quarter q of the atom's 64 bytes)
            for (int task = ct; task < na * BT * 4; task += NCT) {
              const int k = task >> 9, t = (task >> 2) & (BT - 1), q = task & 3;
              const uint4 v = lds128(i8s + si * i8_slab + k * IATOM + t * 64 + q * 16);
              uint32_t o[8];
              if (OP == OP_BF16) {
                const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                  const float x0 = static_cast<float>(static_cast<int8_t>(w4[b] & 0xFF));
                  const float x1 = static_cast<float>(static_cast<int8_t>((w4[b] >> 8) & 0xFF));
                  const float x2 = static_cast<float>(static_cast<int8_t>((w4[b] >> 16) & 0xFF));
                  const float x3 = static_cast<float>(static_cast<int8_t>(w4[b] >> 24));
                  o[2 * b] = bf16x2_of(x0, x1);
                  o[2 * b + 1] = bf16x2_of(x2, x3);
                }
              } else {
                int8x4_to_half(v.x, o[0], o[1]);
                int8x4_to_half(v.y, o[2], o[3]);
                int8x4_to_half(v.z, o[4], o[5]);
                int8x4_to_half(v.w, o[6], o[7]);
              }
              const uint32_t row = f16s + sf * f16_slab + k * ATOM + t * 128;
              sts128(row + (((2 * q) ^ (t & 7)) << 4), o[0], o[1], o[2], o[3]);
              sts128(row + (((2 * q + 1) ^ (t & 7)) << 4), o[4], o[5], o[6], o[7]);
            }
          } else if (ok) {
            // e4m3: int8 box k fills half (k & 1) of 128-u atom k >> 1 (hi / rounded part), and of atom
            // sa / 2 + (k >> 1) (lo part, split only); boxes past the unit's atoms are zeros
            const int na = slab_atoms(it, gs);
            const int nbox = ((na + 1) >> 1) << 1;
            const int half = a.sa >> 1;
            for (int task = ct; task < nbox * BT * 4; task += NCT) {
              const int k = task >> 9, t = (task >> 2) & (BT - 1), q = task & 3;
              const uint4 v = k < na ? lds128(i8s + si * i8_slab + k * IATOM + t * 64 + q * 16) : make_uint4(0, 0, 0, 0);
              const int c = ((k & 1) << 2) + q;  // 16-byte chunk of the 128-byte row
              const uint32_t row = f16s + sf * f16_slab + (k >> 1) * ATOM + t * 128 + ((c ^ (t & 7)) << 4);
              const int m0 = OP == OP_E4M3 ? 0 : 1;
              sts128(row, int8x4_to_e4m3(v.x, m0), int8x4_to_e4m3(v.y, m0), int8x4_to_e4m3(v.z, m0),
                     int8x4_to_e4m3(v.w, m0));
              if (OP == OP_E4M3_SPLIT)
                sts128(row + half * ATOM, int8x4_to_e4m3(v.x, 2), int8x4_to_e4m3(v.y, 2), int8x4_to_e4m3(v.z, 2),
                       int8x4_to_e4m3(v.w, 2));
            }
          }
          fence_proxy_async_smem();
          __syncwarp();
          if (lane == 0) {
            mbar_arrive(&h.i8_empty[si]);
            mbar_arrive(&h.f16_full[sf]);
          }
        }
    }
    if (failed && lane == 0) atomicOr(a.status, SF_DEVERR_TIMEOUT_CONVERT);
  }

  tc_fence_before();
  __syncthreads();
  if (warp == WARP_MMA) {
    tc_fence_after();
    tmem_dealloc(h.tmem_base, a.tmem_cols);
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
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

}  // namespace

size_t sf_batch_smem_bytes(bool beam, int sa, int ni, int nf, uint32_t wtile_bytes) {
  return HEADER + 1024 + (size_t)ni * sa * IATOM + (size_t)nf * sa * ATOM + (beam ? wtile_bytes : 0u);
}

// Work items of one unit of R receivers (see the file comment).
void sf_batch_corr_items(int unit, int R, std::vector<SfBatchItem> &out) {
  const int NR = ((4 * R + 15) / 16) * 16;  // Gram rows / columns holding data
  for (int row0 = 0; row0 < NR; row0 += 128) {
    const int rows = std::min(128, NR - row0);
    const int m = rows > 64 ? 128 : 64;
    const int nra = m / 64;  // row atoms
    for (int c0 = row0; c0 < NR;) {
      const int remaining = NR - c0;
      const bool diag = c0 == row0;
      const int n = diag ? (remaining <= 160 ? remaining : 128) : std::min(128, remaining);
      SfBatchItem it{};
      it.unit = unit;
      it.m = m;
      it.n = n;
      it.row0 = row0;
      it.c0 = c0;
      const int nca = (n + 63) / 64;  // column atoms
      uint32_t atoms = 0;
      int k = 0;
      if (diag) {
        // the row atoms are the first column atoms (a M = 128 item needs both)
        const int na = std::max(nca, nra);
        for (; k < na; ++k) atoms |= static_cast<uint32_t>(row0 / 64 + k) << (8 * k);
        it.b_slot = 0;
      } else {
        for (int r = 0; r < nra; ++r, ++k) atoms |= static_cast<uint32_t>(row0 / 64 + r) << (8 * k);
        it.b_slot = k;
        for (int c = 0; c < nca; ++c, ++k) atoms |= static_cast<uint32_t>(c0 / 64 + c) << (8 * k);
      }
      it.natoms = k;
      it.atoms = atoms;
      out.push_back(it);
      c0 += n;
    }
  }
}

cudaError_t sf_batch_encode_maps(const SfBatchLaunch &L, const int8_t *samples, CUtensorMap *maps) {
  PFN_cuTensorMapEncodeTiled_v12000 encode = encoder();
  if (!encode) return cudaErrorNotSupported;
  for (int c = 0; c < L.n_classes; ++c) {
    const int R = L.class_R[c];
    const cuuint64_t dims[2] = {(cuuint64_t)(4 * R), (cuuint64_t)L.class_rows[c]};
    const cuuint64_t strides[1] = {(cuuint64_t)(4 * R)};
    const cuuint32_t box[2] = {64, BT};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = encode(&maps[c], CU_TENSOR_MAP_DATA_TYPE_UINT8, 2,
                        const_cast<int8_t *>(samples + L.class_base[c]), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
  }
  return cudaSuccess;
}

cudaError_t sf_batch_launch(const SfBatchLaunch &L, bool beam, const int8_t *samples, int32_t *vis,
                            const float2 *weff, __half2 *beams, uint32_t *status, cudaStream_t stream) {
  BatchArgs a;
  memset(&a, 0, sizeof(a));
  cudaError_t e = sf_batch_encode_maps(L, samples, a.tmap);
  if (e != cudaSuccess) return e;
  a.units = L.d_units;
  a.items = beam ? L.d_beam_items : L.d_corr_items;
  a.cta_first = beam ? L.d_beam_first : L.d_corr_first;
  a.order = beam ? L.d_beam_order : L.d_corr_order;
  a.T = L.T;
  a.nst = L.T / BT;
  a.vis = vis;
  a.weff = weff;
  a.beams = beams;
  a.NB = L.NB;
  a.NBG = L.NBG;
  a.BN = ((4 * L.NBG + 15) / 16) * 16;
  a.scales = L.d_scales;
  const int op = L.beam_op;
  const bool f8 = op == OP_E4M3 || op == OP_E4M3_SPLIT;
  a.sa = beam ? L.beam_sa : MAX_SA;
  a.ni = beam ? L.beam_ni : L.corr_ni;
  a.nf = beam ? L.beam_nf : L.corr_nf;
  a.wtile_bytes = beam ? static_cast<uint32_t>((f8 ? (L.max_atoms + 1) / 2 : L.max_atoms) * a.BN * 128) : 0u;
  a.tmem_cols = 512;
  a.status = status;
  if (beam && (a.BN > 256 || 2 * a.BN > 512)) return cudaErrorInvalidConfiguration;
  if (beam && f8 && ((a.sa & 1) || !a.scales)) return cudaErrorInvalidConfiguration;
  const size_t smem = sf_batch_smem_bytes(beam, a.sa, a.ni, a.nf, a.wtile_bytes);
  if (smem > (size_t)sf_device_max_smem()) return cudaErrorInvalidConfiguration;
  const int grid = beam ? L.beam_grid : L.corr_grid;
  if (grid <= 0) return cudaSuccess;
  const void *fn = nullptr;
  if (!beam) fn = reinterpret_cast<const void *>(sf_batch_kernel<false, OP_F16>);
  else if (op == OP_BF16) fn = reinterpret_cast<const void *>(sf_batch_kernel<true, OP_BF16>);
  else if (op == OP_E4M3) fn = reinterpret_cast<const void *>(sf_batch_kernel<true, OP_E4M3>);
  else if (op == OP_E4M3_SPLIT) fn = reinterpret_cast<const void *>(sf_batch_kernel<true, OP_E4M3_SPLIT>);
  else fn = reinterpret_cast<const void *>(sf_batch_kernel<true, OP_F16>);
  e = sf_smem_optin(fn, smem);
  if (e != cudaSuccess) return e;
  if (!beam) sf_batch_kernel<false, OP_F16><<<grid, NTHREADS, smem, stream>>>(a);
  else if (op == OP_BF16) sf_batch_kernel<true, OP_BF16><<<grid, NTHREADS, smem, stream>>>(a);
  else if (op == OP_E4M3) sf_batch_kernel<true, OP_E4M3><<<grid, NTHREADS, smem, stream>>>(a);
  else if (op == OP_E4M3_SPLIT) sf_batch_kernel<true, OP_E4M3_SPLIT><<<grid, NTHREADS, smem, stream>>>(a);
  else sf_batch_kernel<true, OP_F16><<<grid, NTHREADS, smem, stream>>>(a);
  return cudaGetLastError();
}

// Per-beam weight scales for e4m3 operands: s = max over receivers of
// max(|re w|, |im w|) / 448 (the largest finite e4m3), 1 for an all-zero beam.
__global__ void sf_beam_scales_kernel(const SfBatchUnit *units, const float2 *weff, int n_units, int NB,
                                      float *scales) {
  const int row = blockIdx.x * blockDim.y + threadIdx.y;  // (unit, pol, beam)
  if (row >= n_units * 2 * NB) return;
  const int unit = row / (2 * NB), pb = row - unit * 2 * NB;
  const SfBatchUnit un = units[unit];
  const float2 *w = weff + un.weff_off + (size_t)pb * un.R;
  float m = 0.0f;
  for (int r = threadIdx.x; r < un.R; r += 32) m = fmaxf(m, fmaxf(fabsf(w[r].x), fabsf(w[r].y)));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (threadIdx.x == 0) scales[row] = m > 0.0f ? m / 448.0f : 1.0f;
}

cudaError_t sf_batch_launch_scales(const SfBatchLaunch &L, int n_units, const float2 *weff, float *scales,
                                   cudaStream_t stream) {
  const dim3 block(32, 8);
  const int rows = n_units * 2 * L.NB;
  sf_beam_scales_kernel<<<(rows + 7) / 8, block, 0, stream>>>(L.d_units, weff, n_units, L.NB, scales);
  return cudaGetLastError();
}

// Deals items to `grid` CTAs: longest first, each to the least-loaded CTA
// (ties to the lowest index).  cost(item) = stages x (mma_weight x M N / 128
// + conv_weight x atoms per slab x slabs per stage).
void sf_batch_schedule(const std::vector<SfBatchItem> &items, const std::vector<SfBatchUnit> &units, int nst,
                       bool beam, int sa, int nb, int grid, double conv_weight, std::vector<int> &first,
                       std::vector<int> &order) {
  const int n = static_cast<int>(items.size());
  std::vector<double> cost(n);
  for (int i = 0; i < n; ++i) {
    const SfBatchItem &it = items[i];
    double mma, conv;
    if (beam) {
      const int bn = ((4 * nb + 15) / 16) * 16;
      mma = 128.0 * bn * it.natoms * 64 / 8192.0;
      conv = it.natoms;
    } else {
      mma = static_cast<double>(it.m) * it.n * 128 / 8192.0;
      conv = it.natoms;
    }
    (void)sa;
    (void)units;
    cost[i] = nst * (mma + conv_weight * conv);
  }
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return cost[x] > cost[y]; });
  using Load = std::pair<double, int>;
  std::priority_queue<Load, std::vector<Load>, std::greater<Load>> heap;
  for (int b = 0; b < grid; ++b) heap.push({0.0, b});
  std::vector<std::vector<int>> per(grid);
  for (int i : idx) {
    Load l = heap.top();
    heap.pop();
    per[l.second].push_back(i);
    l.first += cost[i];
    heap.push(l);
  }
  first.assign(grid + 1, 0);
  order.clear();
  for (int b = 0; b < grid; ++b) {
    first[b] = static_cast<int>(order.size());
    // within a CTA, keep units together (their items share L2-resident samples)
    std::sort(per[b].begin(), per[b].end(), [&](int x, int y) { return items[x].unit < items[y].unit; });
    order.insert(order.end(), per[b].begin(), per[b].end());
  }
  first[grid] = static_cast<int>(order.size());
}
