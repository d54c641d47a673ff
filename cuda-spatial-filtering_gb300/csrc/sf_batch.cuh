// Internal types of the batched (uneven sub-array) form shared by its
// kernels (sf_batch.cu) and its C ABI (sf_batch_capi.cu).
#pragma once

#include <cuda.h>

#include <cstdint>
#include <vector>

#include "sf_plan.cuh"

constexpr int SF_BATCH_MAX_CLASSES = 8;  // distinct receiver counts in one batch

// One unit (one channel-integration of one sub-array), device side.
struct SfBatchUnit {
  long long row0;      // first sample row of the unit in its class's tensor map (index in class x T)
  long long vis_off;   // int32 elements: [R(R+1)/2][Pol][Pol][2]
  long long weff_off;  // float2 elements: [Pol][2B][R]
  long long beam_off;  // half2 elements: [Pol][2B][T]
  int R, cls;
};

// One work item of the batched correlator (row block x column chunk of a
// unit's Gram matrix) or beamformer (a whole unit).
struct SfBatchItem {
  int unit;
  int m, n;        // correlator MMA M and N
  int row0, c0;    // first Gram row and column (u index)
  int natoms;      // correlator: atoms per slab; beamformer: atoms of the unit (ceil(4R / 64))
                   // beamformer: m unused, c0 = first beam of the group, n = beams in the group
  int b_slot;      // correlator: slab slot of the first B atom
  uint32_t atoms;  // correlator: global atom index of each slab slot (one byte each)
};

// Everything one launch of the batched kernel needs (host copy).
struct SfBatchLaunch {
  int T, NB;  // samples per unit, beams per pol written (2B)
  int n_classes;
  int class_R[SF_BATCH_MAX_CLASSES];
  long long class_rows[SF_BATCH_MAX_CLASSES];  // units in the class x T
  long long class_base[SF_BATCH_MAX_CLASSES];  // byte offset of the class in the samples buffer
  int max_atoms;
  const SfBatchUnit *d_units;
  const SfBatchItem *d_corr_items, *d_beam_items;
  const int *d_corr_first, *d_corr_order, *d_beam_first, *d_beam_order;
  int corr_grid, beam_grid;
  int corr_ni, corr_nf;            // correlator int8 / fp16 ring depths (slabs of four atoms)
  int beam_sa, beam_ni, beam_nf;   // beamformer atoms per slab and ring depths
  int NBG;                         // beams per pol of one beamformer item
  int beam_op;                     // beam operand precision (SF_BEAM_*)
  const float *d_scales;           // per-beam weight scales of e4m3 operands [unit][Pol][NB]
};

size_t sf_batch_smem_bytes(bool beam, int sa, int ni, int nf, uint32_t wtile_bytes);
void sf_batch_corr_items(int unit, int R, std::vector<SfBatchItem> &out);
void sf_batch_schedule(const std::vector<SfBatchItem> &items, const std::vector<SfBatchUnit> &units, int nst,
                       bool beam, int sa, int nb, int grid, double conv_weight, std::vector<int> &first,
                       std::vector<int> &order);
cudaError_t sf_batch_launch(const SfBatchLaunch &L, bool beam, const int8_t *samples, int32_t *vis,
                            const float2 *weff, __half2 *beams, uint32_t *status, cudaStream_t stream);
cudaError_t sf_batch_launch_scales(const SfBatchLaunch &L, int n_units, const float2 *weff, float *scales,
                                   cudaStream_t stream);
