// Internal plan state shared by the C-ABI translation units.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/sf_capi.h"

struct sf_plan {
  sf_shape shape;
  int C, F, Tp, R, Rpp, P, B, T, NBL;
  int device;
  int num_sms;

  // Window offsets (samples into the (P+2)-packet buffer), one per FPGA.
  int32_t *d_off_aligned;  // Tp + sub-packet delay
  int32_t *d_off_packet;   // all zero
  int32_t *h_delays;       // host copy of the delays

  // Per-(channel, pol, receiver) complex factor d = gain x fine-delay phasor.
  float2 *d_factors;   // [C][2][R]
  float2 *h_gains;     // [C][2][R]
  float2 *h_phasors;   // [C][R]
  float2 *h_factors;   // [C][2][R] staging for the upload

  // Stream permutation (canonical output stream <- packet-order source), or
  // identity when d_perm is NULL: entry k = 2 r + p holds (src_r << 1) | src_pol,
  // -1 for a zero stream.
  int32_t *d_perm;     // [2R]
  int32_t *h_perm;     // [2R]

  __half2 *d_weights;  // [C][2][B][R]
  float2 *d_weff;      // [C][2][2B][R] effective weights for the beamformer
  int32_t *d_fixed_counts;  // [C]
  int32_t *h_fixed_counts;  // [C]

  // W_T^k (k < T) for the whole-integration spectra; NULL when T is not a
  // power of two in [64, 16384].
  float2 *d_spec_tw;
  // The 64-point DFT operand (fp16 hi + lo, swizzled) of the tensor-core
  // per-packet spectra; NULL unless Tp == 64.
  uint8_t *d_packet_dft;

  // Steering-synthesis inputs: [B][3] direction cosines then [R][3] antenna
  // positions (doubles), [R] connected flags, [C][2][R] calibration gains.
  double *d_steer;
  int32_t *d_steer_conn;
  float2 *d_steer_cal;
  // pinned staging of the same (so the upload is asynchronous) and the event
  // that marks the last upload's copies done (the staging is reused after it)
  double *h_steer;
  int32_t *h_steer_conn;
  float2 *h_steer_cal;
  cudaEvent_t steer_uploaded;

  // Scratch for the whole-chain entry points.
  int32_t *d_vis;      // [C][NBL][2][2][2]
  float *d_evals;      // [C][2][2][R]
  int32_t *d_counts;   // [C][2]
  uint32_t *d_status;  // error bits
};

// Opts `func` in to `bytes` of dynamic shared memory on the current device.
// The attribute is per device, so the helper remembers (device, kernel,
// bytes) under a mutex and calls cudaFuncSetAttribute once per device and
// kernel (again only for a larger size).  Thread-safe.
cudaError_t sf_smem_optin(const void *func, size_t bytes);
// The current device's opt-in shared-memory limit per block (cached per device).
int sf_device_max_smem();

// Launchers (one per translation unit); each returns a cudaError_t.
cudaError_t sf_launch_correlate(const sf_plan *p, const int8_t *samples, const int16_t *scales,
                                const int32_t *offsets, int32_t *vis, cudaStream_t stream);
int sf_correlate_supported(const sf_plan *p, char *why, size_t why_len);
// Tensor-core correlate (mode bit 0) and/or beamform (bit 1) in one pass.
cudaError_t sf_launch_corrbeam(const sf_plan *p, const int8_t *samples, const int16_t *scales,
                               const int32_t *offsets, int32_t *vis, int n_beams_out, __half2 *beams,
                               int mode, cudaStream_t stream);
int sf_beam_tc_supported(const sf_plan *p, int n_beams_out);
int sf_corrbeam_fused_supported(const sf_plan *p, int n_beams_out);

cudaError_t sf_launch_eig(const sf_plan *p, const int32_t *vis, int eig_mode, int k_rule,
                          float delta, int shrink, float *evals, float2 *evecs, int32_t *counts,
                          __half2 *proj, cudaStream_t stream);
int sf_eig_supported(const sf_plan *p, char *why, size_t why_len);

// One matrix of the batched (uneven sub-array) eigensolver: an n x n same-pol
// covariance read from the packed int32 upper triangle at vis + vis_off
// ([baseline][Pol][Pol][2]), receiver factors at factor_off ([n] float2, or
// none), weights at weight_off ([B][n] half2), effective weights written at
// weff_off ([2B][n] float2), eigenvalues at eval_off ([n]), K at count_idx.
struct SfEigItem {
  long long vis_off, factor_off, weight_off, weff_off, eval_off;
  long long u_off;  // eigenvectors-out form: float2 offset of this matrix's top-K vectors [K][n]
  int n, pol, count_idx, unit;
};

size_t sf_eig_topk_smem(int n, int B);
int sf_eig_topk_max_n();
size_t sf_eig_topk_items_smem(int n_max, int B);
int sf_eig_topk_max_b();
// The plan-layout matrices list[0 .. *list_count) (count read on the device, at most max_count).
cudaError_t sf_launch_eig_topk_list(const sf_plan *p, const int32_t *vis, const int32_t *list, const int32_t *list_count,
                                    int max_count, int k_rule, float delta, int shrink, float *evals, int32_t *counts,
                                    cudaStream_t stream);
cudaError_t sf_launch_eig_topk_vectors(const SfEigItem *items, int first, int count, int n_max, const int32_t *vis,
                                       const int32_t *fixed_counts, int k_rule, float delta, float *evals,
                                       int32_t *counts, float2 *u_out, float2 *scratch, int max_grid,
                                       uint32_t *status, cudaStream_t stream);
cudaError_t sf_launch_eig_topk_items(const SfEigItem *items, int first, int count, int n_max, int B,
                                     const int32_t *vis, const float2 *factors, const __half2 *weights,
                                     const int32_t *fixed_counts, int k_rule, float delta, int shrink, float *evals,
                                     int32_t *counts, float2 *weff, uint32_t *status, cudaStream_t stream);
int sf_eig_topk_supported(const sf_plan *p);
// One CTA per (channel, pol) covariance (sf_eig_small.cu): the adaptive
// path for R <= 128 and B <= 16 (four warps up to 64 receivers, sixteen up to 128).  With list != NULL only the
// matrices list[0 .. *list_count) (count read on the device, at most 2C).
int sf_eig_small_supported(const sf_plan *p);
// The batched form's matrices items[first .. first + count) of at most n_max receivers.
int sf_eig_small_items_supported(int n_max, int B);
cudaError_t sf_launch_eig_small_items(const SfEigItem *items, int first, int count, int n_max, int B,
                                      const int32_t *vis, const float2 *factors, const __half2 *weights,
                                      const int32_t *fixed_counts, int k_rule, float delta, int shrink,
                                      float *evals, int32_t *counts, float2 *weff, uint32_t *status, int num_sms,
                                      cudaStream_t stream);
cudaError_t sf_launch_eig_small(const sf_plan *p, const int32_t *vis, int k_rule, float delta, int shrink,
                                float *evals, int32_t *counts, const int32_t *list, const int32_t *list_count,
                                cudaStream_t stream);
cudaError_t sf_launch_eig_topk(const sf_plan *p, const int32_t *vis, int k_rule, float delta, int shrink,
                               float *evals, int32_t *counts, cudaStream_t stream);

cudaError_t sf_launch_weights_plain(const sf_plan *p, cudaStream_t stream);
cudaError_t sf_launch_beam(const sf_plan *p, const int8_t *samples, const int16_t *scales,
                           const int32_t *offsets, int n_slots, __half2 *beams,
                           cudaStream_t stream);
cudaError_t sf_launch_vis_accumulate(const sf_plan *p, const int32_t *vis, int64_t *accum,
                                     cudaStream_t stream);
cudaError_t sf_launch_vis_to_float(const sf_plan *p, const int64_t *accum, float *out,
                                   cudaStream_t stream);

// Steering-weight synthesis (sf_steering.cu).
cudaError_t sf_launch_steering(const sf_plan *p, const double *d_dircos, const double *d_enu,
                               const int32_t *d_connected, const float2 *d_cal, double base_hz, double bw_hz,
                               int min_ch, cudaStream_t stream);

// Beam spectra (sf_spectra.cu).
int sf_beam_spectra_supported(int T);
int sf_packet_spectra_supported(int Tp);
cudaError_t sf_fill_spectra_twiddles(float2 *d_tw, int T);
int sf_packet_spectra_tc_supported(const sf_plan *p);
size_t sf_packet_dft_bytes();
cudaError_t sf_fill_packet_dft(uint8_t *d_img);
cudaError_t sf_launch_beam_spectra(const sf_plan *p, const __half2 *beams, int n_beams_out,
                                   int downsample, float *out, cudaStream_t stream);
cudaError_t sf_launch_packet_spectra(const sf_plan *p, const __half2 *beams, int n_beams_out,
                                     int trim, float *out, cudaStream_t stream);
